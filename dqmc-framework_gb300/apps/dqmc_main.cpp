// dqmc_main — the reference's main program (src/dqmc_main.cpp) on the GB300 sweep.
//
// usage: dqmc_main [-c CONFIG] [-o OUTPUT] [-f FIELDS] [--walkers W] [--seed S]
//                  [--precision fp64|mixed] [--rng minstd|philox] [--dry-run]
//
// The options -c/--config, -o/--output and -f/--fields and their defaults are
// dqmc_main's (src/dqmc_main.cpp:53-62), so the reference's run scripts need only
// the executable swapped.  The TOML configuration is read by the reference's rules
// (toml_config.hpp).  W independent walkers (Markov chains) on one GPU stand in for
// W MPI ranks: warm-up of sweeps_warmup / 2 forth-and-back pairs, then
// ceil(bin_num / W) bins per walker (Dqmc::thermalize / measure / sweep_forth_and_back,
// src/dqmc.cpp:48-151; with dynamic observables the forward half-sweep is
// sweep_for_dynamic_greens and the equal-time measurement is taken on the backward
// one), the bins of all walkers pooled and analysed as Observable::analyse.  Output as
// dqmc_main writes it: the terminal log (start-up lines, parameter block, wall time and
// maximum wrap error, scalar results) and kstars.out, tgrids.out, swave(.bins).out,
// dos(.bins).out, greens(.bins).out, dss(.bins).out, and the final fields of walker 0
// written back over the --fields file when one was given, else to fields.out.
// --dry-run does all of it that needs no device: the configuration, the parameter
// block, kstars.out, tgrids.out and the fields file read and written back.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/dqmc_gb300.hpp"
#include "text_io.hpp"
#include "toml_config.hpp"

namespace {

struct Args {
  std::string config = "../example/config.toml", output = "../example", fields;
  int walkers = 1;
  unsigned long long seed = 12345;
  std::string precision = "fp64", rng = "minstd";
  bool dry_run = false;
};

bool parse_args(int argc, char** argv, Args& a) {
  for (int i = 1; i < argc; ++i) {
    std::string k = argv[i], v;
    const auto eq = k.find('=');
    if (k.rfind("--", 0) == 0 && eq != std::string::npos) {
      v = k.substr(eq + 1);
      k = k.substr(0, eq);
    }
    const bool flag = (k == "--dry-run" || k == "-h" || k == "--help");
    if (!flag && v.empty()) {
      if (i + 1 >= argc) return false;
      v = argv[++i];
    }
    if (k == "-h" || k == "--help") return false;
    if (k == "--dry-run") a.dry_run = true;
    else if (k == "-c" || k == "--config") a.config = v;
    else if (k == "-o" || k == "--output") a.output = v;
    else if (k == "-f" || k == "--fields") a.fields = v;
    else if (k == "--walkers") a.walkers = std::stoi(v);
    else if (k == "--seed") a.seed = std::stoull(v);
    else if (k == "--precision" && (v == "fp64" || v == "mixed")) a.precision = v;
    else if (k == "--rng" && (v == "minstd" || v == "philox")) a.rng = v;
    else return false;
  }
  return a.walkers >= 1;
}

std::string read_file(const std::string& path) {
  std::ifstream in(path);
  if (!in) throw dqmc_app::ConfigError("cannot read '" + path + "'");
  std::stringstream ss;
  ss << in.rdbuf();
  return ss.str();
}

void write_file(const std::string& path, const std::string& text) {
  std::ofstream out(path, std::ios::trunc);
  out << text;
  if (!out) throw dqmc_app::ConfigError("cannot write '" + path + "'");
}

std::string now_string() {  // boost::posix_time::to_simple_string layout, e.g. 2022-Sep-06 22:42:10
  const std::time_t t = std::time(nullptr);
  char b[64];
  std::strftime(b, sizeof b, "%Y-%b-%d %H:%M:%S", std::localtime(&t));
  return b;
}

// per-walker bins of one run: equal-time [bin][9]; dynamic G(k,tau) [bin][k * ntau + tau],
// D(tau), chi(tau) [bin][tau], the stiffness and the dynamic sign [bin]
struct Bins {
  std::vector<std::vector<double>> eq, greens, dos, dss;
  std::vector<double> rho, sign;
};

}  // namespace

int main(int argc, char** argv) {
  using namespace dqmc_app;
  Args a;
  if (!parse_args(argc, argv, a)) {
    std::fprintf(stderr,
                 "main(): undefined options got from command line.\n"
                 "usage: dqmc_main [-c CONFIG] [-o OUTPUT] [-f FIELDS] [--walkers W] [--seed S]\n"
                 "                 [--precision fp64|mixed] [--rng minstd|philox] [--dry-run]\n");
    return 1;
  }
  const auto t_start = std::chrono::steady_clock::now();
  try {
    const RunConfig cfg = parse_config(read_file(a.config));
    const int L = cfg.L(), dim = cfg.dim(), lt = cfg.time_size;
    const int N = dim == 2 ? L * L : L * L * L;
    const int kidx = cfg.momentum.empty() ? -1 : momentum_index(L, cfg.momentum, dim);
    const auto klist = momentum_list(L, cfg.momentum_list.empty() ? "KstarsAll" : cfg.momentum_list, dim);
    std::filesystem::create_directories(a.output);
    std::vector<signed char> fields;
    if (!a.fields.empty()) fields = parse_fields(read_file(a.fields), lt, N);

    std::printf(">> Current time: %s\n\n", now_string().c_str());
    std::printf(">> Distribute tasks to %d walkers on one GPU.\n\n", a.walkers);
    std::printf(">> Configurations of the bosonic fields %s\n\n",
                a.fields.empty() ? "set to random." : "read from the input config file.");
    std::printf(">> Initialization finished. \n\n>> The simulation is going to get started with parameters shown below :\n\n");
    std::printf("%s", format_init_info(cfg, a.walkers).c_str());
    std::fflush(stdout);
    write_file(a.output + "/kstars.out", format_kstars(L, dim));
    write_file(a.output + "/tgrids.out", format_tgrids(cfg.beta, lt));
    if (a.dry_run) {
      if (!a.fields.empty()) write_file(a.fields, format_fields(fields, lt, N));
      std::fprintf(stderr, "dqmc_main: dry run, no device work\n");
      return 0;
    }

    using namespace dqmc_gb300;
    Model model = cfg.model == "AttractiveHubbard" ? (Model)AttractiveHubbard() : (Model)RepulsiveHubbard();
    model.set_model_params(cfg.hopping_t, cfg.onsite_u, cfg.chemical_potential);
    if (cfg.checkerboard) model.link_checkerboard(); else model.link();
    Square square;
    Cubic cubic;
    if (dim == 2) square.set_lattice_params({L, L}); else cubic.set_lattice_params({L, L, L});
    LatticeBase& lattice = dim == 2 ? (LatticeBase&)square : (LatticeBase&)cubic;
    lattice.momentum_index = kidx;
    DqmcWalker walker;
    walker.set_physical_params(cfg.beta, lt);
    walker.set_stabilization_pace(cfg.stabilization_pace);
    std::vector<uint64_t> seeds(a.walkers);
    for (int w = 0; w < a.walkers; ++w) seeds[w] = a.seed + w;
    const bool eqt = cfg.equaltime(), dyn = cfg.dynamic();
    walker.initial(lattice, model, seeds, a.rng == "philox" ? DQMC_RNG_PHILOX : DQMC_RNG_MINSTD,
                   a.precision == "mixed" ? DQMC_MIXED : DQMC_FP64, dyn);
    if (fields.empty()) {
      walker.set_bosonic_fields_to_random();
    } else {
      const std::vector<int8_t> f(fields.begin(), fields.end());
      for (int w = 0; w < a.walkers; ++w) walker.set_bosonic_fields(w, f);
    }
    walker.initial_greens_functions();
    for (int s = 1; s <= cfg.sweeps_warmup / 2; ++s) {  // Dqmc::thermalize
      walker.sweep_from_0_to_beta(false);
      walker.sweep_from_beta_to_0(false);
    }
    const int nw = a.walkers;
    int nbins = (eqt || dyn) ? (cfg.bin_num + nw - 1) / nw : 0;
    std::vector<Bins> per(nw);
    std::vector<int> taus(lt);
    for (int t = 0; t < lt; ++t) taus[t] = t;
    const auto ks = kstars(L, dim);
    // Fourier factors of the measured momenta, ff[q][r] = cos(-r.k) (square.cpp:148-161, cubic.cpp:186-200)
    std::vector<std::vector<double>> ff(klist.size(), std::vector<double>(N));
    for (size_t q = 0; q < klist.size(); ++q)
      for (int r = 0; r < N; ++r) {
        double rk = (r % L) * ks[klist[q]][0] + ((r / L) % L) * ks[klist[q]][1];
        if (dim == 3) rk += (r / (L * L)) * ks[klist[q]][2];
        ff[q][r] = std::cos(-rk);
      }
    if (eqt && !dyn) {  // equal-time only: bins normalised on the device, one copy out
      const auto out = walker.MeasureBins(nbins, std::max(cfg.bin_size, 2), cfg.sweeps_between_bins);
      for (int w = 0; w < nw; ++w)
        for (int b = 0; b < nbins; ++b)
          per[w].eq.emplace_back(out.begin() + ((size_t)w * nbins + b) * DQMC_NUM_OBS,
                                 out.begin() + ((size_t)w * nbins + b + 1) * DQMC_NUM_OBS);
      nbins = 0;
    }
    std::vector<double> sums((size_t)nw * DQMC_NUM_OBS);
    std::vector<int64_t> counts((size_t)nw * DQMC_NUM_OBS);
    for (int bin = 0; bin < nbins; ++bin) {
      check(dqmc_clear_observables(walker.handle()));
      if (dyn) check(dqmc_clear_dynamic(walker.handle()));
      std::vector<double> sgn(nw, 0.0);
      for (int s = 1; s <= cfg.bin_size / 2; ++s) {  // Dqmc::sweep_forth_and_back
        if (dyn) {
          walker.sweep_for_dynamic_greens(taus);
          for (int w = 0; w < nw; ++w) sgn[w] += walker.ConfigSign(w);
        } else {
          walker.sweep_from_0_to_beta(eqt);
        }
        walker.sweep_from_beta_to_0(eqt);
      }
      if (eqt) {  // MeasureHandler::normalize_stats
        check(dqmc_get_observables_all(walker.handle(), sums.data(), counts.data()));
        for (int w = 0; w < nw; ++w) {
          const double* sw = &sums[(size_t)w * DQMC_NUM_OBS];
          const int64_t* cw = &counts[(size_t)w * DQMC_NUM_OBS];
          const double sign = sw[DQMC_OBS_SIGN] / (double)cw[DQMC_OBS_SIGN];
          std::vector<double> b(DQMC_NUM_OBS);
          for (int k = 0; k < DQMC_OBS_SIGN; ++k) b[k] = sw[k] / ((double)cw[k] * sign);
          b[DQMC_OBS_SIGN] = std::fabs(sign);
          per[w].eq.push_back(b);
        }
      }
      if (dyn) {
        for (int w = 0; w < nw; ++w) {
          std::vector<int64_t> cnt;
          walker.DynamicGreens(w, &cnt);
          const auto S = walker.DynamicGreensR(w);  // [tau][r]
          const auto o = walker.DynamicObs(w);
          const double ms = sgn[w] / std::max<int64_t>(cnt[0], 1);  // the dynamic sign
          std::vector<double> g(klist.size() * lt), d(lt), c(lt);
          for (size_t q = 0; q < klist.size(); ++q)
            for (int t = 0; t < lt; ++t) {  // G(k, tau) = sum_r FourierFactor(r, k) S(r, tau)
              double acc = 0;
              for (int r = 0; r < N; ++r) acc += ff[q][r] * S[(size_t)t * N + r];
              g[q * lt + t] = acc / (cnt[t] * ms);
            }
          double rho = 0;
          for (int t = 0; t < lt; ++t) {
            d[t] = o.density_of_states[t] / (cnt[t] * ms);
            c[t] = o.spin_susceptibility[t] / (cnt[t] * ms);
            rho += o.stiffness_terms[t];
          }
          per[w].greens.push_back(g);
          per[w].dos.push_back(d);
          per[w].dss.push_back(c);
          per[w].rho.push_back(rho / (cnt[0] * ms));
          per[w].sign.push_back(std::fabs(ms));
        }
      }
      for (int s = 0; s < cfg.sweeps_between_bins / 2; ++s) {
        walker.sweep_from_0_to_beta(false);
        walker.sweep_from_beta_to_0(false);
      }
    }
    // pool the walkers' bins in walker order (the reference's MPI gather)
    Bins pool;
    double wrap = 0;
    for (int w = 0; w < nw; ++w) {
      auto app = [](auto& to, const auto& from) { to.insert(to.end(), from.begin(), from.end()); };
      app(pool.eq, per[w].eq);
      app(pool.greens, per[w].greens);
      app(pool.dos, per[w].dos);
      app(pool.dss, per[w].dss);
      app(pool.rho, per[w].rho);
      app(pool.sign, per[w].sign);
      wrap = std::fmax(wrap, walker.WrapError(w));
    }
    std::vector<signed char> final_fields((size_t)lt * N);
    check(dqmc_get_fields(walker.handle(), 0, reinterpret_cast<int8_t*>(final_fields.data())));

    std::map<std::string, std::pair<double, double>> results;
    std::vector<double> mean, err;
    if (eqt) {
      analyse(pool.eq, mean, err);
      static const char* names[DQMC_NUM_OBS] = {"filling_number", "double_occupancy", "kinetic_energy",
                                                "momentum_distribution", "local_spin_corr",
                                                "spin_density_structure_factor", "charge_density_structure_factor",
                                                "s_wave_pairing_corr", "equaltime_sign"};
      for (int k = 0; k < DQMC_NUM_OBS; ++k)
        if (k == DQMC_OBS_SIGN || cfg.has(names[k])) results[names[k]] = {mean[k], err[k]};
      if (cfg.has("s_wave_pairing_corr")) {
        const int k = 7;
        write_file(a.output + "/swave.out", format_scalar(mean[k], err[k]));
        std::vector<double> col;
        for (auto& b : pool.eq) col.push_back(b[k]);
        write_file(a.output + "/swave.bins.out", format_bins_scalar(col));
      }
    }
    if (dyn) {
      auto scalar = [&](const std::vector<double>& v) {
        std::vector<std::vector<double>> b;
        for (double x : v) b.push_back({x});
        analyse(b, mean, err);
        return std::make_pair(mean[0], err[0]);
      };
      results["dynamic_sign"] = scalar(pool.sign);
      if (cfg.has("density_of_states")) {
        analyse(pool.dos, mean, err);
        write_file(a.output + "/dos.out", format_vector(mean, err));
        write_file(a.output + "/dos.bins.out", format_bins_vector(pool.dos));
      }
      if (cfg.has("dynamic_spin_susceptibility")) {
        analyse(pool.dss, mean, err);
        write_file(a.output + "/dss.out", format_vector(mean, err));
        write_file(a.output + "/dss.bins.out", format_bins_vector(pool.dss));
      }
      if (cfg.has("greens_functions")) {
        analyse(pool.greens, mean, err);
        write_file(a.output + "/greens.out", format_matrix(mean, err, (int)klist.size(), lt));
        write_file(a.output + "/greens.bins.out", format_bins_matrix(pool.greens, (int)klist.size(), lt));
      }
      if (cfg.has("superfluid_stiffness")) results["superfluid_stiffness"] = scalar(pool.rho);
    }
    // dqmc_main writes the final fields back over the input fields file (src/dqmc_main.cpp:280-283)
    write_file(a.fields.empty() ? a.output + "/fields.out" : a.fields, format_fields(final_fields, lt, N));
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count();
    std::printf("%s%s", format_ending_info(secs, wrap).c_str(), format_summary(results).c_str());
  } catch (const ConfigError& e) {
    std::fprintf(stderr, "dqmc_main: %s\n", e.what());
    return 1;
  } catch (const dqmc_gb300::Error& e) {
    std::fprintf(stderr, "dqmc_main: status %d: %s\n", e.status, e.what());
    return 1;
  } catch (const std::exception& e) {
    std::fprintf(stderr, "dqmc_main: %s\n", e.what());
    return 1;
  }
  return 0;
}
