// dqmc_run — command-line driver of the GB300 sweep library, written against the
// reference-style C++ interface (include/dqmc_gb300.hpp).  It plays the role of the
// reference's src/dqmc_main.cpp for the hot path: set up model, lattice and
// walkers, thermalize, measure in bins, analyse, print mean +/- error per
// observable, one JSON object per line.
//
// usage: dqmc_run key=value ...   keys: model (repulsive|attractive), lattice (square|cubic),
//        L, t, U, mu, beta, Lt, pace, checkerboard (0|1), walkers, seed, warmup, bins, binsize,
//        between, fields (path of a "t i s" text file, reference fields.out format)
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/dqmc_gb300.hpp"

int main(int argc, char** argv) {
  std::map<std::string, std::string> kv = {
      {"model", "repulsive"}, {"lattice", "square"}, {"L", "4"}, {"t", "1"}, {"U", "4"}, {"mu", "0"}, {"beta", "4"}, {"Lt", "80"},
      {"pace", "10"}, {"checkerboard", "0"}, {"walkers", "1"}, {"seed", "12345"}, {"warmup", "100"},
      {"bins", "10"}, {"binsize", "20"}, {"between", "0"}, {"fields", ""}, {"rng", "minstd"}};
  for (int i = 1; i < argc; ++i) {
    std::string a = argv[i];
    const auto eq = a.find('=');
    if (eq == std::string::npos || !kv.count(a.substr(0, eq))) {
      std::fprintf(stderr, "unknown argument '%s'\n", argv[i]);
      return 2;
    }
    kv[a.substr(0, eq)] = a.substr(eq + 1);
  }
  try {
    using namespace dqmc_gb300;
    Model model = (kv["model"] == "attractive") ? (Model)AttractiveHubbard() : (Model)RepulsiveHubbard();
    model.set_model_params(std::stod(kv["t"]), std::fabs(std::stod(kv["U"])), std::stod(kv["mu"]));
    if (std::stoi(kv["checkerboard"])) model.link_checkerboard(); else model.link();
    const int L = std::stoi(kv["L"]);
    if (kv["lattice"] != "square" && kv["lattice"] != "cubic")
      throw Error(DQMC_ERR_ARG, "lattice must be square or cubic");
    Square square;
    Cubic cubic;
    if (kv["lattice"] == "cubic") cubic.set_lattice_params({L, L, L}); else square.set_lattice_params({L, L});
    const LatticeBase& lattice = (kv["lattice"] == "cubic") ? (const LatticeBase&)cubic : (const LatticeBase&)square;
    DqmcWalker walker;
    walker.set_physical_params(std::stod(kv["beta"]), std::stoi(kv["Lt"]));
    walker.set_stabilization_pace(std::stoi(kv["pace"]));
    const int nw = std::stoi(kv["walkers"]);
    std::vector<uint64_t> seeds(nw);
    for (int w = 0; w < nw; ++w) seeds[w] = std::stoull(kv["seed"]) + w;  // time + rank in the reference
    walker.initial(lattice, model, seeds, kv["rng"] == "philox" ? DQMC_RNG_PHILOX : DQMC_RNG_MINSTD);
    if (kv["fields"].empty()) {
      walker.set_bosonic_fields_to_random();
    } else {  // DqmcIO::read_bosonic_fields_from_file format: "Lt N" then "t i s" lines
      std::ifstream in(kv["fields"]);
      int lt = 0, n = 0;
      in >> lt >> n;
      if (!in || lt != walker.TimeSize() || n != lattice.SpaceSize()) throw Error(DQMC_ERR_ARG, "fields file size mismatch");
      std::vector<int8_t> f((size_t)lt * n, 1);
      int t, i;
      double s;
      while (in >> t >> i >> s) {
        if (t < 0 || t >= lt || i < 0 || i >= n) throw Error(DQMC_ERR_ARG, "fields file: site outside Lt x N");
        f[(size_t)t * n + i] = s > 0 ? 1 : -1;
      }
      for (int w = 0; w < nw; ++w) walker.set_bosonic_fields(w, f);
    }
    walker.initial_greens_functions();
    MeasureHandler meas;
    meas.set_measure_params(std::stoi(kv["warmup"]), std::stoi(kv["bins"]), std::stoi(kv["binsize"]),
                            std::stoi(kv["between"]));
    Dqmc::thermalize(walker, meas);
    Dqmc::measure(walker, meas);
    Dqmc::analyse(meas);
    static const char* names[DQMC_NUM_OBS] = {"filling_number", "double_occupancy", "kinetic_energy",
                                              "momentum_distribution", "local_spin_corr",
                                              "spin_density_structure_factor", "charge_density_structure_factor",
                                              "s_wave_pairing_corr", "equaltime_sign"};
    double wrap = 0;
    for (int w = 0; w < nw; ++w) wrap = std::fmax(wrap, walker.WrapError(w));
    std::printf("{\"bins\": %zu, \"max_wrap_error\": %.6e", meas.bins.size(), wrap);
    for (int k = 0; k < DQMC_NUM_OBS; ++k) std::printf(", \"%s\": [%.12f, %.12f]", names[k], meas.mean[k], meas.error[k]);
    std::printf("}\n");
  } catch (const dqmc_gb300::Error& e) {
    std::fprintf(stderr, "dqmc_run: status %d: %s\n", e.status, e.what());
    return 1;
  }
  return 0;
}
