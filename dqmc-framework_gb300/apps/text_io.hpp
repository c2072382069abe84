// text_io.hpp — the reference's text output, written natively.
//
// DqmcIO's formats (include/dqmc_io.h:101-629): the terminal parameter block,
// ending info and scalar summary, the observable files as means and errors or raw
// bins, the k stars, the imaginary-time grid and the bosonic fields; the lattice
// tables they need (k stars, high-symmetry points and lines of the square and
// cubic lattices, src/lattice/square.cpp:42-145, src/lattice/cubic.cpp:47-183);
// and Observable::analyse (include/measure/observable.h:169-211).  The Python
// module dqmc_gb300.io writes the same bytes.
#pragma once
#include <cmath>
#include <cstdio>
#include <map>
#include <sstream>
#include <string>
#include <utility>
#include <vector>

#include "toml_config.hpp"

namespace dqmc_app {

inline std::string fmt(const char* f, double v) {
  char b[64];
  std::snprintf(b, sizeof b, f, v);
  return b;
}
inline std::string fmti(long long v) {
  char b[32];
  std::snprintf(b, sizeof b, "%20lld", v);
  return b;
}
inline std::string f10(double v) { return fmt("%20.10f", v); }

// ---- lattice tables ---------------------------------------------------------
inline std::vector<std::vector<double>> kstars(int L, int dim) {
  std::vector<std::vector<double>> out;
  const auto m = [L](int i) { return (double)i / L * 2 * M_PI - M_PI; };
  const int lo = (L + 1) / 2;  // ceil(L / 2)
  if (dim == 2) {
    for (int i = lo; i <= L; ++i)
      for (int j = lo; j <= i; ++j) out.push_back({m(i), m(j)});
  } else {  // kz outermost: the tetrahedron (0,0,0), (pi,0,0), (pi,pi,0), (pi,pi,pi)
    for (int k = lo; k <= L; ++k)
      for (int i = k; i <= L; ++i)
        for (int j = k; j <= i; ++j) out.push_back({m(i), m(j), m(k)});
  }
  return out;
}

inline std::map<std::string, int> symmetry_points(int L, int dim) {
  const int h = L / 2;
  const int m_point = (h + 1) * (h + 2) / 2 - 1;  // the last k star of the kz = 0 plane
  std::map<std::string, int> p = {{"GammaPoint", 0}, {"XPoint", m_point - h}, {"MPoint", m_point}};
  if (dim == 3) p["RPoint"] = (int)kstars(L, 3).size() - 1;
  return p;
}

inline int momentum_index(int L, const std::string& name, int dim) {
  const auto p = symmetry_points(L, dim);
  auto it = p.find(name);
  if (it == p.end())
    throw ConfigError("undefined momentum '" + name + "' for " + (dim == 2 ? "2d square" : "3d cubic") + " lattice");
  return it->second;
}

inline std::vector<int> momentum_list(int L, const std::string& name, int dim) {
  const int nk = (int)kstars(L, dim).size(), h = L / 2;
  const auto p = symmetry_points(L, dim);
  const int xp = p.at("XPoint"), mp = p.at("MPoint");
  std::vector<int> v;
  if (name == "KstarsAll") {
    for (int i = 0; i < nk; ++i) v.push_back(i);
  } else if (name == "DeltaLine") {
    for (int i = 0; i <= h; ++i) v.push_back(i * (i + 1) / 2);
  } else if (name == "ZLine") {
    for (int i = 0; i <= h; ++i) v.push_back(xp + i);
  } else if (name == "SigmaLine") {
    for (int i = 0; i <= h; ++i) v.push_back(i * (i + 3) / 2);
  } else if (dim == 2 && name == "Gamma2X2M2GammaLoop") {
    for (int i = 0; i < h; ++i) v.push_back(i * (i + 1) / 2);
    for (int i = 0; i < h; ++i) v.push_back(xp + i);
    for (int i = h; i > 0; --i) v.push_back(i * (i + 3) / 2);
  } else if (dim == 3 && (name == "LambdaLine" || name == "SLine" || name == "TLine")) {
    int cur = name == "LambdaLine" ? 0 : name == "SLine" ? xp : mp;
    v.push_back(cur);
    for (int i = 1; i <= h; ++i) {  // each step skips one kz plane of the tetrahedron
      if (name == "LambdaLine") cur += (h + 2 - i) * (h + 3 - i) / 2;
      else if (name == "SLine") cur += (h + 1 - i) * (h + 2 - i) / 2 + 1;
      else cur += (h + 1 - i) * (h + 2 - i) / 2;
      v.push_back(cur);
    }
  } else if (p.count(name)) {
    v.push_back(p.at(name));
  } else {
    throw ConfigError("undefined momentum list '" + name + "'");
  }
  return v;
}

// ---- files --------------------------------------------------------------------
inline std::string format_kstars(int L, int dim) {
  const auto ks = kstars(L, dim);
  std::string s = fmti((long long)ks.size()) + "\n";
  for (size_t i = 0; i < ks.size(); ++i) {
    s += fmti((long long)i);
    for (double c : ks[i]) s += f10(c);
    s += "\n";
  }
  return s;
}

inline std::string format_tgrids(double beta, int lt) {
  const double dt = beta / lt;
  std::string s = fmti(lt) + fmt("%20.5f", beta) + fmt("%20.5f", dt) + "\n";
  for (int t = 0; t < lt; ++t) s += fmti(t) + f10(t * dt) + "\n";
  return s;
}

// DqmcIO::output_bosonic_fields: "Lt N" then "t i s" lines, fields[t * N + i] = +-1
inline std::string format_fields(const std::vector<signed char>& f, int lt, int n) {
  std::string s = fmti(lt) + fmti(n) + "\n";
  for (int t = 0; t < lt; ++t)
    for (int i = 0; i < n; ++i) s += fmti(t) + fmti(i) + fmt("%20.1f", (double)f[(size_t)t * n + i]) + "\n";
  return s;
}

// DqmcIO::read_bosonic_fields_from_file: returns [Lt * N] of +-1; the sizes must match
inline std::vector<signed char> parse_fields(const std::string& text, int lt, int n) {
  std::istringstream in(text);
  int flt = 0, fn = 0;
  if (!(in >> flt >> fn)) throw ConfigError("fields file: missing 'Lt N' header");
  if (flt != lt || fn != n) throw ConfigError("fields file size does not match the configuration");
  std::vector<signed char> f((size_t)lt * n, 1);
  long long t, i;
  double v;
  while (in >> t >> i >> v) {
    if (t < 0 || t >= lt || i < 0 || i >= n) throw ConfigError("fields file: site outside Lt x N");
    f[(size_t)t * n + i] = v > 0 ? 1 : -1;
  }
  return f;
}

inline std::string format_scalar(double mean, double err) {
  return f10(mean) + f10(err) + f10(mean != 0 ? err / mean : INFINITY) + "\n";
}
inline std::string format_vector(const std::vector<double>& mean, const std::vector<double>& err) {
  std::string s = fmti((long long)mean.size()) + "\n";
  for (size_t i = 0; i < mean.size(); ++i)
    s += fmti((long long)i) + f10(mean[i]) + f10(err[i]) + f10(mean[i] != 0 ? err[i] / mean[i] : INFINITY) + "\n";
  return s;
}
// rows x cols, row-major
inline std::string format_matrix(const std::vector<double>& mean, const std::vector<double>& err, int rows, int cols) {
  std::string s = fmti(rows) + fmti(cols) + "\n";
  for (int r = 0; r < rows; ++r)
    for (int c = 0; c < cols; ++c) {
      const double m = mean[(size_t)r * cols + c], e = err[(size_t)r * cols + c];
      s += fmti(r) + fmti(c) + f10(m) + f10(e) + f10(m != 0 ? e / m : INFINITY) + "\n";
    }
  return s;
}
inline std::string format_bins_scalar(const std::vector<double>& bins) {
  std::string s = fmti((long long)bins.size()) + "\n";
  for (size_t b = 0; b < bins.size(); ++b) s += fmti((long long)b) + f10(bins[b]) + "\n";
  return s;
}
// bins[b][i]
inline std::string format_bins_vector(const std::vector<std::vector<double>>& bins) {
  std::string s = fmti((long long)bins.size()) + fmti((long long)bins[0].size()) + "\n";
  for (size_t b = 0; b < bins.size(); ++b)
    for (size_t i = 0; i < bins[b].size(); ++i) s += fmti((long long)b) + fmti((long long)i) + f10(bins[b][i]) + "\n";
  return s;
}
// bins[b][r * cols + c]
inline std::string format_bins_matrix(const std::vector<std::vector<double>>& bins, int rows, int cols) {
  std::string s = fmti((long long)bins.size()) + fmti(rows) + fmti(cols) + "\n";
  for (size_t b = 0; b < bins.size(); ++b)
    for (int r = 0; r < rows; ++r)
      for (int c = 0; c < cols; ++c)
        s += fmti((long long)b) + fmti(r) + fmti(c) + f10(bins[b][(size_t)r * cols + c]) + "\n";
  return s;
}

// Observable::analyse: mean over bins and sqrt(<x^2> - <x>^2) / sqrt(nbins - 1), elementwise
inline void analyse(const std::vector<std::vector<double>>& bins, std::vector<double>& mean, std::vector<double>& err) {
  const size_t n = bins.size(), m = n ? bins[0].size() : 0;
  mean.assign(m, 0.0);
  err.assign(m, 0.0);
  for (size_t k = 0; k < m; ++k) {
    double s = 0, s2 = 0;
    for (auto& b : bins) {
      s += b[k];
      s2 += b[k] * b[k];
    }
    mean[k] = s / n;
    err[k] = n > 1 ? std::sqrt(std::fmax(s2 / n - mean[k] * mean[k], 0.0)) / std::sqrt((double)n - 1) : 0.0;
  }
}

// ---- terminal -----------------------------------------------------------------
inline std::string summary_line(const std::string& description, double mean, double err) {
  char b[160];
  std::snprintf(b, sizeof b, "%30s%7s%20.12f  pm  %.12f\n", description.c_str(), "->", mean, err);
  return b;
}

// observable_handler.cpp:140-277 descriptions, in dqmc_main's print order (src/dqmc_main.cpp:213-266)
inline const std::vector<std::pair<std::string, std::string>>& summary_order() {
  static const std::vector<std::pair<std::string, std::string>> v = {
      {"filling_number", "Filling number"},
      {"double_occupancy", "Double occupation"},
      {"kinetic_energy", "Kinetic energy"},
      {"local_spin_corr", "Local spin correlation"},
      {"momentum_distribution", "Momentum distribution"},
      {"spin_density_structure_factor", "SDW order parameter"},
      {"charge_density_structure_factor", "CDW order parameter"},
      {"s_wave_pairing_corr", "S-wave pairing correlation"},
      {"superfluid_stiffness", "Superfluid stiffness"}};
  return v;
}

inline std::string format_summary(const std::map<std::string, std::pair<double, double>>& r) {
  std::string s;
  if (r.count("equaltime_sign")) s += summary_line("Averaged sign (equal-time)", r.at("equaltime_sign").first,
                                                   r.at("equaltime_sign").second);
  if (r.count("dynamic_sign")) s += summary_line("Averaged sign (dynamical)", r.at("dynamic_sign").first,
                                                 r.at("dynamic_sign").second);
  s += "\n";
  for (auto& [name, desc] : summary_order())
    if (r.count(name)) s += summary_line(desc, r.at(name).first, r.at(name).second);
  return s;
}

inline std::string param(const std::string& name, const std::string& value) {
  char b[160];
  std::snprintf(b, sizeof b, "%30s%7s%24s\n", name.c_str(), "->", value.c_str());
  return b;
}

// DqmcIO::output_init_info (include/dqmc_io.h:101-236); chains = the reference's MPI ranks
inline std::string format_init_info(const RunConfig& c, int chains) {
  const auto f3 = [](double v) { return fmt("%.3f", v); };
  const auto tf = [](bool b) { return std::string(b ? "True" : "False"); };
  std::string s = std::string("   Model: ") + (c.model == "AttractiveHubbard" ? "Attractive Hubbard" : "Repulsive Hubbard") +
                  "\n" + param("Hopping constant 't'", f3(c.hopping_t)) +
                  param("Onsite interaction 'U'", f3(c.onsite_u)) +
                  param("Checimcal potential 'mu'", f3(c.chemical_potential)) + "\n";  // the reference's spelling
  const int L = c.L(), dim = c.dim();
  const auto ks = kstars(L, dim);
  const auto& k = ks[c.momentum.empty() ? ks.size() - 1 : (size_t)momentum_index(L, c.momentum, dim)];
  char mom[96];
  if (dim == 2) {
    std::snprintf(mom, sizeof mom, "(%.2f, %.2f) pi", k[0] / M_PI, k[1] / M_PI);
    s += "   Lattice: Square lattice\n" + param("Size of cell", std::to_string(L) + " * " + std::to_string(L));
  } else {
    std::snprintf(mom, sizeof mom, "(%.2f, %.2f, %.2f) pi", k[0] / M_PI, k[1] / M_PI, k[2] / M_PI);
    s += "   Lattice: Cubic lattice\n" +
         param("Size of cell", std::to_string(L) + " * " + std::to_string(L) + " * " + std::to_string(L));
  }
  s += param("Momentum point", mom) + param("Checkerboard breakups", tf(c.checkerboard)) + "\n";
  s += "   MonteCarlo Params:\n" + param("Inverse temperature", f3(c.beta)) +
       param("Imaginary-time length", std::to_string(c.time_size)) +
       param("Imaginary-time interval", f3(c.beta / c.time_size)) +
       param("Stabilization pace", std::to_string(c.stabilization_pace)) + "\n";
  s += "   Measuring Params:\n" + param("Warm up", tf(c.sweeps_warmup != 0)) +
       param("Equal-time measure", tf(c.equaltime())) + param("Dynamical measure", tf(c.dynamic())) + "\n";
  const int per_chain = (c.bin_num + chains - 1) / chains;
  s += param("Sweeps for warmup", std::to_string(c.sweeps_warmup)) +
       param("Number of bins", std::to_string(per_chain * chains)) + param("Sweeps per bin", std::to_string(c.bin_size)) +
       param("Sweeps between bins", std::to_string(c.sweeps_between_bins)) + "\n";
  return s;
}

// DqmcIO::output_ending_info (include/dqmc_io.h:240-265)
inline std::string format_ending_info(double seconds, double wrap_error) {
  const long long ms = (long long)(seconds * 1000);  // Dqmc::timer() counts milliseconds
  const long long day = ms / 86400000;
  const long long hour = (long long)((ms / 1000.0 - day * 86400) / 3600);
  const long long minute = (long long)((ms / 1000.0 - day * 86400 - hour * 3600) / 60);
  const double sec = ms / 1000.0 - 86400.0 * day - 3600.0 * hour - 60.0 * minute;
  char t[96];
  if (day) std::snprintf(t, sizeof t, "%lld d %lld h %lld m %.2f s", day, hour, minute, sec);
  else if (hour) std::snprintf(t, sizeof t, "%lld h %lld m %.2f s", hour, minute, sec);
  else if (minute) std::snprintf(t, sizeof t, "%lld m %.2f s", minute, sec);
  else std::snprintf(t, sizeof t, "%.2f s", sec);
  char w[64];
  std::snprintf(w, sizeof w, "%.5e", wrap_error);
  return std::string("\n>> The simulation finished in ") + t + ".\n\n>> Maximum of the wrapping error: " + w + "\n\n";
}

}  // namespace dqmc_app
