// dqmc_gb300.hpp — C++ host interface over the C-ABI (include/dqmc_gb300.h),
// mirroring the reference's operator interface (dqmc-framework):
//   Model::RepulsiveHubbard / AttractiveHubbard   include/model/*.h
//   Lattice::Square / Lattice::Cubic               include/lattice/square.h, cubic.h
//   QuantumMonteCarlo::DqmcWalker                  include/dqmc_walker.h:107-184
//   Measure::MeasureHandler                        include/measure/measure_handler.h
//   QuantumMonteCarlo::Dqmc::thermalize / measure / analyse   src/dqmc.cpp:48-158
// Method names and argument meaning follow the reference.  Differences: one
// object drives a whole batch of walkers (the reference's MPI ranks), and
// failures throw dqmc_gb300::Error instead of calling exit(1).
#pragma once

#include <algorithm>
#include <cmath>
#include <stdexcept>
#include <string>
#include <vector>

#include "dqmc_gb300.h"

namespace dqmc_gb300 {

struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

inline void check(int rc) {
  if (rc != DQMC_OK) throw Error(rc, dqmc_last_error());
}

// ---- Model (src/model/repulsive_hubbard.cpp:32-41) ----------------------------
struct Model {
  int type = DQMC_REPULSIVE_HUBBARD;
  double hopping_t = 1.0, onsite_u = 4.0, chemical_potential = 0.0;
  bool checkerboard = false;
  void set_model_params(double t, double u, double mu) {
    if (t < 0 || u < 0) throw Error(DQMC_ERR_ARG, "set_model_params: need t >= 0 and U >= 0");
    hopping_t = t;
    onsite_u = u;
    chemical_potential = mu;
  }
  void link() { checkerboard = false; }            // dense exp(-dtau K)  (model_base.cpp:38-45)
  void link_checkerboard() { checkerboard = true; } // link(CheckerBoardBase&) (model_base.cpp:48-55)
};
struct RepulsiveHubbard : Model { RepulsiveHubbard() { type = DQMC_REPULSIVE_HUBBARD; } };
struct AttractiveHubbard : Model { AttractiveHubbard() { type = DQMC_ATTRACTIVE_HUBBARD; } };

// ---- Lattice::Square (src/lattice/square.cpp:16-28), Lattice::Cubic (src/lattice/cubic.cpp:19-31)
struct LatticeBase {
  int type = DQMC_SQUARE;
  int side = 4;
  int momentum_index = -1;  // -1 = the last k star: MPoint (pi, pi) / RPoint (pi, pi, pi)
  int SpaceDim() const { return type == DQMC_CUBIC ? 3 : 2; }
  int SpaceSize() const { return type == DQMC_CUBIC ? side * side * side : side * side; }
};
struct Square : LatticeBase {
  void set_lattice_params(const std::vector<int>& side_length_vec) {
    if (side_length_vec.size() != 2 || side_length_vec[0] != side_length_vec[1] || side_length_vec[0] < 2)
      throw Error(DQMC_ERR_ARG, "Square: need two equal sides >= 2");
    side = side_length_vec[0];
  }
};
struct Cubic : LatticeBase {
  Cubic() { type = DQMC_CUBIC; }
  void set_lattice_params(const std::vector<int>& side_length_vec) {
    if (side_length_vec.size() != 3 || side_length_vec[0] != side_length_vec[1] ||
        side_length_vec[0] != side_length_vec[2] || side_length_vec[0] < 2)
      throw Error(DQMC_ERR_ARG, "Cubic: need three equal sides >= 2");
    side = side_length_vec[0];
  }
};

// ---- MeasureHandler (src/measure/measure_handler.cpp) ------------------------
struct MeasureHandler {
  int sweeps_warmup = 512, bin_num = 20, bin_size = 100, sweeps_between_bins = 20;
  bool equaltime = true;
  // bins[b][k]: normalised bin values (normalize_stats + write_stats_to_bins)
  std::vector<std::vector<double>> bins;
  std::vector<double> mean, error;
  void set_measure_params(int warmup, int nbin, int size, int between) {
    sweeps_warmup = warmup;
    bin_num = nbin;
    bin_size = size;
    sweeps_between_bins = between;
  }
  bool isWarmUp() const { return sweeps_warmup != 0; }
  bool isEqualTime() const { return equaltime; }
  int WarmUpSweeps() const { return sweeps_warmup; }
  int BinsNum() const { return bin_num; }
  int BinsSize() const { return bin_size; }
  int SweepsBetweenBins() const { return sweeps_between_bins; }
  // Observable::analyse (include/measure/observable.h:169-193) over all bins
  void analyse_stats() {
    const size_t nb = bins.size();
    mean.assign(DQMC_NUM_OBS, 0.0);
    error.assign(DQMC_NUM_OBS, 0.0);
    if (nb == 0) return;
    for (int k = 0; k < DQMC_NUM_OBS; ++k) {
      double s = 0, s2 = 0;
      for (auto& b : bins) { s += b[k]; s2 += b[k] * b[k]; }
      mean[k] = s / nb;
      error[k] = nb > 1 ? std::sqrt(std::fmax(s2 / nb - mean[k] * mean[k], 0.0)) / std::sqrt((double)nb - 1) : 0.0;
    }
  }
};

// ---- DqmcWalker: a batch of n walkers sharing model/lattice parameters --------
class DqmcWalker {
 public:
  DqmcWalker() = default;
  DqmcWalker(const DqmcWalker&) = delete;
  DqmcWalker& operator=(const DqmcWalker&) = delete;
  ~DqmcWalker() { if (b_) dqmc_batch_destroy(b_); }

  void set_physical_params(double beta, int time_size) {
    if (!(beta > 0) || time_size < 1) throw Error(DQMC_ERR_ARG, "set_physical_params: beta > 0, Lt >= 1");
    beta_ = beta;
    lt_ = time_size;
  }
  void set_stabilization_pace(int pace) {
    if (pace < 1) throw Error(DQMC_ERR_ARG, "set_stabilization_pace: pace >= 1");
    pace_ = pace;
  }
  // one walker per seed; rng = DQMC_RNG_MINSTD reproduces the reference stream; precision
  // DQMC_MIXED selects the tensor-core path; hbm puts every walker on the HBM path
  void initial(const LatticeBase& lat, const Model& model, const std::vector<uint64_t>& seeds,
               int rng = DQMC_RNG_MINSTD, int precision = DQMC_FP64, bool hbm = false) {
    std::vector<dqmc_walker_desc> d(seeds.size());
    for (size_t w = 0; w < seeds.size(); ++w) {
      d[w] = dqmc_walker_desc{model.type, lat.side, model.hopping_t, model.onsite_u, model.chemical_potential,
                              beta_, lt_, pace_, model.checkerboard ? 1 : 0, lat.momentum_index, seeds[w],
                              lat.type};
    }
    dqmc_batch_options o{rng, precision, 0, 1, hbm ? 1 : 0};
    if (b_) dqmc_batch_destroy(b_);
    b_ = nullptr;
    check(dqmc_batch_create(d.data(), (int)d.size(), &o, &b_));
    n_ = (int)d.size();
    N_ = lat.SpaceSize();
  }
  void set_bosonic_fields_to_random() { for (int w = 0; w < n_; ++w) check(dqmc_fields_random(b_, w)); }
  // fields of walker w, [Lt][N] of +1/-1: the library reads exactly Lt * N bytes
  void set_bosonic_fields(int w, const std::vector<int8_t>& f) {
    if (f.size() != (size_t)lt_ * N_) throw Error(DQMC_ERR_ARG, "set_bosonic_fields: expected Lt * N values");
    check(dqmc_set_fields(b_, w, f.data()));
  }
  void initial_greens_functions() { check(dqmc_init_greens(b_)); }  // stacks + G(0) + sign
  void sweep_from_0_to_beta(bool measure = false) { check(dqmc_sweep_0_to_beta(b_, measure)); }
  void sweep_from_beta_to_0(bool measure = false) { check(dqmc_sweep_beta_to_0(b_, measure)); }
  // sweep_for_dynamic_greens (include/dqmc_walker.h:131) + G(k,tau) at the listed tau; the
  // accessors below return one entry per tau of the last list
  void sweep_for_dynamic_greens(const std::vector<int>& taus) {
    check(dqmc_sweep_dynamic(b_, taus.data(), (int)taus.size()));
    ntau_ = (int)taus.size();
  }
  // G(k,tau) accumulators of walker w in the order of the last tau list
  std::vector<double> DynamicGreens(int w, std::vector<int64_t>* counts = nullptr) const {
    std::vector<double> s(std::max(ntau_, 1));
    std::vector<int64_t> c(std::max(ntau_, 1));
    check(dqmc_get_dynamic(b_, w, s.data(), c.data()));
    s.resize(ntau_);
    c.resize(ntau_);
    if (counts) *counts = c;
    return s;
  }
  // per-displacement sums [tau][r] of the time-displaced Green's function: G(k,tau) of
  // measure_greens_functions for any momentum list is sum_r FourierFactor(r, k) S[tau][r]
  std::vector<double> DynamicGreensR(int w) const {
    std::vector<double> s((size_t)std::max(ntau_, 1) * N_);
    check(dqmc_get_dynamic_r(b_, w, s.data()));
    s.resize((size_t)ntau_ * N_);
    return s;
  }
  // Dqmc::measure with the bins normalised on the device: [walker][bin][9]
  std::vector<double> MeasureBins(int nbins, int bin_size, int sweeps_between) {
    std::vector<double> out((size_t)n_ * std::max(nbins, 1) * DQMC_NUM_OBS);
    check(dqmc_measure_bins(b_, nbins, bin_size, sweeps_between, out.data()));
    out.resize((size_t)n_ * std::max(nbins, 0) * DQMC_NUM_OBS);
    return out;
  }
  // measure_density_of_states, measure_dynamic_spin_susceptibility and the per-tau terms of
  // measure_superfluid_stiffness (src/measure/measure_methods.cpp:315-461), sums per listed tau
  struct DynamicObservables { std::vector<double> density_of_states, spin_susceptibility, stiffness_terms; };
  DynamicObservables DynamicObs(int w) const {
    const size_t n = std::max(ntau_, 1);
    DynamicObservables o{std::vector<double>(n), std::vector<double>(n), std::vector<double>(n)};
    check(dqmc_get_dynamic_obs(b_, w, o.density_of_states.data(), o.spin_susceptibility.data(),
                               o.stiffness_terms.data()));
    o.density_of_states.resize(ntau_);
    o.spin_susceptibility.resize(ntau_);
    o.stiffness_terms.resize(ntau_);
    return o;
  }
  std::vector<double> Greent0Up(int w) const { return green_dyn(w, 0, 0); }  // G(beta,0) after the last dynamic half-sweep
  std::vector<double> Greent0Dn(int w) const { return green_dyn(w, 0, 1); }
  std::vector<double> Green0tUp(int w) const { return green_dyn(w, 1, 0); }
  std::vector<double> Green0tDn(int w) const { return green_dyn(w, 1, 1); }

  std::vector<double> GreenttUp(int w) const { return green(w, 0); }
  std::vector<double> GreenttDn(int w) const { return green(w, 1); }
  double ConfigSign(int w) const { double v; check(dqmc_get_config_sign(b_, w, &v)); return v; }
  double WrapError(int w) const { double v; check(dqmc_get_wrap_error(b_, w, &v)); return v; }
  int Walkers() const { return n_; }
  int SpaceSize() const { return N_; }
  int TimeSize() const { return lt_; }
  dqmc_batch* handle() const { return b_; }

 private:
  std::vector<double> green_dyn(int w, int which, int spin) const {
    std::vector<double> g((size_t)N_ * N_);
    check(dqmc_get_green_dynamic(b_, w, which, spin, g.data()));
    return g;
  }
  std::vector<double> green(int w, int spin) const {
    std::vector<double> g((size_t)N_ * N_);
    check(dqmc_get_green(b_, w, spin, g.data()));
    return g;
  }
  dqmc_batch* b_ = nullptr;
  int n_ = 0, N_ = 0, lt_ = 80, pace_ = 10;
  int ntau_ = 0;  // length of the last dynamic tau list
  double beta_ = 4.0;
};

// ---- Dqmc driver (src/dqmc.cpp:48-158), sweeps counted as half-sweeps ----------
struct Dqmc {
  static void sweep_forth_and_back(DqmcWalker& walker, MeasureHandler& meas) {
    walker.sweep_from_0_to_beta(meas.isEqualTime());
    walker.sweep_from_beta_to_0(meas.isEqualTime());
  }
  static void thermalize(DqmcWalker& walker, MeasureHandler& meas) {
    for (int s = 1; s <= meas.WarmUpSweeps() / 2; ++s) {
      walker.sweep_from_0_to_beta(false);
      walker.sweep_from_beta_to_0(false);
    }
  }
  // each bin pools every walker of the batch (the reference pools MPI ranks' bins)
  static void measure(DqmcWalker& walker, MeasureHandler& meas) {
    const int nw = walker.Walkers();
    std::vector<double> sums((size_t)nw * DQMC_NUM_OBS);
    std::vector<int64_t> counts((size_t)nw * DQMC_NUM_OBS);
    meas.bins.clear();
    for (int bin = 0; bin < meas.BinsNum(); ++bin) {
      check(dqmc_clear_observables(walker.handle()));
      for (int s = 1; s <= meas.BinsSize() / 2; ++s) sweep_forth_and_back(walker, meas);
      check(dqmc_get_observables_all(walker.handle(), sums.data(), counts.data()));
      for (int w = 0; w < nw; ++w) {  // normalize_stats (measure_handler.cpp:170-189)
        const double* s = &sums[(size_t)w * DQMC_NUM_OBS];
        const int64_t* c = &counts[(size_t)w * DQMC_NUM_OBS];
        const double sign = s[DQMC_OBS_SIGN] / (double)c[DQMC_OBS_SIGN];
        std::vector<double> b(DQMC_NUM_OBS);
        for (int k = 0; k < DQMC_OBS_SIGN; ++k) b[k] = s[k] / ((double)c[k] * sign);
        b[DQMC_OBS_SIGN] = std::fabs(sign);
        meas.bins.push_back(b);
      }
      for (int s = 0; s < meas.SweepsBetweenBins() / 2; ++s) {
        walker.sweep_from_0_to_beta(false);
        walker.sweep_from_beta_to_0(false);
      }
    }
  }
  static void analyse(MeasureHandler& meas) { meas.analyse_stats(); }
};

}  // namespace dqmc_gb300
