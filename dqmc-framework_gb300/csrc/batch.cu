// batch.cu — C-ABI implementation: batch arena, per-walker constants,
// parity-mode uniform streams and the half-sweep schedule.
//
// Schedule of one half-sweep (src/dqmc_walker.cpp:246-412), for step
// j = 0 .. nstack-1 of every walker:
//   segment kernel   slices of stabilization interval j (wrap, Metropolis,
//                    measurement, B-chain started from the pushed stack's top)
//   push kernel      stack push of the chain (QRP), right/left pop implicit
//   greens kernel    fresh G from both stacks, wrap error, trace
//   measure kernel   forward: the slice closing interval j;
//                    backward: slot Lt-1 after the final stabilization
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <random>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/dqmc_gb300.h"
#include "dqmc_device.cuh"
#include "ozaki.cuh"

namespace dqmc {
cudaError_t configure_fp64_kernels(int maxN);
void launch_segment(int mode, const WalkerDev* W, int nw, int j, int measure, int maxN, cudaStream_t st);
void launch_push(int mode, const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st);
void launch_greens(int mode, const WalkerDev* W, int nw, int j, int check, int trace_slot, int maxN, cudaStream_t st);
void launch_measure(int mode, const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st);
void launch_sign(const WalkerDev* W, int nw, int maxN, cudaStream_t st);
double run_fp64_probe(cudaError_t* err);
void launch_bump(unsigned long long* ctr, cudaStream_t st);
void launch_bin_close(const WalkerDev* W, int nw, double* bins, int nbins, int bin, cudaStream_t st);
// general (N > 64) walkers, kernels_general.cu
cudaError_t configure_general_kernels();
void general_slice_pre(int mode, const WalkerDev* W, int nw, int j, int q, int maxN, bool any_dense, bool any_cb,
                       bool mixed, cudaStream_t st);
void general_slice_metro(int mode, const WalkerDev* W, int nw, int j, int q, int maxN, int measure, bool mixed,
                         int kd, int smax, int tc_flush, cudaStream_t st);
void general_slice_post(int mode, const WalkerDev* W, int nw, int j, int q, int maxN, bool any_dense, bool any_cb,
                        bool mixed, cudaStream_t st);
void launch_metropolis_delayed(bool mixed, const WalkerDev* W, int nw, int mode, int j, int q, int maxN, int S_max,
                               int KD, int tc_flush, cudaStream_t st);
size_t delayed_smem_bytes_host(int N, int S, int KD);
cudaError_t configure_delayed_kernels();
cudaError_t configure_submatrix_kernel();
size_t submatrix_scratch_bytes(int N);
void launch_metropolis_sub(const WalkerDev* W, int nw, int mode, int j, int q, int maxN, int S_max, cudaStream_t st);
void launch_metropolis_sub_split(const WalkerDev* W, int nw, int mode, int j, int q, int maxN, int S_max,
                                 cudaStream_t st);
int delayed_pick_kd(int N, int S);
void general_chain_init(int mode, const WalkerDev* W, int nw, int j, cudaStream_t st);
void general_push(int mode, const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st);
void general_dynamic_wrap(const WalkerDev* W, int nw, int j, int q, int maxN, bool mixed, bool any_dense,
                          bool any_cb, cudaStream_t st);
void general_dynamic_prop(const WalkerDev* W, int nw, int j, int q, int maxN, bool mixed, bool any_dense,
                          bool any_cb, cudaStream_t st);
void general_dynamic_chain(const WalkerDev* W, int nw, int j, int q, int maxN, bool mixed, bool any_dense,
                           bool any_cb, cudaStream_t st);
void general_dynamic_stab(const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st);
void general_dynamic_stab_measure(const WalkerDev* W, int nw, int j, cudaStream_t st);
void general_dynamic_begin(const WalkerDev* W, int nw, cudaStream_t st);
void general_dynamic_end(const WalkerDev* W, int nw, int maxN, cudaStream_t st);
void oz_push(int mode, const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st);
void oz_greens(int mode, const WalkerDev* W, int nw, int j, int trace_slot, int maxN, cudaStream_t st,
               bool dyn = false);
cudaError_t configure_stab_oz_kernels(int maxN);
void general_greens(int mode, const WalkerDev* W, int nw, int j, int trace_slot, int maxN, cudaStream_t st);
void general_measure_after(int mode, const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st);
void general_sign(const WalkerDev* W, int nw, int maxN, cudaStream_t st);
// mixed-precision products, kernels_ozaki.cu
cudaError_t configure_ozaki_kernels();
void mixed_wrap_fwd(const WalkerDev* W, int nw, int maxN, int j, int q, cudaStream_t st);
void mixed_wrap_bwd(const WalkerDev* W, int nw, int maxN, int j, int q, cudaStream_t st);
void mixed_chain(const WalkerDev* W, int nw, int maxN, int mode, int j, int q, cudaStream_t st);
void oz_slice_const(const double* X, unsigned short* out, int* exps, int N, int ldk, int role, int bits, int slices,
                    int layout, cudaStream_t st);
void oz_set_shape(int shape);
void oz_selftest(const double* A, const double* B, double* C, unsigned short* sa, int* ea, unsigned short* sb, int* eb,
                 int N, cudaStream_t st);
}  // namespace dqmc

using namespace dqmc;

namespace {

// walkers of the tensor-core path with 128 <= N <= 768 are stabilized by the
// blocked QR of kernels_stab_oz.cu (its FP64 panel of 32 columns fits shared memory)
constexpr int kMaxOzN = 768;
bool uses_ozstab(int N, int precision) { return precision == DQMC_MIXED && N >= 128 && N <= kMaxOzN; }

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_err = buf;
  return code;
}

#define CUDA_TRY(expr)                                                                  \
  do {                                                                                  \
    cudaError_t e_ = (expr);                                                            \
    if (e_ != cudaSuccess) return fail(DQMC_ERR_CUDA, "%s: %s", #expr, cudaGetErrorString(e_)); \
  } while (0)

// exp(x K) and exp(-x K) for symmetric K by one cyclic Jacobi diagonalisation (host, once
// per lattice in a batch).
std::pair<std::vector<double>, std::vector<double>> sym_exp_pair(int n, std::vector<double> a, double x) {
  auto A = [&](int r, int c) -> double& { return a[(size_t)c * n + r]; };
  std::vector<double> v((size_t)n * n, 0.0);
  auto V = [&](int r, int c) -> double& { return v[(size_t)c * n + r]; };
  for (int i = 0; i < n; ++i) V(i, i) = 1.0;
  for (int sweep = 0; sweep < 100; ++sweep) {
    double off = 0, dg = 0;
    for (int c = 0; c < n; ++c)
      for (int r = 0; r < n; ++r) (r == c ? dg : off) += A(r, c) * A(r, c);
    if (off == 0.0 || off <= 1e-32 * (dg + off)) break;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        const double apq = A(p, q);
        if (apq == 0.0) continue;
        const double th = (A(q, q) - A(p, p)) / (2 * apq);
        const double t = (th >= 0 ? 1.0 : -1.0) / (std::fabs(th) + std::sqrt(th * th + 1));
        const double c = 1 / std::sqrt(t * t + 1), s = t * c;
        for (int k = 0; k < n; ++k) {
          const double x1 = A(k, p), x2 = A(k, q);
          A(k, p) = c * x1 - s * x2;
          A(k, q) = s * x1 + c * x2;
        }
        for (int k = 0; k < n; ++k) {
          const double x1 = A(p, k), x2 = A(q, k);
          A(p, k) = c * x1 - s * x2;
          A(q, k) = s * x1 + c * x2;
        }
        for (int k = 0; k < n; ++k) {
          const double x1 = V(k, p), x2 = V(k, q);
          V(k, p) = c * x1 - s * x2;
          V(k, q) = s * x1 + c * x2;
        }
      }
  }
  auto form = [&](double y) {
    std::vector<double> out((size_t)n * n, 0.0);
    for (int m = 0; m < n; ++m) {
      const double e = std::exp(y * A(m, m));
      for (int c = 0; c < n; ++c) {
        const double vc = V(c, m) * e;
        for (int r = 0; r < n; ++r) out[(size_t)c * n + r] += V(r, m) * vc;
      }
    }
    return out;
  };
  return {form(x), form(-x)};
}

int lattice_sites(int L, int dim) { return dim == 3 ? L * L * L : L * L; }
int desc_sites(const dqmc_walker_desc& d) { return lattice_sites(d.L, d.lattice == DQMC_CUBIC ? 3 : 2); }

// K = -t H + mu I on the periodic square lattice (src/lattice/square.cpp:164-177) or cubic
// lattice (src/lattice/cubic.cpp:203-219): bonds to the +x, +y (, +z) neighbours, the hopping
// matrix zero-initialised.
std::vector<double> kinetic_matrix(int L, double t, double mu, int dim) {
  const int N = lattice_sites(L, dim);
  std::vector<double> K((size_t)N * N, 0.0);
  for (int i = 0; i < N; ++i) {
    const int x = i % L, y = (i / L) % L, z = i / (L * L);
    const int jx = i - x + (x + 1) % L, jy = i + ((y + 1) % L - y) * L, jz = i + ((z + 1) % L - z) * L * L;
    for (int a = 0; a < dim; ++a) {
      const int j = a == 0 ? jx : a == 1 ? jy : jz;
      K[(size_t)j * N + i] += -t;
      K[(size_t)i * N + j] += -t;
    }
  }
  for (int i = 0; i < N; ++i) K[(size_t)i * N + i] += mu;
  return K;
}

// The k stars of the lattice (src/lattice/square.cpp:42-66: the triangle (0,0), (pi,0),
// (pi,pi); src/lattice/cubic.cpp:47-81: the tetrahedron (0,0,0), (pi,0,0), (pi,pi,0),
// (pi,pi,pi), z outermost), as (kx, ky, kz) triples.
std::vector<std::array<double, 3>> k_stars(int L, int dim) {
  std::vector<std::array<double, 3>> ks;
  const auto mom = [&](int i) { return (double)i / L * 2 * M_PI - M_PI; };
  const int lo = (L + 1) / 2;
  if (dim == 2) {
    for (int i = lo; i <= L; ++i)
      for (int j = lo; j <= i; ++j) ks.push_back({mom(i), mom(j), 0.0});
  } else {
    for (int k = lo; k <= L; ++k)
      for (int i = k; i <= L; ++i)
        for (int j = k; j <= i; ++j) ks.push_back({mom(i), mom(j), mom(k)});
  }
  return ks;
}

// Fourier factors cos(-r.k) per displacement index (the site index of the displacement
// vector) for k-star kidx (src/lattice/square.cpp:148-161, cubic.cpp:186-200).
std::vector<double> fourier_table(int L, int kidx, int dim) {
  const auto ks = k_stars(L, dim);
  if (kidx < 0) kidx = (int)ks.size() - 1;  // (pi, pi) or (pi, pi, pi)
  const int N = lattice_sites(L, dim);
  std::vector<double> f((size_t)N);
  for (int d = 0; d < N; ++d) {
    const int x = d % L, y = (d / L) % L, z = d / (L * L);
    f[d] = (dim == 2) ? std::cos(-x * ks[kidx][0] - y * ks[kidx][1])
                      : std::cos(-x * ks[kidx][0] - y * ks[kidx][1] - z * ks[kidx][2]);
  }
  return f;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

// exp(-dtau K) and exp(+dtau K) of a lattice, kept for the life of the process: the Jacobi
// diagonalisation costs seconds at N = 576 and every batch of the same lattice reuses it
std::pair<std::vector<double>, std::vector<double>> dense_exponentials(int L, int dim, double t, double mu,
                                                                       double dtau) {
  static std::mutex mu_cache;
  static std::map<std::tuple<int, int, double, double, double>, std::pair<std::vector<double>, std::vector<double>>>
      cache;
  const auto key = std::make_tuple(L, dim, t, mu, dtau);
  {
    std::lock_guard<std::mutex> lock(mu_cache);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
  }
  auto v = sym_exp_pair(lattice_sites(L, dim), kinetic_matrix(L, t, mu, dim), -dtau);
  std::lock_guard<std::mutex> lock(mu_cache);
  return cache.emplace(key, std::move(v)).first->second;
}

}  // namespace

namespace dqmc {
int set_last_error(int code, const char* msg) { return fail(code, "%s", msg); }
}  // namespace dqmc

struct dqmc_batch {
  int nw = 0, maxN = 0, maxNs = 0, maxLt = 0;
  // walkers split by kernel family: N <= 64 (SMEM-resident) and N > 64 (general)
  int maxN_small = 0, maxN_general = 0, maxPace_general = 0;
  bool any_small = false, any_general = false, any_general_dense = false, any_general_cb = false;
  bool any_ozstab = false;  // walkers stabilized by the tensor-core blocked QR
  int maxN_oz = 0;
  bool mixed = false;
  int kd = 0, smax = 1;  // delayed-update block size of the general walkers (0: rank-1 kernel)
  // Metropolis of HBM walkers: 0 delayed with FP64 flush, 1 delayed with tensor-core
  // flush, 2 submatrix updates with tensor-core flush (mixed walkers, one CTA per walker),
  // 3 the same split per 32-site block into a decision and a multi-CTA flush kernel
  int tc_flush = 1;
  bool tuned = false;
  std::vector<std::pair<std::pair<int, int>, float>> tune_log;  // ((kd, tc), ms) per candidate
  // tile shape of the tensor-core wrap and chain products (oz_set_shape), tuned with the
  // time of one slice's products of the whole batch per shape
  int oz_shape = 0;
  bool shape_tuned = false;
  std::vector<std::pair<int, float>> shape_log;
  dqmc_batch_options opt{};
  std::vector<dqmc_walker_desc> desc;
  std::vector<WalkerDev> hw;        // host copies of the descriptors
  // dynamic half-sweep: buffers allocated on first use, the listed tau, stack position
  char* dyn_arena = nullptr;
  // shared-memory walkers (N <= 64) take the HBM path's kernels in the dynamic half-sweep:
  // their ping-pong chain, product temporary and stabilization scratch, per walker
  struct DynGen { double* chain = nullptr; double* work = nullptr; double* scr = nullptr; };
  std::vector<DynGen> dyn_gen;
  // the dynamic half-sweep captured once (walker-group branches) and its kernel nodes
  cudaGraphExec_t dyn_exec = nullptr;
  int64_t dyn_nodes = 0;
  int* d_taus = nullptr;
  std::vector<int> taus;
  bool at_zero = false;  // stacks of t = 0 (after set-up or a backward half-sweep)
  WalkerDev* dW = nullptr;          // device descriptors
  char* arena = nullptr;
  size_t arena_bytes = 0;
  cudaStream_t own = nullptr, stream = nullptr;
  // the general walkers' half-sweep runs as ngroups independent branches (walker
  // ranges on their own streams, forked from and joined to `stream`), so that the
  // latency-bound kernels of one group overlap the other groups' work
  static constexpr int kMaxGroups = 16;
  int ngroups = 1;
  cudaStream_t gst[kMaxGroups] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[kMaxGroups] = {};
  std::vector<std::minstd_rand0> eng;
  double* h_uni = nullptr;          // pinned [nw][maxLt*maxN]
  double* d_uni = nullptr;
  size_t uni_stride = 0;
  bool initialised = false;
  unsigned long long* d_sweep = nullptr;  // Philox half-sweep counter (device)
  // one CUDA graph per (mode, measure) half-sweep; kernel-node counts for accounting
  cudaGraphExec_t gexec[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
  // profiled graphs: the same half-sweep with CUDA-event nodes around each kernel class
  cudaGraphExec_t pexec[3][2] = {{nullptr, nullptr}, {nullptr, nullptr}, {nullptr, nullptr}};
  int64_t nodes[3][2] = {{-1, -1}, {-1, -1}, {-1, -1}};
  int64_t launches = 0;
  int trace_count = 0, trace_cap = 0;
  // per-walker device scalars
  struct Scal {
    double sign, sign_Lt;
    unsigned long long wrap_bits;
    long long accepts;
    int status, pad;
    double obs[kNumObs];
    long long obs_cnt[kNumObs];
  };
  Scal* d_scal = nullptr;
  // kernel-class profiling: event pairs recorded around launches
  bool prof = false;
  struct Mark { int cls; cudaEvent_t a, b; };
  std::vector<Mark> marks;
  std::vector<Mark> pmarks[3][2];  // event nodes of the profiled graphs
  std::vector<cudaEvent_t> pool;
  double prof_ms[DQMC_NUM_KCLASS] = {};
  int64_t prof_n[DQMC_NUM_KCLASS] = {};
  cudaEvent_t ev() {
    if (pool.empty()) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      return e;
    }
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  bool capturing = false;  // inside a stream capture: events become graph event-record nodes
  template <class F>
  void timed(int cls, F launch) {
    if (!prof) { launch(); return; }
    Mark m{cls, ev(), ev()};
    const unsigned fl = capturing ? cudaEventRecordExternal : 0u;
    cudaEventRecordWithFlags(m.a, stream, fl);
    launch();
    cudaEventRecordWithFlags(m.b, stream, fl);
    marks.push_back(m);
  }
  void collect() {
    for (auto& m : marks) {
      float ms = 0;
      cudaEventSynchronize(m.b);
      cudaEventElapsedTime(&ms, m.a, m.b);
      prof_ms[m.cls] += ms;
      prof_n[m.cls] += 1;
      pool.push_back(m.a);
      pool.push_back(m.b);
    }
    marks.clear();
  }
};

extern "C" {

const char* dqmc_last_error(void) { return g_err.c_str(); }
int dqmc_abi_version(void) { return DQMC_ABI_VERSION; }

int dqmc_batch_create(const dqmc_walker_desc* descs, int n, const dqmc_batch_options* opt, dqmc_batch** out) {
  if (!descs || n <= 0 || !out) return fail(DQMC_ERR_ARG, "dqmc_batch_create: null argument or n_walkers <= 0");
  *out = nullptr;
  dqmc_batch_options o{};
  if (opt) o = *opt;
  if (o.rng != DQMC_RNG_MINSTD && o.rng != DQMC_RNG_PHILOX) return fail(DQMC_ERR_ARG, "unknown rng mode %d", o.rng);
  if (o.precision != DQMC_FP64 && o.precision != DQMC_MIXED)
    return fail(DQMC_ERR_ARG, "unknown precision mode %d", o.precision);
  for (int w = 0; w < n; ++w) {
    const auto& d = descs[w];
    if (d.model != DQMC_REPULSIVE_HUBBARD && d.model != DQMC_ATTRACTIVE_HUBBARD)
      return fail(DQMC_ERR_ARG, "walker %d: unknown model %d", w, d.model);
    if (d.lattice != DQMC_SQUARE && d.lattice != DQMC_CUBIC)
      return fail(DQMC_ERR_ARG, "walker %d: unknown lattice %d", w, d.lattice);
    if (d.L < 2) return fail(DQMC_ERR_ARG, "walker %d: lattice side %d < 2", w, d.L);
    if (d.L > kMaxN || desc_sites(d) > kMaxN)
      return fail(DQMC_ERR_ARG, "walker %d: N = %lld exceeds the supported %d", w,
                  (long long)d.L * d.L * (d.lattice == DQMC_CUBIC ? d.L : 1), kMaxN);
    if (d.checkerboard && d.lattice == DQMC_CUBIC)  // dqmc_initializer.cpp:169-182
      return fail(DQMC_ERR_ARG, "walker %d: the checkerboard break-up is built for the square lattice only", w);
    if (d.checkerboard && (d.L % 2)) return fail(DQMC_ERR_ARG, "walker %d: checkerboard needs an even side", w);
    if (d.Lt < 1 || d.pace < 1) return fail(DQMC_ERR_ARG, "walker %d: Lt and pace must be >= 1", w);
    if (!(d.beta > 0) || !(d.onsite_u >= 0) || !(d.hopping_t >= 0))
      return fail(DQMC_ERR_ARG, "walker %d: need beta > 0, U >= 0, t >= 0", w);
    const int nk = (int)k_stars(d.L, d.lattice == DQMC_CUBIC ? 3 : 2).size();
    if (d.momentum_index >= nk) return fail(DQMC_ERR_ARG, "walker %d: momentum index out of range", w);
  }
  int dev_count = 0;
  if (cudaGetDeviceCount(&dev_count) != cudaSuccess || dev_count == 0)
    return fail(DQMC_ERR_CUDA, "no CUDA device available");

  auto* b = new dqmc_batch();
  b->nw = n;
  b->opt = o;
  b->desc.assign(descs, descs + n);
  for (auto& d : b->desc) {
    const int N = desc_sites(d);
    if (N > kMaxSmemN || o.precision == DQMC_MIXED || o.hbm) {
      b->any_general = true;
      b->maxN_general = std::max(b->maxN_general, N);
      b->maxPace_general = std::max(b->maxPace_general, d.pace);
      if (d.checkerboard) b->any_general_cb = true; else b->any_general_dense = true;
      if (uses_ozstab(N, o.precision)) {
        b->any_ozstab = true;
        b->maxN_oz = std::max(b->maxN_oz, N);
      }
    } else {
      b->any_small = true;
      b->maxN_small = std::max(b->maxN_small, N);
    }
    b->maxN = std::max(b->maxN, desc_sites(d));
    const int ns = (d.Lt % d.pace == 0) ? d.Lt / d.pace : d.Lt / d.pace + 1;
    b->maxNs = std::max(b->maxNs, ns);
    b->maxLt = std::max(b->maxLt, d.Lt);
  }
  b->trace_cap = o.trace ? 4 * b->maxNs : 0;
  b->mixed = (o.precision == DQMC_MIXED);
  for (auto& d : b->desc)
    if (d.model == DQMC_REPULSIVE_HUBBARD) b->smax = 2;
  if (b->any_general) b->kd = delayed_pick_kd(b->maxN_general, b->smax);
  if (b->mixed) b->tc_flush = 2;  // submatrix updates until the tuner has timed the candidates

  // ---- arena layout ----
  struct Off { size_t G, chain, work, scr, sl, sle, stack, fields, ff, trace, msub, zsl; int dense_id; };
  std::vector<Off> off(n);
  std::map<std::tuple<int, int, double, double, double>, int> dense_ids;  // (L, dim, t, mu, dtau) -> id
  std::vector<std::pair<std::vector<double>, std::vector<double>>> dense;
  std::map<std::tuple<int, int, int>, size_t> ff_off;  // (L, dim, k star) -> offset
  size_t cur = 0;
  auto take = [&](size_t bytes) { size_t o2 = cur; cur = align256(cur + bytes); return o2; };
  const size_t scal_off = take(sizeof(dqmc_batch::Scal) * n);
  const size_t sweep_off = take(sizeof(unsigned long long));
  const size_t desc_off = take(sizeof(WalkerDev) * n);
  for (int w = 0; w < n; ++w) {
    const auto& d = b->desc[w];
    const int N = desc_sites(d);
    const int S = (d.model == DQMC_ATTRACTIVE_HUBBARD) ? 1 : 2;
    const int ns = (d.Lt % d.pace == 0) ? d.Lt / d.pace : d.Lt / d.pace + 1;
    const size_t lvl = (2 * (size_t)N * N + N + 31) & ~(size_t)31;
    const bool general = N > kMaxSmemN || o.precision == DQMC_MIXED || o.hbm;
    const int ldk = (N + 15) / 16 * 16;
    off[w].sl = (o.precision == DQMC_MIXED)
                    ? take(sizeof(unsigned short) * S * ozaki::kMaxSlices * ozaki::tc_slice_elems(N, ldk)) : 0;
    off[w].sle = (o.precision == DQMC_MIXED) ? take(sizeof(int) * S * (size_t)N) : 0;
    off[w].G = take(sizeof(double) * 2 * N * N);
    off[w].chain = take(sizeof(double) * (general ? 2 : 1) * S * N * N);
    off[w].work = general ? take(sizeof(double) * S * N * N) : 0;
    off[w].scr = general ? take(sizeof(double) * 2 * S * N * N) : 0;
    off[w].stack = take(sizeof(double) * 2 * S * ns * lvl);
    off[w].fields = take((size_t)d.Lt * N);
    off[w].trace = b->trace_cap ? take(sizeof(double) * (size_t)b->trace_cap * 2 * N * N) : 0;
    off[w].msub = (o.precision == DQMC_MIXED) ? take((size_t)S * submatrix_scratch_bytes(N)) : 0;
    off[w].zsl = uses_ozstab(N, o.precision)
                     ? take(sizeof(unsigned short) * (size_t)S * 2 * 9 * ozaki::tc_lines(N) * (size_t)((N + 31) / 32 * 32))
                     : 0;
    off[w].dense_id = -1;
    if (!d.checkerboard) {
      const int dim = d.lattice == DQMC_CUBIC ? 3 : 2;
      auto key = std::make_tuple(d.L, dim, d.hopping_t, d.mu, d.beta / d.Lt);
      auto it = dense_ids.find(key);
      if (it == dense_ids.end()) {
        dense.push_back(dense_exponentials(d.L, dim, d.hopping_t, d.mu, d.beta / d.Lt));
        it = dense_ids.emplace(key, (int)dense.size() - 1).first;
      }
      off[w].dense_id = it->second;
    }
    auto fk = std::make_tuple(d.L, d.lattice == DQMC_CUBIC ? 3 : 2, d.momentum_index < 0 ? -1 : d.momentum_index);
    if (!ff_off.count(fk)) ff_off[fk] = take(sizeof(double) * N);
    off[w].ff = ff_off[fk];
  }
  std::vector<size_t> dense_off(dense.size()), dense_sl(dense.size()), dense_sle(dense.size());
  std::vector<int> dense_n(dense.size());
  for (auto& kv : dense_ids) dense_n[kv.second] = lattice_sites(std::get<0>(kv.first), std::get<1>(kv.first));
  for (size_t i = 0; i < dense.size(); ++i) {
    const size_t nn = dense[i].first.size();
    dense_off[i] = take(sizeof(double) * 2 * nn);
    if (o.precision == DQMC_MIXED) {  // 4 sliced copies: expK (A, B roles), invK (A, B roles)
      const int N = dense_n[i], ldk = (N + 15) / 16 * 16;
      dense_sl[i] = take(sizeof(unsigned short) * 4 * ozaki::kMaxSlices * ozaki::tc_slice_elems(N, ldk));
      dense_sle[i] = take(sizeof(int) * 4 * (size_t)N);
    }
  }
  b->uni_stride = (size_t)b->maxLt * b->maxN;
  const size_t uni_off = (o.rng == DQMC_RNG_MINSTD) ? take(sizeof(double) * b->uni_stride * n) : 0;
  b->arena_bytes = cur;

  cudaError_t e = cudaMalloc(&b->arena, b->arena_bytes);
  if (e != cudaSuccess) {
    delete b;
    return fail(DQMC_ERR_CUDA, "cudaMalloc(%zu bytes): %s", cur, cudaGetErrorString(e));
  }
  e = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = configure_fp64_kernels(kMaxSmemN);
  if (e == cudaSuccess) e = configure_general_kernels();
  if (e == cudaSuccess) e = configure_ozaki_kernels();
  if (e == cudaSuccess) e = configure_delayed_kernels();
  if (e == cudaSuccess) e = configure_submatrix_kernel();
  if (e == cudaSuccess) e = configure_stab_oz_kernels(kMaxOzN);
  if (e != cudaSuccess) {
    dqmc_batch_destroy(b);  // frees the arena and the stream, if it was created
    return fail(DQMC_ERR_CUDA, "stream/kernel set-up: %s", cudaGetErrorString(e));
  }
  b->stream = b->own;
  {
    // walker groups of the general path: one branch per 8 walkers, up to 16
    // (DQMC_STREAM_GROUPS=1..16 overrides)
    int ng = std::min(16, std::max(1, n / 8));
    if (const char* env = std::getenv("DQMC_STREAM_GROUPS")) ng = std::atoi(env);
    b->ngroups = std::max(1, std::min(ng, dqmc_batch::kMaxGroups));
    for (int g = 0; g < b->ngroups && e == cudaSuccess; ++g) {
      e = cudaStreamCreateWithFlags(&b->gst[g], cudaStreamNonBlocking);
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join[g], cudaEventDisableTiming);
    }
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e != cudaSuccess) {
      dqmc_batch_destroy(b);
      return fail(DQMC_ERR_CUDA, "stream groups: %s", cudaGetErrorString(e));
    }
  }
  cudaMemsetAsync(b->arena, 0, b->arena_bytes, b->stream);

  char* base = b->arena;
  b->d_scal = reinterpret_cast<dqmc_batch::Scal*>(base + scal_off);
  b->d_sweep = reinterpret_cast<unsigned long long*>(base + sweep_off);
  b->dW = reinterpret_cast<WalkerDev*>(base + desc_off);
  if (o.rng == DQMC_RNG_MINSTD) {
    b->d_uni = reinterpret_cast<double*>(base + uni_off);
    e = cudaMallocHost(&b->h_uni, sizeof(double) * b->uni_stride * n);
    if (e != cudaSuccess) {
      b->h_uni = nullptr;
      dqmc_batch_destroy(b);
      return fail(DQMC_ERR_CUDA, "cudaMallocHost(%zu bytes): %s", sizeof(double) * b->uni_stride * n,
                  cudaGetErrorString(e));
    }
  }
  // upload dense matrices and Fourier tables
  for (size_t i = 0; i < dense.size(); ++i) {
    const size_t nn = dense[i].first.size();
    cudaMemcpyAsync(base + dense_off[i], dense[i].first.data(), sizeof(double) * nn, cudaMemcpyHostToDevice, b->stream);
    cudaMemcpyAsync(base + dense_off[i] + sizeof(double) * nn, dense[i].second.data(), sizeof(double) * nn,
                    cudaMemcpyHostToDevice, b->stream);
    if (o.precision == DQMC_MIXED) {
      const int N = dense_n[i], ldk = (N + 15) / 16 * 16;
      const auto c = ozaki::cfg_for_k(N);
      const auto cfg = std::make_pair(c.bits, c.slices);
      const size_t one = ozaki::kMaxSlices * ozaki::tc_slice_elems(N, ldk);
      auto* sl = reinterpret_cast<unsigned short*>(base + dense_sl[i]);
      auto* se = reinterpret_cast<int*>(base + dense_sle[i]);
      const double* ek = reinterpret_cast<const double*>(base + dense_off[i]);
      const double* ik = ek + nn;
      oz_slice_const(ek, sl + 0 * one, se + 0 * N, N, ldk, 0, cfg.first, cfg.second, 1, b->stream);  // expK as A
      oz_slice_const(ek, sl + 1 * one, se + 1 * N, N, ldk, 1, cfg.first, cfg.second, 1, b->stream);  // expK as B
      oz_slice_const(ik, sl + 2 * one, se + 2 * N, N, ldk, 0, cfg.first, cfg.second, 1, b->stream);  // invK as A
      oz_slice_const(ik, sl + 3 * one, se + 3 * N, N, ldk, 1, cfg.first, cfg.second, 1, b->stream);  // invK as B
    }
  }
  std::vector<std::vector<double>> fftabs;
  for (auto& kv : ff_off) {
    fftabs.push_back(fourier_table(std::get<0>(kv.first), std::get<2>(kv.first), std::get<1>(kv.first)));
    cudaMemcpyAsync(base + kv.second, fftabs.back().data(), sizeof(double) * fftabs.back().size(),
                    cudaMemcpyHostToDevice, b->stream);
  }

  b->hw.resize(n);
  b->eng.resize(n);
  std::vector<dqmc_batch::Scal> scal(n);
  for (int w = 0; w < n; ++w) {
    const auto& d = b->desc[w];
    WalkerDev& h = b->hw[w];
    std::memset(&h, 0, sizeof h);
    const int N = desc_sites(d);
    h.N = N;
    h.L = d.L;
    h.dim = (d.lattice == DQMC_CUBIC) ? 3 : 2;
    h.Lt = d.Lt;
    h.pace = d.pace;
    h.nstack = (d.Lt % d.pace == 0) ? d.Lt / d.pace : d.Lt / d.pace + 1;
    h.S = (d.model == DQMC_ATTRACTIVE_HUBBARD) ? 1 : 2;
    h.model = d.model;
    h.cb = d.checkerboard;
    h.rng = o.rng;
    h.hop_t = d.hopping_t;
    const double dtau = d.beta / d.Lt;
    const double alpha = std::acosh(std::exp(0.5 * dtau * d.onsite_u));  // repulsive_hubbard.cpp:50
    // exactly the exponentials the reference evaluates, s = +1 and s = -1
    h.e_pa = std::exp(+1.0 * alpha * 1.0);
    h.e_ma = std::exp(-1.0 * alpha * 1.0);
    for (int si = 0; si < 2; ++si) {
      const double s = si == 0 ? 1.0 : -1.0;
      h.cm[si] = std::exp(-2 * alpha * s) - 1;
      h.cp[si] = std::exp(+2 * alpha * s) - 1;
      h.ex2[si] = std::exp(2 * alpha * s);
    }
    auto plaq = [](double* m, double ch, double sh, double f) {
      const double v[16] = {ch * ch, ch * sh, ch * sh, sh * sh, ch * sh, ch * ch, sh * sh, ch * sh,
                            ch * sh, sh * sh, ch * ch, ch * sh, sh * sh, ch * sh, ch * sh, ch * ch};
      for (int k = 0; k < 16; ++k) m[k] = f * v[k];
    };
    // checkerboard/square.cpp:34-49 (note its exp(+0.5 dtau mu) sign)
    plaq(h.cbP, std::cosh(dtau * d.hopping_t), std::sinh(dtau * d.hopping_t), std::exp(0.5 * dtau * d.mu));
    plaq(h.cbI, std::cosh(-dtau * d.hopping_t), std::sinh(-dtau * d.hopping_t), std::exp(-0.5 * dtau * d.mu));
    h.G = reinterpret_cast<double*>(base + off[w].G);
    h.chain = reinterpret_cast<double*>(base + off[w].chain);
    const bool gen = N > kMaxSmemN || o.precision == DQMC_MIXED || o.hbm;
    h.path = (o.precision == DQMC_MIXED) ? 2 : (gen ? 1 : 0);
    h.work = gen ? reinterpret_cast<double*>(base + off[w].work) : nullptr;
    h.scr = gen ? reinterpret_cast<double*>(base + off[w].scr) : nullptr;
    h.msub = (o.precision == DQMC_MIXED) ? reinterpret_cast<unsigned char*>(base + off[w].msub) : nullptr;
    h.ozstab = uses_ozstab(N, o.precision) ? 1 : 0;
    h.zld = (N + 31) / 32 * 32;
    h.zsl = h.ozstab ? reinterpret_cast<unsigned short*>(base + off[w].zsl) : nullptr;
    if (o.precision == DQMC_MIXED) {
      h.ldk = (N + 15) / 16 * 16;
      h.slice_bits = ozaki::cfg_for_k(N).bits;
      h.slices = ozaki::cfg_for_k(N).slices;
      h.sl = reinterpret_cast<unsigned short*>(base + off[w].sl);
      h.sle = reinterpret_cast<int*>(base + off[w].sle);
      if (off[w].dense_id >= 0) {
        const int id = off[w].dense_id;
        const size_t one = ozaki::kMaxSlices * ozaki::tc_slice_elems(N, h.ldk);
        auto* sl = reinterpret_cast<const unsigned short*>(base + dense_sl[id]);
        auto* se = reinterpret_cast<const int*>(base + dense_sle[id]);
        h.kA = sl; h.kB = sl + one; h.iA = sl + 2 * one; h.iB = sl + 3 * one;
        h.kAe = se; h.kBe = se + N; h.iAe = se + 2 * N; h.iBe = se + 3 * N;
      }
    }
    h.stack = reinterpret_cast<double*>(base + off[w].stack);
    h.lvl_stride = (long long)((2 * (size_t)N * N + N + 31) & ~(size_t)31);
    h.side_stride = (long long)h.S * h.nstack * h.lvl_stride;
    h.fields = reinterpret_cast<int8_t*>(base + off[w].fields);
    if (off[w].dense_id >= 0) {
      h.expK = reinterpret_cast<const double*>(base + dense_off[off[w].dense_id]);
      h.invK = h.expK + (size_t)N * N;
    }
    h.ff = reinterpret_cast<const double*>(base + off[w].ff);
    dqmc_batch::Scal* sc = b->d_scal + w;
    h.obs = sc->obs;
    h.obs_cnt = sc->obs_cnt;
    h.sign = &sc->sign;
    h.sign_Lt = &sc->sign_Lt;
    h.wrap_bits = &sc->wrap_bits;
    h.accepts = &sc->accepts;
    h.status = &sc->status;
    h.uni = b->d_uni ? b->d_uni + b->uni_stride * w : nullptr;
    h.seed = d.seed;
    h.widx = w;
    h.wait_limit = kDefaultWaitLimit;
    h.sweep_ctr = b->d_sweep;
    h.trace = b->trace_cap ? reinterpret_cast<double*>(base + off[w].trace) : nullptr;
    h.trace_cap = b->trace_cap;
    b->eng[w].seed((unsigned)d.seed);
    std::memset(&scal[w], 0, sizeof scal[w]);
    scal[w].sign = 1.0;
    // fields default to +1 until set
    std::vector<int8_t> ones((size_t)d.Lt * N, 1);
    cudaMemcpyAsync(h.fields, ones.data(), ones.size(), cudaMemcpyHostToDevice, b->stream);
    cudaStreamSynchronize(b->stream);
  }
  cudaMemcpyAsync(b->d_scal, scal.data(), sizeof(dqmc_batch::Scal) * n, cudaMemcpyHostToDevice, b->stream);
  cudaMemcpyAsync(b->dW, b->hw.data(), sizeof(WalkerDev) * n, cudaMemcpyHostToDevice, b->stream);
  e = cudaStreamSynchronize(b->stream);
  if (e != cudaSuccess) {
    dqmc_batch_destroy(b);
    return fail(DQMC_ERR_CUDA, "batch upload: %s", cudaGetErrorString(e));
  }
  *out = b;
  return DQMC_OK;
}

int dqmc_batch_destroy(dqmc_batch* b) {
  if (!b) return DQMC_OK;
  if (b->stream) cudaStreamSynchronize(b->stream);
  b->collect();
  for (auto e : b->pool) cudaEventDestroy(e);
  for (auto& row : b->gexec)
    for (auto& g : row)
      if (g) cudaGraphExecDestroy(g);
  for (auto& row : b->pexec)
    for (auto& g : row)
      if (g) cudaGraphExecDestroy(g);
  if (b->dyn_exec) cudaGraphExecDestroy(b->dyn_exec);
  for (auto& row : b->pmarks)
    for (auto& v : row)
      for (auto& m : v) { cudaEventDestroy(m.a); cudaEventDestroy(m.b); }
  if (b->h_uni) cudaFreeHost(b->h_uni);
  if (b->arena) cudaFree(b->arena);
  if (b->dyn_arena) cudaFree(b->dyn_arena);
  for (int g = 0; g < dqmc_batch::kMaxGroups; ++g) {
    if (b->gst[g]) cudaStreamDestroy(b->gst[g]);
    if (b->ev_join[g]) cudaEventDestroy(b->ev_join[g]);
  }
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->own) cudaStreamDestroy(b->own);
  delete b;
  return DQMC_OK;
}

int dqmc_set_stream(dqmc_batch* b, void* s) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->stream = s ? static_cast<cudaStream_t>(s) : b->own;
  return DQMC_OK;
}

int dqmc_synchronize(dqmc_batch* b) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}

static int check_walker(dqmc_batch* b, int w) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  if (w < 0 || w >= b->nw) return fail(DQMC_ERR_ARG, "walker index %d out of range [0,%d)", w, b->nw);
  return DQMC_OK;
}

int dqmc_fields_random(dqmc_batch* b, int w) {
  if (int r = check_walker(b, w)) return r;
  const auto& d = b->desc[w];
  const int N = desc_sites(d);
  std::vector<int8_t> f((size_t)d.Lt * N);
  for (int t = 0; t < d.Lt; ++t)
    for (int i = 0; i < N; ++i)  // bernoulli(0.5): u < 0.5 -> +1 (repulsive_hubbard.cpp:92-97)
      f[(size_t)t * N + i] = (std::generate_canonical<double, 53>(b->eng[w]) < 0.5) ? 1 : -1;
  CUDA_TRY(cudaMemcpyAsync(b->hw[w].fields, f.data(), f.size(), cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->initialised = false;
  return DQMC_OK;
}

int dqmc_set_fields(dqmc_batch* b, int w, const int8_t* f) {
  if (int r = check_walker(b, w)) return r;
  if (!f) return fail(DQMC_ERR_ARG, "null fields");
  const auto& d = b->desc[w];
  const size_t n = (size_t)d.Lt * desc_sites(d);
  for (size_t k = 0; k < n; ++k)
    if (f[k] != 1 && f[k] != -1) return fail(DQMC_ERR_ARG, "field value %d at %zu is not +/-1", (int)f[k], k);
  CUDA_TRY(cudaMemcpyAsync(b->hw[w].fields, f, n, cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->initialised = false;
  return DQMC_OK;
}

int dqmc_get_fields(dqmc_batch* b, int w, int8_t* f) {
  if (int r = check_walker(b, w)) return r;
  if (!f) return fail(DQMC_ERR_ARG, "null output");
  const auto& d = b->desc[w];
  CUDA_TRY(cudaMemcpyAsync(f, b->hw[w].fields, (size_t)d.Lt * desc_sites(d), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}

static int launch_check(const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return fail(DQMC_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  return DQMC_OK;
}

// Autotuner of the Metropolis of HBM walkers: times one slice of every walker
// for each candidate (block size k, update kind) on the batch's own state,
// restoring G, the fields and the walker scalars after each trial, and keeps
// the fastest.  Candidates: delayed updates with k in {32, 16, 8} that fit
// shared memory; on the mixed path, submatrix updates (k = 32) fused in one
// kernel per walker and split per block (decision and multi-CTA flush kernels),
// and each delayed k with the tensor-core flush and with the FP64 flush.
static int autotune_delayed(dqmc_batch* b) {
  std::vector<std::pair<int, int>> cand;
  const int kmax = b->kd;
  if (b->mixed) {
    cand.push_back({32, 2});
    cand.push_back({32, 3});
  }
  for (int kd : {32, 16, 8}) {
    if (kd > kmax) continue;
    if (b->mixed && kd >= 16) cand.push_back({kd, 1});
    cand.push_back({kd, 0});
  }
  // DQMC_METROPOLIS_KIND=0..3 keeps only the candidates of that update kind (tests)
  if (const char* env = std::getenv("DQMC_METROPOLIS_KIND")) {
    const int kind = std::atoi(env);
    std::vector<std::pair<int, int>> keep;
    for (auto c : cand)
      if (c.second == kind) keep.push_back(c);
    if (!keep.empty()) cand = keep;
  }
  // back up what one Metropolis slice changes: G (spins < S) into work, fields into scr
  std::vector<dqmc_batch::Scal> scal(b->nw);
  CUDA_TRY(cudaMemcpyAsync(scal.data(), b->d_scal, sizeof(dqmc_batch::Scal) * b->nw, cudaMemcpyDeviceToHost,
                           b->stream));
  for (int w = 0; w < b->nw; ++w) {
    const WalkerDev& h = b->hw[w];
    if (h.path == 0) continue;
    CUDA_TRY(cudaMemcpyAsync(h.work, h.G, sizeof(double) * h.S * h.N * h.N, cudaMemcpyDeviceToDevice, b->stream));
    CUDA_TRY(cudaMemcpyAsync(h.scr, h.fields, (size_t)h.Lt * h.N, cudaMemcpyDeviceToDevice, b->stream));
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  std::pair<int, int> pick = cand.empty() ? std::make_pair(b->kd, 1) : cand[0];
  b->tune_log.clear();
  for (auto c : cand) {
    for (int rep = 0; rep < 2; ++rep) {  // first run warms caches and code
      cudaEventRecord(e0, b->stream);
      if (c.second == 2)
        launch_metropolis_sub(b->dW, b->nw, MODE_FWD, 0, 0, b->maxN_general, b->smax, b->stream);
      else if (c.second == 3)
        launch_metropolis_sub_split(b->dW, b->nw, MODE_FWD, 0, 0, b->maxN_general, b->smax, b->stream);
      else
        launch_metropolis_delayed(b->mixed, b->dW, b->nw, MODE_FWD, 0, 0, b->maxN_general, b->smax, c.first,
                                  c.second, b->stream);
      cudaEventRecord(e1, b->stream);
      CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      for (int w = 0; w < b->nw; ++w) {  // restore
        const WalkerDev& h = b->hw[w];
        if (h.path == 0) continue;
        CUDA_TRY(cudaMemcpyAsync(h.G, h.work, sizeof(double) * h.S * h.N * h.N, cudaMemcpyDeviceToDevice, b->stream));
        CUDA_TRY(cudaMemcpyAsync(h.fields, h.scr, (size_t)h.Lt * h.N, cudaMemcpyDeviceToDevice, b->stream));
      }
      if (rep == 1) {
        b->tune_log.push_back({c, ms});
        if (ms < best) { best = ms; pick = c; }
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CUDA_TRY(cudaMemcpyAsync(b->d_scal, scal.data(), sizeof(dqmc_batch::Scal) * b->nw, cudaMemcpyHostToDevice,
                           b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (int r = launch_check("autotune")) return r;
  b->kd = pick.first;
  b->tc_flush = pick.second;
  b->tuned = true;
  return DQMC_OK;
}

// Tile shape of the tensor-core wrap and chain products: one forward slice's wrap and chain
// products of the whole batch timed with each shape (G backed up into the stabilization
// scratch and restored after each trial; work and the chain are rebuilt before they are
// read again), the faster kept.
static int autotune_products(dqmc_batch* b) {
  for (int w = 0; w < b->nw; ++w) {
    const WalkerDev& h = b->hw[w];
    if (h.path != 2) continue;
    CUDA_TRY(cudaMemcpyAsync(h.scr, h.G, sizeof(double) * h.S * h.N * h.N, cudaMemcpyDeviceToDevice, b->stream));
  }
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best = 1e30f;
  int pick = 0;
  b->shape_log.clear();
  std::vector<int> shapes = {0, 1};
  if (const char* env = std::getenv("DQMC_PRODUCT_TILE")) {  // holds the tuner to one shape (tests)
    const int s = std::atoi(env);
    if (s == 0 || s == 1) shapes = {s};
  }
  for (int shape : shapes) {
    oz_set_shape(shape);
    for (int rep = 0; rep < 2; ++rep) {  // first run warms caches and code
      cudaEventRecord(e0, b->stream);
      mixed_wrap_fwd(b->dW, b->nw, b->maxN_general, 0, 0, b->stream);
      mixed_chain(b->dW, b->nw, b->maxN_general, MODE_FWD, 0, 0, b->stream);
      cudaEventRecord(e1, b->stream);
      CUDA_TRY(cudaEventSynchronize(e1));
      float ms = 0;
      cudaEventElapsedTime(&ms, e0, e1);
      for (int w = 0; w < b->nw; ++w) {
        const WalkerDev& h = b->hw[w];
        if (h.path != 2) continue;
        CUDA_TRY(cudaMemcpyAsync(h.G, h.scr, sizeof(double) * h.S * h.N * h.N, cudaMemcpyDeviceToDevice, b->stream));
      }
      if (rep == 1) {
        b->shape_log.push_back({shape, ms});
        if (ms < best) { best = ms; pick = shape; }
      }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (int r = launch_check("product tile autotune")) return r;
  b->oz_shape = pick;
  oz_set_shape(pick);
  b->shape_tuned = true;
  return DQMC_OK;
}

int dqmc_init_greens(dqmc_batch* b) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  oz_set_shape(b->oz_shape);
  for (int j = 0; j < b->maxNs; ++j) {
    if (b->any_small) {
      launch_segment(MODE_INIT, b->dW, b->nw, j, 0, b->maxN_small, b->stream);
      launch_push(MODE_INIT, b->dW, b->nw, j, b->maxN_small, b->stream);
    }
    if (b->any_general) {
      general_chain_init(MODE_INIT, b->dW, b->nw, j, b->stream);
      for (int q = 0; q < b->maxPace_general; ++q)
        general_slice_post(MODE_INIT, b->dW, b->nw, j, q, b->maxN_general, b->any_general_dense, b->any_general_cb,
                           b->mixed, b->stream);  // the transposed B-chain of the initial right stack
      general_push(MODE_INIT, b->dW, b->nw, j, b->maxN_general, b->stream);
      if (b->any_ozstab) oz_push(MODE_INIT, b->dW, b->nw, j, b->maxN_oz, b->stream);
    }
  }
  if (b->any_small) {
    launch_greens(MODE_INIT, b->dW, b->nw, 0, 0, -1, b->maxN_small, b->stream);
    launch_sign(b->dW, b->nw, b->maxN_small, b->stream);
  }
  if (b->any_general) {
    general_greens(MODE_INIT, b->dW, b->nw, 0, -1, b->maxN_general, b->stream);
    if (b->any_ozstab) oz_greens(MODE_INIT, b->dW, b->nw, 0, -1, b->maxN_oz, b->stream);
    general_sign(b->dW, b->nw, b->maxN_general, b->stream);
  }
  if (int r = launch_check("init kernels")) return r;
  // wrap error and accumulators start from zero (DqmcWalker::initial, dqmc_walker.cpp:41-49)
  for (int w = 0; w < b->nw; ++w) {
    CUDA_TRY(cudaMemsetAsync(&b->d_scal[w].wrap_bits, 0, sizeof(unsigned long long), b->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->initialised = true;
  b->at_zero = true;
  b->trace_count = 0;
  if (b->any_general && (b->kd > 0 || b->mixed) && !b->tuned) {
    if (int r = autotune_delayed(b)) return r;
  }
  if (b->mixed && b->any_general_dense && !b->shape_tuned) {
    if (int r = autotune_products(b)) return r;
  }
  return DQMC_OK;
}

// Level j of the general walkers W[0..nw) on stream st (kernel classes timed when profiling).
static void issue_general_level(dqmc_batch* b, int mode, int measure, int j, int slot, const WalkerDev* W, int nw,
                                cudaStream_t st) {
  b->timed(DQMC_KCLASS_SEGMENT, [&] { general_chain_init(mode, W, nw, j, st); });
  for (int q = 0; q < b->maxPace_general; ++q) {
    b->timed(DQMC_KCLASS_PRODUCT, [&] {
      general_slice_pre(mode, W, nw, j, q, b->maxN_general, b->any_general_dense, b->any_general_cb, b->mixed, st);
    });
    b->timed(DQMC_KCLASS_METROPOLIS, [&] {
      general_slice_metro(mode, W, nw, j, q, b->maxN_general, measure, b->mixed, b->kd, b->smax, b->tc_flush, st);
    });
    b->timed(DQMC_KCLASS_PRODUCT, [&] {
      general_slice_post(mode, W, nw, j, q, b->maxN_general, b->any_general_dense, b->any_general_cb, b->mixed, st);
    });
  }
  b->timed(DQMC_KCLASS_PUSH, [&] {
    general_push(mode, W, nw, j, b->maxN_general, st);
    if (b->any_ozstab) oz_push(mode, W, nw, j, b->maxN_oz, st);
  });
  b->timed(DQMC_KCLASS_GREENS, [&] {
    general_greens(mode, W, nw, j, slot, b->maxN_general, st);
    if (b->any_ozstab) oz_greens(mode, W, nw, j, slot, b->maxN_oz, st);
  });
  if (measure) b->timed(DQMC_KCLASS_MEASURE, [&] { general_measure_after(mode, W, nw, j, b->maxN_general, st); });
}

static int trace_slot(const dqmc_batch* b, int j) {
  return (b->trace_cap && b->trace_count + j < b->trace_cap) ? b->trace_count + j : -1;
}

// All device work of one half-sweep, in stream order (captured into a graph).
// Profiled replays keep one branch (class events on one stream); otherwise the
// general walkers run as b->ngroups forked branches.
static void issue_half_sweep(dqmc_batch* b, int mode, int measure) {
  oz_set_shape(b->oz_shape);
  if (b->opt.rng == DQMC_RNG_MINSTD)
    cudaMemcpyAsync(b->d_uni, b->h_uni, sizeof(double) * b->uni_stride * b->nw, cudaMemcpyHostToDevice, b->stream);
  else
    launch_bump(b->d_sweep, b->stream);  // Philox counter: the half-sweep index
  const int ng = (b->any_general && !b->prof) ? std::min(b->ngroups, b->nw) : 1;
  if (ng > 1) {
    cudaEventRecord(b->ev_fork, b->stream);
    for (int g = 0; g < ng; ++g) {
      const int w0 = (int)((long long)b->nw * g / ng), w1 = (int)((long long)b->nw * (g + 1) / ng);
      cudaStreamWaitEvent(b->gst[g], b->ev_fork, 0);
      for (int j = 0; j < b->maxNs; ++j)
        issue_general_level(b, mode, measure, j, trace_slot(b, j), b->dW + w0, w1 - w0, b->gst[g]);
      cudaEventRecord(b->ev_join[g], b->gst[g]);
    }
  }
  for (int j = 0; j < b->maxNs; ++j) {
    const int slot = trace_slot(b, j);
    if (b->any_small) {
      b->timed(DQMC_KCLASS_SEGMENT,
               [&] { launch_segment(mode, b->dW, b->nw, j, measure, b->maxN_small, b->stream); });
      b->timed(DQMC_KCLASS_PUSH, [&] { launch_push(mode, b->dW, b->nw, j, b->maxN_small, b->stream); });
      b->timed(DQMC_KCLASS_GREENS,
               [&] { launch_greens(mode, b->dW, b->nw, j, 1, slot, b->maxN_small, b->stream); });
      if (measure)
        b->timed(DQMC_KCLASS_MEASURE, [&] { launch_measure(mode, b->dW, b->nw, j, b->maxN_small, b->stream); });
    }
    if (b->any_general && ng == 1) issue_general_level(b, mode, measure, j, slot, b->dW, b->nw, b->stream);
  }
  if (ng > 1)
    for (int g = 0; g < ng; ++g) cudaStreamWaitEvent(b->stream, b->ev_join[g], 0);
}

// owns a captured graph until the end of its scope, error returns included
struct GraphGuard {
  cudaGraph_t g = nullptr;
  ~GraphGuard() {
    if (g) cudaGraphDestroy(g);
  }
};

static int half_sweep(dqmc_batch* b, int mode, int measure) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  if (!b->initialised) return fail(DQMC_ERR_STATE, "sweep before dqmc_init_greens");
  if (b->opt.rng == DQMC_RNG_MINSTD) {
    // one uniform per site attempt in sweep order, drawn as bernoulli_distribution does
    for (int w = 0; w < b->nw; ++w) {
      const auto& d = b->desc[w];
      const size_t n = (size_t)d.Lt * desc_sites(d);
      double* u = b->h_uni + b->uni_stride * w;
      for (size_t k = 0; k < n; ++k) u[k] = std::generate_canonical<double, 53>(b->eng[w]);
    }
  }
  const int ms = measure ? 1 : 0;
  const bool use_graph = b->opt.graphs && !b->trace_cap;
  if (use_graph && b->prof) {
    // profiled replay: event nodes around each kernel class, read after the replay
    if (!b->pexec[mode][ms]) {
      GraphGuard g;
      const size_t m0 = b->marks.size();
      CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      b->capturing = true;
      issue_half_sweep(b, mode, measure);
      b->capturing = false;
      CUDA_TRY(cudaStreamEndCapture(b->stream, &g.g));
      b->pmarks[mode][ms].assign(b->marks.begin() + m0, b->marks.end());
      b->marks.resize(m0);
      CUDA_TRY(cudaGraphInstantiate(&b->pexec[mode][ms], g.g, 0));
    }
    CUDA_TRY(cudaGraphLaunch(b->pexec[mode][ms], b->stream));
    for (auto& m : b->pmarks[mode][ms]) {
      float t = 0;
      CUDA_TRY(cudaEventSynchronize(m.b));
      CUDA_TRY(cudaEventElapsedTime(&t, m.a, m.b));
      b->prof_ms[m.cls] += t;
      b->prof_n[m.cls] += 1;
    }
  }
  if (b->nodes[mode][ms] < 0 || (use_graph && !b->prof && !b->gexec[mode][ms])) {
    // capture the half-sweep: its kernel nodes give the launch count; replayed when graphs are on
    GraphGuard g;
    const bool prof = b->prof;
    b->prof = false;
    CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    issue_half_sweep(b, mode, measure);
    b->prof = prof;
    CUDA_TRY(cudaStreamEndCapture(b->stream, &g.g));
    size_t nn = 0;
    CUDA_TRY(cudaGraphGetNodes(g.g, nullptr, &nn));
    std::vector<cudaGraphNode_t> nodes(nn);
    CUDA_TRY(cudaGraphGetNodes(g.g, nodes.data(), &nn));
    int64_t k = 0;
    for (auto nd : nodes) {
      cudaGraphNodeType ty;
      cudaGraphNodeGetType(nd, &ty);
      if (ty == cudaGraphNodeTypeKernel) ++k;
    }
    b->nodes[mode][ms] = k;
    if (use_graph && !b->prof) CUDA_TRY(cudaGraphInstantiate(&b->gexec[mode][ms], g.g, 0));
  }
  if (use_graph && !b->prof) CUDA_TRY(cudaGraphLaunch(b->gexec[mode][ms], b->stream));
  else if (!use_graph) issue_half_sweep(b, mode, measure);
  b->launches += b->nodes[mode][ms];
  if (b->trace_cap) b->trace_count = std::min(b->trace_count + b->maxNs, b->trace_cap);
  if (b->opt.rng == DQMC_RNG_MINSTD) {
    // the pinned staging buffer is rewritten by the next half-sweep
    CUDA_TRY(cudaStreamSynchronize(b->stream));
  }
  return launch_check("half-sweep kernels");
}

int dqmc_set_wait_limit(dqmc_batch* b, int limit) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  for (auto& h : b->hw) h.wait_limit = (limit < 0) ? kDefaultWaitLimit : limit;
  CUDA_TRY(cudaMemcpyAsync(b->dW, b->hw.data(), sizeof(WalkerDev) * b->nw, cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}

int dqmc_tuning(dqmc_batch* b, int* kd, int* tc_flush, int* n_candidates, int* cand_kd, int* cand_tc,
                float* cand_ms) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  if (kd) *kd = b->kd;
  if (tc_flush) *tc_flush = b->tc_flush;
  if (n_candidates) *n_candidates = (int)b->tune_log.size();
  for (size_t k = 0; k < b->tune_log.size(); ++k) {
    if (cand_kd) cand_kd[k] = b->tune_log[k].first.first;
    if (cand_tc) cand_tc[k] = b->tune_log[k].first.second;
    if (cand_ms) cand_ms[k] = b->tune_log[k].second;
  }
  return DQMC_OK;
}

int dqmc_tuning_products(dqmc_batch* b, int* shape, int* n_candidates, int* cand_shape, float* cand_ms) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  if (shape) *shape = b->oz_shape;
  if (n_candidates) *n_candidates = (int)b->shape_log.size();
  for (size_t k = 0; k < b->shape_log.size(); ++k) {
    if (cand_shape) cand_shape[k] = b->shape_log[k].first;
    if (cand_ms) cand_ms[k] = b->shape_log[k].second;
  }
  return DQMC_OK;
}

int dqmc_launch_count(dqmc_batch* b, int64_t* launches) {
  if (!b || !launches) return fail(DQMC_ERR_ARG, "null argument");
  *launches = b->launches;
  return DQMC_OK;
}

int dqmc_sweep_0_to_beta(dqmc_batch* b, int measure) {
  const int r = half_sweep(b, MODE_FWD, measure);
  if (r == DQMC_OK) b->at_zero = false;
  return r;
}
int dqmc_sweep_beta_to_0(dqmc_batch* b, int measure) {
  const int r = half_sweep(b, MODE_BWD, measure);
  if (r == DQMC_OK) b->at_zero = true;
  return r;
}

// ---- dynamic half-sweep ------------------------------------------------------------
static constexpr int kMaxTau = 256;

static int dyn_alloc(dqmc_batch* b) {
  if (b->dyn_arena) return DQMC_OK;
  size_t cur = 0;
  auto take = [&](size_t bytes) { const size_t o = cur; cur = align256(cur + bytes); return o; };
  const size_t taus_off = take(sizeof(int) * kMaxTau);
  constexpr int kOff = 13;
  std::vector<size_t> off(b->nw * kOff);
  for (int w = 0; w < b->nw; ++w) {
    const WalkerDev& h = b->hw[w];
    const size_t NN = (size_t)h.N * h.N;
    off[kOff * w + 0] = take(sizeof(double) * 2 * h.S * NN);  // G(t,0)
    off[kOff * w + 1] = take(sizeof(double) * 2 * h.S * NN);  // G(0,t)
    off[kOff * w + 2] = take(sizeof(double) * h.S * NN);      // X1
    off[kOff * w + 3] = take(sizeof(int) * h.S * h.N);        // LU pivots
    off[kOff * w + 4] = take(sizeof(double) * kMaxTau);
    off[kOff * w + 5] = take(sizeof(long long) * kMaxTau);
    off[kOff * w + 6] = take(sizeof(double) * 3 * kMaxTau);           // DOS, chi, stiffness sums
    off[kOff * w + 7] = take(sizeof(double) * 2 * kMaxTau * h.N);     // parts awaiting G(beta,beta)
    off[kOff * w + 8] = take(sizeof(double) * 2 * kMaxTau);
    off[kOff * w + 9] = take(sizeof(double) * kMaxTau * h.N);        // per-displacement G sums
    if (h.path == 0) {  // HBM-path buffers of a shared-memory walker
      off[kOff * w + 10] = take(sizeof(double) * 2 * h.S * NN);  // chain (ping-pong)
      off[kOff * w + 11] = take(sizeof(double) * h.S * NN);      // work
      off[kOff * w + 12] = take(sizeof(double) * 2 * h.S * NN);  // scr
    }
  }
  cudaError_t e = cudaMalloc(&b->dyn_arena, cur);
  if (e != cudaSuccess) {
    b->dyn_arena = nullptr;
    return fail(DQMC_ERR_CUDA, "dynamic buffers (%zu bytes): %s", cur, cudaGetErrorString(e));
  }
  CUDA_TRY(cudaMemsetAsync(b->dyn_arena, 0, cur, b->stream));
  b->d_taus = reinterpret_cast<int*>(b->dyn_arena + taus_off);
  for (int w = 0; w < b->nw; ++w) {
    WalkerDev& h = b->hw[w];
    h.gt0 = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 0]);
    h.g0t = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 1]);
    h.dynx = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 2]);
    h.dpiv = reinterpret_cast<int*>(b->dyn_arena + off[kOff * w + 3]);
    h.dyn_sum = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 4]);
    h.dyn_cnt = reinterpret_cast<long long*>(b->dyn_arena + off[kOff * w + 5]);
    h.dyn_obs = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 6]);
    h.dyn_vec = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 7]);
    h.dyn_part = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 8]);
    h.dyn_r = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 9]);
    b->dyn_gen.resize(b->nw);
    if (h.path == 0) {
      b->dyn_gen[w].chain = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 10]);
      b->dyn_gen[w].work = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 11]);
      b->dyn_gen[w].scr = reinterpret_cast<double*>(b->dyn_arena + off[kOff * w + 12]);
    }
    h.dyn_taus = b->d_taus;
    h.dyn_ntau = 0;
  }
  CUDA_TRY(cudaMemcpyAsync(b->dW, b->hw.data(), sizeof(WalkerDev) * b->nw, cudaMemcpyHostToDevice, b->stream));
  return DQMC_OK;
}

int dqmc_clear_dynamic(dqmc_batch* b) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  if (!b->dyn_arena) return DQMC_OK;
  for (int w = 0; w < b->nw; ++w) {
    CUDA_TRY(cudaMemsetAsync(b->hw[w].dyn_sum, 0, sizeof(double) * kMaxTau, b->stream));
    CUDA_TRY(cudaMemsetAsync(b->hw[w].dyn_cnt, 0, sizeof(long long) * kMaxTau, b->stream));
    CUDA_TRY(cudaMemsetAsync(b->hw[w].dyn_obs, 0, sizeof(double) * 3 * kMaxTau, b->stream));
    CUDA_TRY(cudaMemsetAsync(b->hw[w].dyn_r, 0, sizeof(double) * kMaxTau * b->hw[w].N, b->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}

// The dynamic half-sweep's launch sequence: the walkers' largest N and pace, and which
// kinds of exp(-dtau K) occur
struct DynShape {
  int maxN, maxPace;
  bool any_dense, any_cb;
};

// Forward step j of the dynamic half-sweep for walkers W[0..nw) on stream st
static void issue_dynamic_level(dqmc_batch* b, const DynShape& ds, int j, const WalkerDev* W, int nw,
                                cudaStream_t st) {
  const int maxN = ds.maxN;
  b->timed(DQMC_KCLASS_SEGMENT, [&] { general_chain_init(MODE_FWD, W, nw, j, st); });
  for (int q = 0; q < ds.maxPace; ++q) {
    b->timed(DQMC_KCLASS_PRODUCT,
             [&] { general_dynamic_wrap(W, nw, j, q, maxN, b->mixed, ds.any_dense, ds.any_cb, st); });
    b->timed(DQMC_KCLASS_DYNAMIC,
             [&] { general_dynamic_prop(W, nw, j, q, maxN, b->mixed, ds.any_dense, ds.any_cb, st); });
    b->timed(DQMC_KCLASS_PRODUCT,
             [&] { general_dynamic_chain(W, nw, j, q, maxN, b->mixed, ds.any_dense, ds.any_cb, st); });
  }
  b->timed(DQMC_KCLASS_PUSH, [&] {
    general_push(MODE_FWD, W, nw, j, maxN, st);
    if (b->any_ozstab) oz_push(MODE_FWD, W, nw, j, b->maxN_oz, st);
  });
  b->timed(DQMC_KCLASS_GREENS, [&] { general_greens(MODE_FWD, W, nw, j, -1, maxN, st); });
  // the tensor-core walkers' equal-time assembly and their G(t,0), G(0,t) come from one
  // oz_greens (one factorization of M), timed in this class
  b->timed(DQMC_KCLASS_DYN_STAB, [&] {
    general_dynamic_stab(W, nw, j, maxN, st);
    if (b->any_ozstab) oz_greens(MODE_FWD, W, nw, j, -1, b->maxN_oz, st, true);
    general_dynamic_stab_measure(W, nw, j, st);
  });
}

// All device work of one dynamic half-sweep: as the updating half-sweeps, walker groups
// run as forked branches (one branch when profiling)
static void issue_dynamic(dqmc_batch* b, const DynShape& ds) {
  const int ng = b->prof ? 1 : std::min(b->ngroups, b->nw);
  b->timed(DQMC_KCLASS_DYNAMIC, [&] { general_dynamic_begin(b->dW, b->nw, b->stream); });
  if (ng > 1) {
    cudaEventRecord(b->ev_fork, b->stream);
    for (int g = 0; g < ng; ++g) {
      const int w0 = (int)((long long)b->nw * g / ng), w1 = (int)((long long)b->nw * (g + 1) / ng);
      cudaStreamWaitEvent(b->gst[g], b->ev_fork, 0);
      for (int j = 0; j < b->maxNs; ++j) issue_dynamic_level(b, ds, j, b->dW + w0, w1 - w0, b->gst[g]);
      cudaEventRecord(b->ev_join[g], b->gst[g]);
    }
    for (int g = 0; g < ng; ++g) cudaStreamWaitEvent(b->stream, b->ev_join[g], 0);
  } else {
    for (int j = 0; j < b->maxNs; ++j) issue_dynamic_level(b, ds, j, b->dW, b->nw, b->stream);
  }
  b->timed(DQMC_KCLASS_DYNAMIC, [&] { general_dynamic_end(b->dW, b->nw, ds.maxN, b->stream); });
}

int dqmc_sweep_dynamic(dqmc_batch* b, const int* taus, int ntau) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  if (!b->initialised) return fail(DQMC_ERR_STATE, "dynamic sweep before dqmc_init_greens");
  if (!b->at_zero)
    return fail(DQMC_ERR_STATE, "dynamic sweep needs the stacks of t = 0 (after set-up or a backward half-sweep)");
  if (ntau < 0 || ntau > kMaxTau || (ntau > 0 && !taus)) return fail(DQMC_ERR_ARG, "ntau must be in [0, 256]");
  for (int k = 0; k < ntau; ++k)
    for (int w = 0; w < b->nw; ++w)
      if (taus[k] < 0 || taus[k] >= b->desc[w].Lt)
        return fail(DQMC_ERR_ARG, "tau %d outside [0, Lt) of walker %d", taus[k], w);
  if (int r = dyn_alloc(b)) return r;
  const std::vector<int> tv(taus, taus + ntau);
  if (tv != b->taus) {  // a new tau list restarts the accumulators
    b->taus = tv;
    if (ntau) CUDA_TRY(cudaMemcpyAsync(b->d_taus, b->taus.data(), sizeof(int) * ntau, cudaMemcpyHostToDevice, b->stream));
    for (auto& h : b->hw) h.dyn_ntau = ntau;
    if (int r = dqmc_clear_dynamic(b)) return r;
  }
  // walkers of the tensor-core path with 128 <= N <= 768 stabilize with the blocked QR
  // (oz_push, oz_greens with the second right-hand side), the others with the FP64 kernels;
  // shared-memory walkers run this half-sweep on the HBM path's kernels with their own
  // buffers (the stacks, G and the fields are laid out alike on both paths)
  std::vector<WalkerDev> hv = b->hw;
  int maxN = 0, maxPace = 0;
  bool any_dense = false, any_cb = false;
  for (int w = 0; w < b->nw; ++w) {
    WalkerDev& h = hv[w];
    if (h.path == 0) {
      h.path = 1;
      h.chain = b->dyn_gen[w].chain;
      h.work = b->dyn_gen[w].work;
      h.scr = b->dyn_gen[w].scr;
    }
    maxN = std::max(maxN, h.N);
    maxPace = std::max(maxPace, h.pace);
    if (h.cb) any_cb = true; else any_dense = true;
  }
  CUDA_TRY(cudaMemcpyAsync(b->dW, hv.data(), sizeof(WalkerDev) * b->nw, cudaMemcpyHostToDevice, b->stream));
  oz_set_shape(b->oz_shape);
  const DynShape ds{maxN, maxPace, any_dense, any_cb};
  if (b->opt.graphs && !b->prof) {
    // captured once (the tau list and the per-walker descriptors are read on the device)
    if (!b->dyn_exec) {
      GraphGuard g;
      CUDA_TRY(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
      issue_dynamic(b, ds);
      CUDA_TRY(cudaStreamEndCapture(b->stream, &g.g));
      size_t nn = 0;
      CUDA_TRY(cudaGraphGetNodes(g.g, nullptr, &nn));
      std::vector<cudaGraphNode_t> nodes(nn);
      CUDA_TRY(cudaGraphGetNodes(g.g, nodes.data(), &nn));
      int64_t k = 0;
      for (auto nd : nodes) {
        cudaGraphNodeType ty;
        cudaGraphNodeGetType(nd, &ty);
        if (ty == cudaGraphNodeTypeKernel) ++k;
      }
      b->dyn_nodes = k;
      CUDA_TRY(cudaGraphInstantiate(&b->dyn_exec, g.g, 0));
    }
    CUDA_TRY(cudaGraphLaunch(b->dyn_exec, b->stream));
    b->launches += b->dyn_nodes;
  } else {
    issue_dynamic(b, ds);  // eager, one branch when profiling
  }
  CUDA_TRY(cudaMemcpyAsync(b->dW, b->hw.data(), sizeof(WalkerDev) * b->nw, cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (int r = launch_check("dynamic sweep")) return r;
  b->at_zero = false;
  return DQMC_OK;
}

int dqmc_get_dynamic(dqmc_batch* b, int w, double* sums, int64_t* counts) {
  if (int r = check_walker(b, w)) return r;
  if (!b->dyn_arena || b->taus.empty()) return DQMC_OK;
  const int n = (int)b->taus.size();
  std::vector<long long> c(n);
  if (sums) CUDA_TRY(cudaMemcpyAsync(sums, b->hw[w].dyn_sum, sizeof(double) * n, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaMemcpyAsync(c.data(), b->hw[w].dyn_cnt, sizeof(long long) * n, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (counts)
    for (int k = 0; k < n; ++k) counts[k] = c[k];
  return DQMC_OK;
}

int dqmc_get_dynamic_obs(dqmc_batch* b, int w, double* dos, double* chi, double* rho) {
  if (int r = check_walker(b, w)) return r;
  if (!b->dyn_arena || b->taus.empty()) return DQMC_OK;
  const int n = (int)b->taus.size();
  std::vector<double> v(3 * (size_t)n);
  CUDA_TRY(cudaMemcpyAsync(v.data(), b->hw[w].dyn_obs, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (int k = 0; k < n; ++k) {
    if (dos) dos[k] = v[3 * k + 0];
    if (chi) chi[k] = v[3 * k + 1];
    if (rho) rho[k] = v[3 * k + 2];
  }
  return DQMC_OK;
}

int dqmc_get_dynamic_r(dqmc_batch* b, int w, double* out) {
  if (int r = check_walker(b, w)) return r;
  if (!out) return fail(DQMC_ERR_ARG, "null output");
  if (!b->dyn_arena || b->taus.empty()) return DQMC_OK;
  const size_t n = b->taus.size() * (size_t)b->hw[w].N;
  CUDA_TRY(cudaMemcpyAsync(out, b->hw[w].dyn_r, sizeof(double) * n, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}

int dqmc_get_green_dynamic(dqmc_batch* b, int w, int which, int spin, double* out) {
  if (int r = check_walker(b, w)) return r;
  if (which < 0 || which > 1 || spin < 0 || spin > 1 || !out) return fail(DQMC_ERR_ARG, "bad which, spin or output");
  if (!b->dyn_arena) return fail(DQMC_ERR_STATE, "no dynamic half-sweep has run");
  const WalkerDev& h = b->hw[w];
  const size_t NN = (size_t)h.N * h.N;
  const int sp = spin < h.S ? spin : 0;
  const double* src = (which == 0 ? h.gt0 : h.g0t) + ((size_t)(h.Lt & 1) * h.S + sp) * NN;
  CUDA_TRY(cudaMemcpyAsync(out, src, sizeof(double) * NN, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}

int dqmc_get_green(dqmc_batch* b, int w, int spin, double* out) {
  if (int r = check_walker(b, w)) return r;
  if (spin < 0 || spin > 1 || !out) return fail(DQMC_ERR_ARG, "bad spin or null output");
  const int N = b->hw[w].N;
  CUDA_TRY(cudaMemcpyAsync(out, b->hw[w].G + (size_t)spin * N * N, sizeof(double) * N * N, cudaMemcpyDeviceToHost,
                           b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}

int dqmc_set_green(dqmc_batch* b, int w, int spin, const double* g) {
  if (int r = check_walker(b, w)) return r;
  if (spin < 0 || spin > 1 || !g) return fail(DQMC_ERR_ARG, "bad spin or null input");
  if (!b->initialised) return fail(DQMC_ERR_STATE, "dqmc_set_green before dqmc_init_greens");
  const int N = b->hw[w].N;
  CUDA_TRY(cudaMemcpyAsync(b->hw[w].G + (size_t)spin * N * N, g, sizeof(double) * N * N, cudaMemcpyHostToDevice,
                           b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}

static int read_scal_bytes(dqmc_batch* b, int w, const void* dptr, void* out, size_t bytes) {
  if (int r = check_walker(b, w)) return r;
  if (!out) return fail(DQMC_ERR_ARG, "null output");
  CUDA_TRY(cudaMemcpyAsync(out, dptr, bytes, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}
#define read_scal(b, w, dptr, out) read_scal_bytes(b, w, dptr, out, sizeof(*(out)))

int dqmc_get_config_sign(dqmc_batch* b, int w, double* out) {
  if (int r = check_walker(b, w)) return r;
  return read_scal(b, w, &b->d_scal[w].sign, out);
}
int dqmc_get_wrap_error(dqmc_batch* b, int w, double* out) {
  if (int r = check_walker(b, w)) return r;
  unsigned long long bits = 0;
  if (int r = read_scal(b, w, &b->d_scal[w].wrap_bits, &bits)) return r;
  std::memcpy(out, &bits, sizeof bits);
  return DQMC_OK;
}
int dqmc_get_accept_count(dqmc_batch* b, int w, int64_t* out) {
  if (int r = check_walker(b, w)) return r;
  long long v = 0;
  if (int r = read_scal(b, w, &b->d_scal[w].accepts, &v)) return r;
  *out = v;
  return DQMC_OK;
}
int dqmc_get_status(dqmc_batch* b, int w, int* out) {
  if (int r = check_walker(b, w)) return r;
  return read_scal(b, w, &b->d_scal[w].status, out);
}

int dqmc_get_observables(dqmc_batch* b, int w, double* sums, int64_t* counts) {
  if (int r = check_walker(b, w)) return r;
  if (!sums || !counts) return fail(DQMC_ERR_ARG, "null output");
  dqmc_batch::Scal s;
  CUDA_TRY(cudaMemcpyAsync(&s, &b->d_scal[w], sizeof s, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (int k = 0; k < kNumObs; ++k) {
    sums[k] = s.obs[k];
    counts[k] = s.obs_cnt[k];
  }
  return DQMC_OK;
}

int dqmc_get_observables_all(dqmc_batch* b, double* sums, int64_t* counts) {
  if (!b || !sums || !counts) return fail(DQMC_ERR_ARG, "null argument");
  std::vector<dqmc_batch::Scal> s(b->nw);
  CUDA_TRY(cudaMemcpyAsync(s.data(), b->d_scal, sizeof(dqmc_batch::Scal) * b->nw, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (int w = 0; w < b->nw; ++w)
    for (int k = 0; k < kNumObs; ++k) {
      sums[(size_t)w * kNumObs + k] = s[w].obs[k];
      counts[(size_t)w * kNumObs + k] = s[w].obs_cnt[k];
    }
  return DQMC_OK;
}

int dqmc_measure_bins(dqmc_batch* b, int nbins, int bin_size, int sweeps_between, double* out) {
  if (!b || !out) return fail(DQMC_ERR_ARG, "null argument");
  if (nbins <= 0 || bin_size < 2 || sweeps_between < 0) return fail(DQMC_ERR_ARG, "bad bin counts");
  if (!b->initialised) return fail(DQMC_ERR_STATE, "measurement before dqmc_init_greens");
  const size_t n = (size_t)b->nw * nbins * kNumObs;
  double* d_bins = nullptr;
  CUDA_TRY(cudaMalloc(&d_bins, sizeof(double) * n));
  int r = DQMC_OK;
  for (int w = 0; w < b->nw && r == DQMC_OK; ++w) {
    if (cudaMemsetAsync(b->d_scal[w].obs, 0, sizeof(double) * kNumObs, b->stream) != cudaSuccess ||
        cudaMemsetAsync(b->d_scal[w].obs_cnt, 0, sizeof(long long) * kNumObs, b->stream) != cudaSuccess)
      r = fail(DQMC_ERR_CUDA, "clearing the accumulators");
  }
  for (int bin = 0; bin < nbins && r == DQMC_OK; ++bin) {
    for (int s = 0; s < bin_size / 2 && r == DQMC_OK; ++s) {
      r = dqmc_sweep_0_to_beta(b, 1);
      if (r == DQMC_OK) r = dqmc_sweep_beta_to_0(b, 1);
    }
    if (r == DQMC_OK) launch_bin_close(b->dW, b->nw, d_bins, nbins, bin, b->stream);
    for (int s = 0; s < sweeps_between / 2 && r == DQMC_OK; ++s) {
      r = dqmc_sweep_0_to_beta(b, 0);
      if (r == DQMC_OK) r = dqmc_sweep_beta_to_0(b, 0);
    }
  }
  if (r == DQMC_OK) {
    if (cudaMemcpyAsync(out, d_bins, sizeof(double) * n, cudaMemcpyDeviceToHost, b->stream) != cudaSuccess ||
        cudaStreamSynchronize(b->stream) != cudaSuccess)
      r = fail(DQMC_ERR_CUDA, "reading the bins");
  } else {
    cudaStreamSynchronize(b->stream);
  }
  cudaFree(d_bins);
  return r;
}

int dqmc_clear_observables(dqmc_batch* b) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  for (int w = 0; w < b->nw; ++w) {
    CUDA_TRY(cudaMemsetAsync(b->d_scal[w].obs, 0, sizeof(double) * kNumObs, b->stream));
    CUDA_TRY(cudaMemsetAsync(b->d_scal[w].obs_cnt, 0, sizeof(long long) * kNumObs, b->stream));
  }
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}

int dqmc_trace_count(dqmc_batch* b, int* count) {
  if (!b || !count) return fail(DQMC_ERR_ARG, "null argument");
  *count = b->trace_count;
  return DQMC_OK;
}
int dqmc_trace_get(dqmc_batch* b, int w, int k, int spin, double* out) {
  if (int r = check_walker(b, w)) return r;
  if (!b->trace_cap) return fail(DQMC_ERR_STATE, "batch created without trace");
  if (k < 0 || k >= b->trace_count || spin < 0 || spin > 1 || !out) return fail(DQMC_ERR_ARG, "bad trace index");
  const int N = b->hw[w].N;
  CUDA_TRY(cudaMemcpyAsync(out, b->hw[w].trace + ((size_t)k * 2 + spin) * N * N, sizeof(double) * N * N,
                           cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return DQMC_OK;
}
int dqmc_trace_clear(dqmc_batch* b) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  b->trace_count = 0;
  return DQMC_OK;
}

int dqmc_profile_enable(dqmc_batch* b, int on) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  b->collect();
  b->prof = on != 0;
  for (int k = 0; k < DQMC_NUM_KCLASS; ++k) { b->prof_ms[k] = 0; b->prof_n[k] = 0; }
  return DQMC_OK;
}

int dqmc_profile_read(dqmc_batch* b, int cls, double* total_ms, int64_t* launches) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  if (cls < 0 || cls >= DQMC_NUM_KCLASS || !total_ms || !launches) return fail(DQMC_ERR_ARG, "bad kernel class");
  b->collect();
  *total_ms = b->prof_ms[cls];
  *launches = b->prof_n[cls];
  return DQMC_OK;
}

int dqmc_product_check(int n, const double* a, const double* b, double* c) {
  if (n < 1 || n > kMaxN || !a || !b || !c) return fail(DQMC_ERR_ARG, "dqmc_product_check: bad arguments");
  int nd = 0;
  if (cudaGetDeviceCount(&nd) != cudaSuccess || nd == 0) return fail(DQMC_ERR_CUDA, "no CUDA device available");
  const size_t nn = (size_t)n * n, ldk = (n + 15) / 16 * 16;
  // every piece 256-byte aligned (the product kernel copies slices in 16-byte chunks)
  const size_t o_b = align256(nn * sizeof(double)), o_c = o_b + align256(nn * sizeof(double));
  const size_t o_sa = o_c + align256(nn * sizeof(double));
  const size_t sl_bytes = align256(ozaki::kMaxSlices * (size_t)n * ldk * sizeof(unsigned short));
  const size_t o_sb = o_sa + sl_bytes, o_ea = o_sb + sl_bytes, o_eb = o_ea + align256(n * sizeof(int));
  const size_t bytes = o_eb + align256(n * sizeof(int));
  char* buf = nullptr;
  CUDA_TRY(cudaMalloc(&buf, bytes));
  double* dA = reinterpret_cast<double*>(buf);
  double* dB = reinterpret_cast<double*>(buf + o_b);
  double* dC = reinterpret_cast<double*>(buf + o_c);
  auto* sa = reinterpret_cast<unsigned short*>(buf + o_sa);
  auto* sb = reinterpret_cast<unsigned short*>(buf + o_sb);
  int* ea = reinterpret_cast<int*>(buf + o_ea);
  int* eb = reinterpret_cast<int*>(buf + o_eb);
  const char* step = "upload";
  cudaError_t e = cudaMemcpy(dA, a, nn * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(dB, b, nn * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) { step = "kernel set-up"; e = configure_ozaki_kernels(); }
  if (e == cudaSuccess) {
    step = "product launch";
    oz_selftest(dA, dB, dC, sa, ea, sb, eb, n, nullptr);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) { step = "download"; e = cudaMemcpy(c, dC, nn * sizeof(double), cudaMemcpyDeviceToHost); }
  cudaFree(buf);
  if (e != cudaSuccess) return fail(DQMC_ERR_CUDA, "dqmc_product_check (%s): %s", step, cudaGetErrorString(e));
  return DQMC_OK;
}

int dqmc_microbench_fp64(double* gflops) {
  if (!gflops) return fail(DQMC_ERR_ARG, "null output");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) return fail(DQMC_ERR_CUDA, "no CUDA device available");
  cudaError_t e = cudaSuccess;
  *gflops = run_fp64_probe(&e);
  if (e != cudaSuccess) return fail(DQMC_ERR_CUDA, "fp64 probe: %s", cudaGetErrorString(e));
  return DQMC_OK;
}

int dqmc_batch_info(dqmc_batch* b, int* nw, int64_t* upd) {
  if (!b) return fail(DQMC_ERR_ARG, "null batch");
  if (nw) *nw = b->nw;
  if (upd) {
    int64_t s = 0;
    for (auto& d : b->desc) s += (int64_t)desc_sites(d) * d.Lt;
    *upd = s;
  }
  return DQMC_OK;
}

}  // extern "C"
