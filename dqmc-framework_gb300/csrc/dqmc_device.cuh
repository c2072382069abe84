// dqmc_device.cuh — device data model of a walker batch (FP64 plain method).
//
// One WalkerDev per walker, in device memory.  Everything a CTA needs to run
// one walker's segment or stabilization is reachable from it: the Green's
// functions, the B-chain buffer, the UDT stacks, the Ising fields, the dense
// exp(+/-dtau K) (shared by walkers with equal lattice parameters), the
// Fourier table of the measured momentum and the per-walker accumulators.
//
// Layouts (all column-major, leading dimension N, 256-byte aligned bases):
//   G      [2][N*N]      spin 0 = up, spin 1 = down (attractive: spin 1 aliases 0)
//   chain  [S][N*N]      running B-chain product of the current segment
//   stack  [side][S][level] { U (N*N) | F (N*N) | D (N) }, side 0 left, 1 right
//   fields [Lt][N] int8  +/-1, slice-major (reference: Lt x N Eigen matrix of doubles)
#pragma once
#include <cstdint>

namespace dqmc {

constexpr int kThreads = 256;
constexpr int kMaxSmemN = 64;    // N handled by the SMEM-resident kernels
constexpr int kMaxN = 1024;      // largest N of the general (HBM-resident) kernels
constexpr int kNumObs = 9;

enum SweepMode { MODE_INIT = 0, MODE_FWD = 1, MODE_BWD = 2 };

// status bits (per walker)
enum : int {
  ST_NONFINITE_G = 1,
  ST_SINGULAR = 2,
  ST_NONFINITE_RATIO = 4,
  ST_TIMEOUT = 8,  // a bounded device-side wait gave up (the kernel skipped its output)
};

struct WalkerDev {
  int N, L, Lt, pace, nstack, S, model, cb;  // model: 0 repulsive, 1 attractive
  int dim;                                    // 2 square (N = L^2), 3 cubic (N = L^3)
  int rng;                                    // 0 host uniforms, 1 Philox
  int path;                                   // 0 SMEM FP64, 1 HBM FP64, 2 HBM mixed (tensor-core products)
  double hop_t;
  // B-matrix diagonal factors exp(+alpha), exp(-alpha)
  double e_pa, e_ma;
  // ratio constants indexed by [s>0 ? 0 : 1]: exp(-2 alpha s) - 1, exp(+2 alpha s) - 1, exp(2 alpha s)
  double cm[2], cp[2], ex2[2];
  double cbP[16], cbI[16];   // checkerboard plaquettes exp(+dtau t h) e^{0.5 dtau mu}, inverse
  double* G;                 // [2][N*N]
  double* chain;             // [S][N*N] (general walkers: [2][S][N*N], ping-pong)
  double* work;              // general walkers: GEMM temporary [S][N*N]
  double* scr;               // general walkers: stabilization scratch [S][2][N*N]
  // mixed walkers, submatrix Metropolis: per spin T [N][32] FP64, then the BF16
  // slices of T and of G0(:, accepted sites) [2][6][N][40] and their exponents [2][N]
  unsigned char* msub;
  // time-displaced Green's functions (dynamic half-sweep), allocated on first use:
  // G(t,0) and G(0,t) ping-pong [2][S][N*N], second right-hand side [S][N*N],
  // LU pivots [S][N], G(k,tau) accumulators [dyn_ntau]
  double* gt0;
  double* g0t;
  double* dynx;
  int* dpiv;
  double* dyn_sum;
  long long* dyn_cnt;
  const int* dyn_taus;
  int dyn_ntau;
  // dynamic observables: sums [tau][3] (density of states, spin susceptibility, stiffness),
  // per-half-sweep parts awaiting G(beta,beta): vectors [tau][2][N] and scalars [tau][2]
  double* dyn_obs;
  double* dyn_vec;
  double* dyn_part;
  double* dyn_r;  // [tau][N] sign * 0.5 sum_i (G_up + G_dn)(i + r, i) / N: G(k,tau) of any k
  int zld;                   // line stride of zsl (N rounded up to 32)
  // tensor-core stabilization: BF16 slices of both operands of the current product,
  // [S][2 operands][9 slices][N][zld]
  unsigned short* zsl;
  // mixed walkers: BF16 slices of the operand being multiplied, [S][slices][N][ldk]
  unsigned short* sl;
  int* sle;                  // slice exponents [S][N]
  int ldk;                   // padded slice row length (multiple of 16)
  int slice_bits, slices;
  // constant slices of exp(-dtau K) and exp(+dtau K) as left (A) and right (B) operands
  const unsigned short* kA; const unsigned short* kB; const unsigned short* iA; const unsigned short* iB;
  const int* kAe; const int* kBe; const int* iAe; const int* iBe;
  double* stack;             // see header
  long long lvl_stride;      // doubles per stack level (2 N^2 + N, padded)
  long long side_stride;     // doubles per side (S * nstack * lvl_stride)
  int8_t* fields;            // [Lt][N]
  const double* expK;        // dense exp(-dtau K)  (N*N) or null
  const double* invK;        // dense exp(+dtau K)
  const double* ff;          // Fourier factor per displacement index, measured k
  double* obs;               // [kNumObs] sums of sign * O
  long long* obs_cnt;        // [kNumObs]
  double* sign;              // current configuration sign
  double* sign_Lt;           // sign recorded at t = Lt of the backward half-sweep
  unsigned long long* wrap_bits;  // running max |G_fresh - G_wrapped| (bit pattern)
  long long* accepts;
  int* status;
  const double* uni;         // parity uniforms of the current half-sweep [Lt*N]
  unsigned long long seed;   // Philox key
  const unsigned long long* sweep_ctr;  // Philox counter word: the batch's half-sweep index (device)
  double* trace;             // [trace_cap][2][N*N] or null
  int trace_cap;
  int ozstab;                // 1: stabilization by the tensor-core blocked QR (kernels_stab_oz.cu)
  int widx;                  // index of the walker in its batch (Philox counter word)
  // iteration limit of the wraps' and B-chain products' waits for their operands to land
  // (oz_prod_tc_kernel); kDefaultWaitLimit unless a test lowers it (dqmc_set_wait_limit)
  int wait_limit;
};

constexpr int kDefaultWaitLimit = 1 << 24;

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11): uniform double in [0,1)
// keyed by the walker's seed, counter (site attempt, half-sweep, walker).
__device__ __forceinline__ double philox_uniform(unsigned long long seed, unsigned walker, unsigned long long sweep,
                                                 unsigned attempt) {
  unsigned c0 = attempt, c1 = (unsigned)sweep, c2 = (unsigned)(sweep >> 32), c3 = walker;
  unsigned k0 = (unsigned)seed, k1 = (unsigned)(seed >> 32);
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned hi0 = __umulhi(0xD2511F53u, c0), lo0 = 0xD2511F53u * c0;
    const unsigned hi1 = __umulhi(0xCD9E8D57u, c2), lo1 = 0xCD9E8D57u * c2;
    const unsigned n0 = hi1 ^ c1 ^ k0, n2 = hi0 ^ c3 ^ k1;
    c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  const unsigned long long m = ((unsigned long long)(c0 >> 5) << 26) | (unsigned long long)(c1 >> 6);
  return (double)m * (1.0 / 9007199254740992.0);
}

// Metropolis ratio of flipping the field s of a site whose equal-time diagonals are
// gu = G_up(i,i), gd = G_dn(i,i) (si = 0 for s = +1, 1 for s = -1):
//   repulsive   r = (1 + (1 - gu)(e^{-2as} - 1)) (1 + (1 - gd)(e^{+2as} - 1))
//   attractive  r = e^{2as} (1 + (1 - gu)(e^{-2as} - 1)) (1 + (1 - gd)(e^{-2as} - 1))
// (get_update_ratio, src/model/repulsive_hubbard.cpp:112-124 and
// src/model/attractive_hubbard.cpp:112-125), each operation rounded on its own in the
// reference's order, never contracted into an FMA, so equal diagonals give bit-equal
// ratios and decisions on every path.  Every Metropolis kernel evaluates it here.
struct FlipRatio {
  double r;       // the ratio
  double ru, rd;  // its spin factors 1 + (1 - G_ii) Delta
  double cu, cd;  // Delta_up, Delta_dn (e^{-+2as} - 1)
};

__device__ __forceinline__ FlipRatio flip_ratio(const WalkerDev& w, int si, double gu, double gd) {
  FlipRatio q;
  q.cu = w.cm[si];
  q.cd = (w.model == 0) ? w.cp[si] : w.cm[si];
  q.ru = __dadd_rn(1.0, __dmul_rn(__dsub_rn(1.0, gu), q.cu));
  q.rd = __dadd_rn(1.0, __dmul_rn(__dsub_rn(1.0, gd), q.cd));
  q.r = (w.model == 0) ? __dmul_rn(q.ru, q.rd) : __dmul_rn(__dmul_rn(w.ex2[si], q.ru), q.rd);
  return q;
}

// The factors f_sigma = Delta_sigma / (1 + (1 - G_ii) Delta_sigma) of the accepted flip's
// rank-1 update (update_greens_function, src/model/repulsive_hubbard.cpp:127-155; the
// attractive model's factor_dn equals factor_up, src/model/attractive_hubbard.cpp:149).
__device__ __forceinline__ void flip_factors(const WalkerDev& w, const FlipRatio& q, double* f) {
  f[0] = __ddiv_rn(q.cu, q.ru);
  f[1] = (w.model == 0) ? __ddiv_rn(q.cd, q.rd) : f[0];
}

// Site i of a walker's lattice is x + L y (+ L^2 z).  The displacement from site i to site j
// as the site index of its vector, each component mod L (src/lattice/square.cpp:88-105,
// src/lattice/cubic.cpp:112-132), and the neighbour of site i in direction +x, +y or +z.
__device__ __forceinline__ int site_disp(int L, int dim, int i, int j) {
  if (dim == 2) {
    int dx = j % L - i % L, dy = j / L - i / L;
    dx += (dx < 0) ? L : 0;
    dy += (dy < 0) ? L : 0;
    return dx + dy * L;
  }
  const int LL = L * L;
  int dx = j % L - i % L, dy = (j / L) % L - (i / L) % L, dz = j / LL - i / LL;
  dx += (dx < 0) ? L : 0;
  dy += (dy < 0) ? L : 0;
  dz += (dz < 0) ? L : 0;
  return dx + dy * L + dz * LL;
}
__device__ __forceinline__ int site_nn(int L, int i, int a) {
  const int w = (a == 0) ? 1 : (a == 1) ? L : L * L;
  const int c = (i / w) % L;
  return i + ((c + 1) % L - c) * w;
}
// the site at displacement r from site i
__device__ __forceinline__ int site_shift(int L, int dim, int i, int r) {
  int j = 0;
  for (int a = 0, w = 1; a < dim; ++a, w *= L) j += (((i / w) % L + (r / w) % L) % L) * w;
  return j;
}

__host__ __device__ inline double* stack_level(const WalkerDev& w, int side, int spin, int level) {
  return w.stack + side * w.side_stride + ((long long)spin * w.nstack + level) * w.lvl_stride;
}

}  // namespace dqmc
