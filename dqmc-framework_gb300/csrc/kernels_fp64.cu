// kernels_fp64.cu — FP64 plain-method kernels, SMEM-resident (N <= 64).
//
// One CTA owns one walker (segment, measurement, sign) or one (walker, spin)
// (stabilization).  GB300 executes FP64 at a small fraction of its FP32 rate,
// so these kernels are FP64-pipe bound: they keep G in shared memory for a
// whole stabilization segment, avoid redundant FP64 work (the reference's
// per-call MatrixV() re-product, the separate chain x U GEMM of the push) and
// use column-pivoted Householder QR instead of an SVD for the UDV stack.
//
// Reference behaviour restated here:
//   segment_kernel  src/dqmc_walker.cpp:246-325 / 334-412 (wrap, Metropolis,
//                   B-chain), src/dqmc_walker.cpp:173-197 (Metropolis),
//                   src/model/repulsive_hubbard.cpp:112-243 and
//                   src/model/attractive_hubbard.cpp:112-245 (ratio, update, B),
//                   src/checkerboard/square.cpp:66-226 (break-up order),
//                   src/measure/measure_methods.cpp:22-255 (fused measurement).
//   push_kernel     src/svd_stack.cpp:34-61 (stack push; QRP replaces dgesvd).
//   greens_kernel   include/utils/numerical_stable.hpp:34-239 (stable G, wrap error).
#include <cuda_runtime.h>
#include <cstdint>

#include "dqmc_device.cuh"

namespace dqmc {

// --------------------------------------------------------------------------
// small helpers
// --------------------------------------------------------------------------
__device__ __forceinline__ double& at(double* m, int ld, int r, int c) { return m[(long long)c * ld + r]; }
__device__ __forceinline__ double at(const double* m, int ld, int r, int c) { return m[(long long)c * ld + r]; }

__device__ __forceinline__ double warp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// Block reduction of NV values (all threads call); result valid in thread 0.
template <int NV>
__device__ void block_sum(double (&v)[NV], double* red /* >= NV*8 */) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    double s = warp_sum(v[k]);
    if (lane == 0) red[k * 8 + wid] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      double s = 0;
      for (int q = 0; q < kThreads / 32; ++q) s += red[k * 8 + q];
      v[k] = s;
    }
  }
  __syncthreads();
}

__device__ double block_max(double v, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  v = warp_max(v);
  if (lane == 0) red[wid] = v;
  __syncthreads();
  double m = 0;
  for (int q = 0; q < kThreads / 32; ++q) m = fmax(m, red[q]);
  __syncthreads();
  return m;
}

// spin factor of the B matrices: repulsive couples spin down with -1, attractive +1
__device__ __forceinline__ int spin_sign(const WalkerDev& w, int spin) {
  return (w.model == 0 && spin == 1) ? -1 : 1;
}
// exp(+/- alpha) for the product sgn * s
__device__ __forceinline__ double bdiag(const WalkerDev& w, int sgn_times_s) {
  return sgn_times_s > 0 ? w.e_pa : w.e_ma;
}

// --------------------------------------------------------------------------
// Checkerboard passes (src/checkerboard/square.cpp).  A layer of parity p
// mixes the 4 sites {(x,y),(x+1,y),(x,y+1),(x+1,y+1)} of every plaquette with
// corner (x,y), x = p, p+2, ..., y likewise.  Plaquettes of one layer are
// disjoint, so one pass updates the matrix in place.
//   left pass : rows r_a  <- sum_b P[a][b] rows r_b     (optionally pre/post-scaled)
//   right pass: cols c_b  <- sum_a cols c_a P[a][b]
// --------------------------------------------------------------------------
__device__ __forceinline__ void plaq_sites(int L, int q, int parity, int (&idx)[4]) {
  const int half = L >> 1;
  const int x = 2 * (q % half) + parity, y = 2 * (q / half) + parity;
  const int x1 = (x + 1) % L, y1 = (y + 1) % L;
  idx[0] = x + L * y;
  idx[1] = x1 + L * y;
  idx[2] = x + L * y1;
  idx[3] = x1 + L * y1;
}

// pre: scale inputs by d[row] (d from the scale table sd, null = none); post likewise on outputs
__device__ void cb_left(double* M, int ld, int N, int L, int parity, const double* P,
                        const double* pre, const double* post) {
  const int nq = (L >> 1) * (L >> 1);
  for (int it = threadIdx.x; it < nq * N; it += kThreads) {
    const int q = it % nq, c = it / nq;
    int idx[4];
    plaq_sites(L, q, parity, idx);
    double v[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      v[a] = at(M, ld, idx[a], c);
      if (pre) v[a] *= pre[idx[a]];
    }
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      double o = P[a * 4 + 0] * v[0];
      o = fma(P[a * 4 + 1], v[1], o);
      o = fma(P[a * 4 + 2], v[2], o);
      o = fma(P[a * 4 + 3], v[3], o);
      if (post) o *= post[idx[a]];
      at(M, ld, idx[a], c) = o;
    }
  }
}

__device__ void cb_right(double* M, int ld, int N, int L, int parity, const double* P,
                         const double* pre, const double* post) {
  const int nq = (L >> 1) * (L >> 1);
  for (int it = threadIdx.x; it < nq * N; it += kThreads) {
    const int r = it % N, q = it / N;
    int idx[4];
    plaq_sites(L, q, parity, idx);
    double v[4];
#pragma unroll
    for (int a = 0; a < 4; ++a) {
      v[a] = at(M, ld, r, idx[a]);
      if (pre) v[a] *= pre[idx[a]];
    }
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      double o = v[0] * P[0 * 4 + b];
      o = fma(v[1], P[1 * 4 + b], o);
      o = fma(v[2], P[2 * 4 + b], o);
      o = fma(v[3], P[3 * 4 + b], o);
      if (post) o *= post[idx[b]];
      at(M, ld, r, idx[b]) = o;
    }
  }
}

// --------------------------------------------------------------------------
// Register-tiled block GEMM for N <= 64: each of the 16x16 threads owns a
// T x T tile (rows ty+16a, cols tx+16b).  out(r,c) = sum_k A(r,k) B(k,c).
// The caller-supplied loaders/stores make it serve in-place products
// (SMEM or global: everyone reads before anyone writes).
// --------------------------------------------------------------------------
template <int T, class FA, class FB, class FS>
__device__ __forceinline__ void tile_gemm(int N, int kbeg, FA A, FB B, FS store) {
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  double acc[T][T];
#pragma unroll
  for (int a = 0; a < T; ++a)
#pragma unroll
    for (int b = 0; b < T; ++b) acc[a][b] = 0.0;
  for (int k = kbeg; k < N; ++k) {
    double av[T], bv[T];
#pragma unroll
    for (int a = 0; a < T; ++a) {
      const int r = ty + 16 * a;
      av[a] = (r < N) ? A(r, k) : 0.0;
    }
#pragma unroll
    for (int b = 0; b < T; ++b) {
      const int c = tx + 16 * b;
      bv[b] = (c < N) ? B(k, c) : 0.0;
    }
#pragma unroll
    for (int a = 0; a < T; ++a)
#pragma unroll
      for (int b = 0; b < T; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
  }
  __syncthreads();
#pragma unroll
  for (int a = 0; a < T; ++a)
#pragma unroll
    for (int b = 0; b < T; ++b) {
      const int r = ty + 16 * a, c = tx + 16 * b;
      if (r < N && c < N) store(r, c, acc[a][b]);
    }
  __syncthreads();
}

// dispatch on N to the smallest tile that covers it
template <class FA, class FB, class FS>
__device__ __forceinline__ void block_gemm(int N, FA A, FB B, FS store, int kbeg = 0) {
  if (N <= 16) tile_gemm<1>(N, kbeg, A, B, store);
  else if (N <= 32) tile_gemm<2>(N, kbeg, A, B, store);
  else if (N <= 48) tile_gemm<3>(N, kbeg, A, B, store);
  else tile_gemm<4>(N, kbeg, A, B, store);
}

// --------------------------------------------------------------------------
// B-matrix products on a matrix M (ld) for slice t (uses field row t-1).
// sd[i] holds the row/col scale of the current slice and spin.
// --------------------------------------------------------------------------
// M <- B(t) M = diag(e^{+sa s}) expK M   (mult_B_from_left)
__device__ void mult_B_left(const WalkerDev& w, double* M, int ld, const double* dpos) {
  const int N = w.N;
  if (w.cb) {
    cb_left(M, ld, N, w.L, 1, w.cbP, nullptr, nullptr);  // sublattice B first
    __syncthreads();
    cb_left(M, ld, N, w.L, 0, w.cbP, nullptr, dpos);     // then A, scale rows
    __syncthreads();
  } else {
    const double* K = w.expK;
    block_gemm(N, [&](int r, int k) { return __ldg(K + (long long)k * N + r); },
               [&](int k, int c) { return at(M, ld, k, c); },
               [&](int r, int c, double v) { at(M, ld, r, c) = v * dpos[r]; });
  }
}
// M <- M B(t)^-1 = M expK^-1 diag(e^{-sa s})   (mult_invB_from_right)
__device__ void mult_invB_right(const WalkerDev& w, double* M, int ld, const double* dneg) {
  const int N = w.N;
  if (w.cb) {
    cb_right(M, ld, N, w.L, 1, w.cbI, nullptr, nullptr);  // B then A
    __syncthreads();
    cb_right(M, ld, N, w.L, 0, w.cbI, nullptr, dneg);
    __syncthreads();
  } else {
    const double* K = w.invK;
    block_gemm(N, [&](int r, int k) { return at(M, ld, r, k); },
               [&](int k, int c) { return __ldg(K + (long long)c * N + k); },
               [&](int r, int c, double v) { at(M, ld, r, c) = v * dneg[c]; });
  }
}
// M <- M B(t) = M diag(e^{+sa s}) expK   (mult_B_from_right)
__device__ void mult_B_right(const WalkerDev& w, double* M, int ld, const double* dpos) {
  const int N = w.N;
  if (w.cb) {
    cb_right(M, ld, N, w.L, 0, w.cbP, dpos, nullptr);  // scale cols, A then B
    __syncthreads();
    cb_right(M, ld, N, w.L, 1, w.cbP, nullptr, nullptr);
    __syncthreads();
  } else {
    const double* K = w.expK;
    block_gemm(N, [&](int r, int k) { return at(M, ld, r, k) * dpos[k]; },
               [&](int k, int c) { return __ldg(K + (long long)c * N + k); },
               [&](int r, int c, double v) { at(M, ld, r, c) = v; });
  }
}
// M <- B(t)^-1 M = expK^-1 diag(e^{-sa s}) M   (mult_invB_from_left)
__device__ void mult_invB_left(const WalkerDev& w, double* M, int ld, const double* dneg) {
  const int N = w.N;
  if (w.cb) {
    cb_left(M, ld, N, w.L, 0, w.cbI, dneg, nullptr);  // scale rows, A then B
    __syncthreads();
    cb_left(M, ld, N, w.L, 1, w.cbI, nullptr, nullptr);
    __syncthreads();
  } else {
    const double* K = w.invK;
    block_gemm(N, [&](int r, int k) { return __ldg(K + (long long)k * N + r); },
               [&](int k, int c) { return at(M, ld, k, c) * dneg[k]; },
               [&](int r, int c, double v) { at(M, ld, r, c) = v; });
  }
}
// M <- B(t)^T M = expK^T diag(e^{+sa s}) M   (mult_transB_from_left)
__device__ void mult_transB_left(const WalkerDev& w, double* M, int ld, const double* dpos) {
  const int N = w.N;
  if (w.cb) {
    cb_left(M, ld, N, w.L, 0, w.cbP, dpos, nullptr);  // scale rows, A then B
    __syncthreads();
    cb_left(M, ld, N, w.L, 1, w.cbP, nullptr, nullptr);
    __syncthreads();
  } else {
    const double* K = w.expK;  // (expK^T)(r,k) = expK(k,r)
    block_gemm(N, [&](int r, int k) { return __ldg(K + (long long)r * N + k); },
               [&](int k, int c) { return at(M, ld, k, c) * dpos[k]; },
               [&](int r, int c, double v) { at(M, ld, r, c) = v; });
  }
}

// --------------------------------------------------------------------------
// Fused equal-time measurement of one slice (measure_methods.cpp:22-255).
// gu/gd in shared memory (ld), sg the recorded sign of the slice.
// --------------------------------------------------------------------------
__device__ void measure_slice(const WalkerDev& w, const double* gu, const double* gd, int ld, double sg,
                              double* scratch /* 2N */, double* red) {
  const int N = w.N, L = w.L, LL = L * L;
  double* du = scratch;
  double* dd = scratch + N;
  __shared__ signed char s_x[kMaxSmemN], s_y[kMaxSmemN], s_z[kMaxSmemN];
  for (int i = threadIdx.x; i < N; i += kThreads) {
    du[i] = 1.0 - at(gu, ld, i, i);
    dd[i] = 1.0 - at(gd, ld, i, i);
    s_x[i] = (signed char)(i % L);
    s_y[i] = (signed char)((i / L) % L);
    s_z[i] = (signed char)(i / LL);  // 0 on the square lattice
  }
  __syncthreads();
  // v: 0 trace, 1 double occ, 2 local spin, 3 kinetic, 4 n(k), 5 common, 6 cross, 7 s-wave
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < N; i += kThreads) {
    const double a = at(gu, ld, i, i), b = at(gd, ld, i, i);
    v[0] += a + b;
    v[1] += du[i] * dd[i];
    v[2] += a + b - 2 * a * b;
    // bonds to the +x, +y (, +z) neighbours (measure_methods.cpp:87-95)
    const int jx = site_nn(L, i, 0), jy = site_nn(L, i, 1);
    double kin = at(gu, ld, i, jx) + at(gd, ld, i, jx) + at(gu, ld, i, jy) + at(gd, ld, i, jy);
    if (w.dim == 3) {
      const int jz = site_nn(L, i, 2);
      kin += at(gu, ld, i, jz) + at(gd, ld, i, jz);
    }
    v[3] += kin;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = wid; j < N; j += kThreads / 32)
  for (int i = lane; i < N; i += 32) {
    int dx = s_x[j] - s_x[i], dy = s_y[j] - s_y[i], dz = s_z[j] - s_z[i];
    dx += (dx < 0) ? L : 0;
    dy += (dy < 0) ? L : 0;
    dz += (dz < 0) ? L : 0;
    const double ff = w.ff[dx + dy * L + dz * LL];
    const double gu_ij = at(gu, ld, i, j), gu_ji = at(gu, ld, j, i);
    const double gd_ij = at(gd, ld, i, j), gd_ji = at(gd, ld, j, i);
    const double dij = (i == j) ? 1.0 : 0.0;
    const double guc_ij = dij - gu_ji, gdc_ij = dij - gd_ji;
    v[4] += (gu_ji + gd_ji) * ff;
    v[5] += ff * (du[i] * du[j] + guc_ij * gu_ij + dd[i] * dd[j] + gdc_ij * gd_ij);
    v[6] += ff * (dd[i] * du[j] + du[i] * dd[j]);
    v[7] += guc_ij * gdc_ij;
  }
  block_sum<8>(v, red);
  if (threadIdx.x == 0) {
    const double n = (double)N;
    double* o = w.obs;
    o[0] += sg * (2.0 - v[0] / n);
    o[1] += sg * v[1] / n;
    o[2] += sg * (2.0 * w.hop_t) * v[3] / n;
    o[3] += sg * (1.0 - 0.5 * v[4] / n);
    o[4] += sg * v[2] / n;
    o[5] += sg * (v[5] - v[6]) / (n * n);
    o[6] += sg * (v[5] + v[6]) / (n * n);
    o[7] += sg * v[7] / n;
    o[8] += sg;
    for (int k = 0; k < kNumObs; ++k) w.obs_cnt[k] += 1;
  }
  __syncthreads();
}

// --------------------------------------------------------------------------
// Segment kernel: the slices of one stabilization interval for one walker.
//   MODE_FWD: for t up:   wrap into t, Metropolis(t), measure, chain <- B(t) chain
//   MODE_BWD: for t down: Metropolis(t), measure, chain <- B(t)^T chain, wrap out of t
//   MODE_INIT: chain <- B(t)^T chain only (initial_svd_stacks)
// The chain starts from U_top diag(D_top) of the stack being pushed (or I), so
// the push needs no separate (chain x U) product: B_p..B_1 (U D) = ((B_p..B_1) U) D
// column by column, the scale-separated order svd_stack.cpp:51 asks for.
// --------------------------------------------------------------------------
template <int MODE>
__global__ void __launch_bounds__(kThreads) segment_kernel(const WalkerDev* __restrict__ W, int j, int measure) {
  const WalkerDev& w = W[blockIdx.x];
  if (j >= w.nstack || w.path != 0) return;
  extern __shared__ double smem[];
  const int N = w.N, ld = N + 1, S = w.S, Lt = w.Lt, p = w.pace;
  double* Gs[2];
  Gs[0] = smem;
  Gs[1] = (S == 2) ? smem + (long long)N * ld : smem;
  double* vec = smem + (long long)S * N * ld;  // ucol[2][N], wrow[2][N]
  double* dtab = vec + 4 * N;                   // [2 spins][2 (pos,neg)][N]
  double* red = dtab + 4 * N;                   // 64
  double* scratch = red + 64;                   // 2N
  __shared__ int s_next;
  __shared__ double s_f[2];
  __shared__ int8_t s_field[kMaxSmemN];
  __shared__ double diag_pre[2 * kMaxSmemN];

  const int k = (MODE == MODE_FWD) ? j : (w.nstack - 1 - j);
  const int t_lo = k * p + 1, t_hi = min((k + 1) * p, Lt);
  const int side = (MODE == MODE_FWD) ? 0 : 1;

  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  constexpr int nwarp = kThreads / 32;
  // chain <- U_top diag(D_top)  or  I
  for (int sp = 0; sp < S; ++sp) {
    double* C = w.chain + (long long)sp * N * N;
    const double* lv = (j == 0) ? nullptr : stack_level(w, side, sp, j - 1);
    for (int c = wid; c < N; c += nwarp) {
      const double dc = lv ? lv[2LL * N * N + c] : 1.0;
      for (int r = lane; r < N; r += 32)
        C[(long long)c * N + r] = lv ? lv[(long long)c * N + r] * dc : ((r == c) ? 1.0 : 0.0);
    }
  }
  if (MODE != MODE_INIT) {
    for (int sp = 0; sp < S; ++sp) {
      const double* Gg = w.G + (long long)sp * N * N;
      for (int c = wid; c < N; c += nwarp)
        for (int r = lane; r < N; r += 32) at(Gs[sp], ld, r, c) = Gg[(long long)c * N + r];
    }
  }
  __syncthreads();

  double sign = *w.sign;
  long long acc_count = 0;
  const unsigned long long sweep = (w.rng == 1) ? *w.sweep_ctr : 0ULL;
  const int nsl = t_hi - t_lo + 1;
  for (int q = 0; q < nsl; ++q) {
    const int t = (MODE == MODE_FWD) ? t_lo + q : t_hi - q;
    const int eff = t - 1;  // 1 <= t <= Lt
    const int8_t* frow = w.fields + (long long)eff * N;
    for (int i = threadIdx.x; i < N; i += kThreads) s_field[i] = frow[i];
    __syncthreads();
    // scale tables for this slice: dtab[sp][0][i] = e^{+sa s_i}, dtab[sp][1][i] = e^{-sa s_i}
    for (int e = threadIdx.x; e < S * N; e += kThreads) {
      const int sp = e / N, i = e % N;
      const int ss = spin_sign(w, sp) * (int)s_field[i];
      dtab[(sp * 2 + 0) * N + i] = bdiag(w, ss);
      dtab[(sp * 2 + 1) * N + i] = bdiag(w, -ss);
    }
    __syncthreads();

    if (MODE == MODE_FWD) {  // wrap_from_0_to_beta(t-1): G <- B(t) G B(t)^-1
      for (int sp = 0; sp < S; ++sp) {
        mult_B_left(w, Gs[sp], ld, dtab + (sp * 2 + 0) * N);
        mult_invB_right(w, Gs[sp], ld, dtab + (sp * 2 + 1) * N);
      }
    }

    if (MODE != MODE_INIT) {
      // Metropolis over sites i = 0..N-1 (dqmc_walker.cpp:173-197).
      // Warp 0 decides; warps 1.. apply the rank-1 update of the last accepted
      // site meanwhile.  Sites rejected in between leave G unchanged, so the
      // decision thread scans ahead with the diagonal the pending update will
      // produce, computed with the same fma the update uses (bit-identical).
      auto decide_from = [&](int i0, bool pending) {
        // returns the next accepted site (or N); thread 0 only
        for (int i = i0; i < N; ++i) {
          const int s = s_field[i];
          const int si = s > 0 ? 0 : 1;
          double gu, gd;
          if (pending) {
            gu = fma(-vec[(2 + 0) * N + i], vec[0 * N + i], diag_pre[i]);
            gd = (S == 2) ? fma(-vec[(2 + 1) * N + i], vec[1 * N + i], diag_pre[N + i]) : gu;
          } else {
            gu = at(Gs[0], ld, i, i);
            gd = at(Gs[1], ld, i, i);
          }
          const FlipRatio q = flip_ratio(w, si, gu, gd);  // reference operation order
          const double r = q.r;
          const int attempt = (MODE == MODE_FWD) ? (eff * N + i) : ((Lt - t) * N + i);
          const double u = (w.rng == 0) ? w.uni[attempt]
                                        : philox_uniform(w.seed, (unsigned)w.widx, sweep, (unsigned)(eff * N + i));
          const double prob = fmin(1.0, fabs(r));
          if (!isfinite(r)) atomicOr(w.status, ST_NONFINITE_RATIO);
          if (u < prob) {
            flip_factors(w, q, s_f);
            s_field[i] = (int8_t)(-s);
            sign = (r >= 0) ? sign : -sign;
            ++acc_count;
            return i;
          }
        }
        return N;
      };
      if (threadIdx.x == 0) s_next = decide_from(0, false);
      __syncthreads();
      while (s_next < N) {
        const int i = s_next;
        // vectors of site i from the fully updated G, and the diagonal before its update
        if (threadIdx.x < N) {
          const int r = threadIdx.x;
          for (int sp = 0; sp < S; ++sp) {
            const double* g = Gs[sp];
            vec[sp * N + r] = s_f[sp] * at(g, ld, r, i);                       // f u
            vec[(2 + sp) * N + r] = ((r == i) ? 1.0 : 0.0) - at(g, ld, i, r);  // e_i - G(i,:)
            diag_pre[sp * N + r] = at(g, ld, r, r);
          }
        }
        __syncthreads();
        if (threadIdx.x < 32) {
          if (threadIdx.x == 0) s_next = decide_from(i + 1, true);
        } else {
          // warps 1..7: column c per warp, rows lane and lane+32 per lane
          const int lane = threadIdx.x & 31, uw = (threadIdx.x >> 5) - 1;
          const int r0 = lane, r1 = lane + 32;
          for (int sp = 0; sp < S; ++sp) {
            double* g = Gs[sp];
            const double* wv = vec + (2 + sp) * N;
            const double u0 = (r0 < N) ? vec[sp * N + r0] : 0.0;
            const double u1 = (r1 < N) ? vec[sp * N + r1] : 0.0;
            for (int c = uw; c < N; c += kThreads / 32 - 1) {
              const double wc = -wv[c];
              if (r0 < N) at(g, ld, r0, c) = fma(wc, u0, at(g, ld, r0, c));
              if (r1 < N) at(g, ld, r1, c) = fma(wc, u1, at(g, ld, r1, c));
            }
          }
        }
        __syncthreads();
      }
      // write back the flipped fields of this slice
      int8_t* frw = w.fields + (long long)eff * N;
      for (int i = threadIdx.x; i < N; i += kThreads) frw[i] = s_field[i];
      // the slice's B matrices below use the updated fields
      for (int e = threadIdx.x; e < S * N; e += kThreads) {
        const int sp = e / N, i = e % N;
        const int ss = spin_sign(w, sp) * (int)s_field[i];
        dtab[(sp * 2 + 0) * N + i] = bdiag(w, ss);
        dtab[(sp * 2 + 1) * N + i] = bdiag(w, -ss);
      }
      __syncthreads();

      // equal-time measurement of slot t-1 (the slot closing a forward
      // segment and slot Lt-1 of the backward sweep are measured after
      // their stabilization, dqmc_walker.cpp:307-310 and :408-411)
      if (measure) {
        const bool here = (MODE == MODE_FWD) ? (t != t_hi) : (t != Lt);
        if (here) measure_slice(w, Gs[0], Gs[1], ld, sign, scratch, red);
      }
      if (MODE == MODE_BWD && t == Lt && threadIdx.x == 0) *w.sign_Lt = sign;
    }

    // B-chain of the stabilization interval
    for (int sp = 0; sp < S; ++sp) {
      double* C = w.chain + (long long)sp * N * N;
      if (MODE == MODE_FWD) mult_B_left(w, C, N, dtab + (sp * 2 + 0) * N);
      else mult_transB_left(w, C, N, dtab + (sp * 2 + 0) * N);
    }

    if (MODE == MODE_BWD) {  // wrap_from_beta_to_0(t): G <- B(t)^-1 G B(t)
      for (int sp = 0; sp < S; ++sp) {
        mult_B_right(w, Gs[sp], ld, dtab + (sp * 2 + 0) * N);
        mult_invB_left(w, Gs[sp], ld, dtab + (sp * 2 + 1) * N);
      }
    }
    __syncthreads();
  }

  if (MODE != MODE_INIT) {
    for (int sp = 0; sp < S; ++sp) {
      double* Gg = w.G + (long long)sp * N * N;
      for (int c = wid; c < N; c += nwarp)
        for (int r = lane; r < N; r += 32) Gg[(long long)c * N + r] = at(Gs[sp], ld, r, c);
    }
    if (threadIdx.x == 0) {
      *w.sign = sign;
      *w.accepts += acc_count;
    }
  }
}

// --------------------------------------------------------------------------
// Stack push (svd_stack.cpp:34-61 with QRP for the SVD):
//   X = chain (= B_p..B_1 U_top D_top), X P = Q R,
//   U = Q, D = |diag R|, F_new = (D^-1 R P^T) F_prev.
// One CTA of kPushThreads per (walker, spin); thread j owns column j.  GB300
// issues an FP64 warp instruction every ~64 cycles per SM sub-partition, so
// the kernel avoids FP64 shuffle reductions in the O(N^3) parts: every dot
// product runs down one thread's own column.  Q is formed in place from the
// reflectors (LAPACK dorg2r order), so one N x N tile of SMEM suffices.
// --------------------------------------------------------------------------
constexpr int kPushThreads = 64;

// argmax of non-negative key over threads (ties -> lowest index); all threads get it
__device__ __forceinline__ int block64_argmax(double v, int idx, bool valid, int* s_i, long long* s_k) {
  long long key = valid ? __double_as_longlong(v) : -1LL;  // non-negative doubles order as integers
  int bi = idx;
  for (int o = 16; o > 0; o >>= 1) {
    const long long ok = __shfl_xor_sync(0xffffffffu, key, o);
    const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
    if (ok > key || (ok == key && oi < bi)) { key = ok; bi = oi; }
  }
  const int wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) { s_k[wid] = key; s_i[wid] = bi; }
  __syncthreads();
  int best = s_i[0];
  long long bk = s_k[0];
  for (int q = 1; q < kPushThreads / 32; ++q)
    if (s_k[q] > bk || (s_k[q] == bk && s_i[q] < best)) { bk = s_k[q]; best = s_i[q]; }
  __syncthreads();
  return best;
}

__device__ __forceinline__ double block64_sum(double v, double* s_d) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int wid = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) s_d[wid] = v;
  __syncthreads();
  double t = 0;
  for (int q = 0; q < kPushThreads / 32; ++q) t += s_d[q];
  __syncthreads();
  return t;
}

template <int MODE>
__global__ void __launch_bounds__(kPushThreads) push_kernel(const WalkerDev* __restrict__ W, int j) {
  const int wi = blockIdx.x >> 1, sp = blockIdx.x & 1;
  const WalkerDev& w = W[wi];
  if (j >= w.nstack || sp >= w.S || w.path != 0) return;
  extern __shared__ double smem[];
  const int N = w.N, ld = N + 1;
  const int side = (MODE == MODE_FWD) ? 0 : 1;
  double* X = smem;
  double* vn1 = X + (long long)N * ld;
  double* vn2 = vn1 + N;
  double* tau = vn2 + N;
  double* invd = tau + N;
  int* perm = (int*)(invd + N);
  __shared__ int s_i[kPushThreads / 32];
  __shared__ long long s_k[kPushThreads / 32];
  __shared__ double s_d[kPushThreads / 32];
  __shared__ double s_tau, s_scal, s_beta;
  const int tj = threadIdx.x;  // column / row owned by this thread
  const bool own = tj < N;

  const double* C = w.chain + (long long)sp * N * N;
  for (int c = 0; c < N; ++c)
    if (own) at(X, ld, tj, c) = C[(long long)c * N + tj];
  __syncthreads();
  if (own) {
    double s0 = 0, s1 = 0;
    int r = 0;
    for (; r + 1 < N; r += 2) {
      const double a = at(X, ld, r, tj), b = at(X, ld, r + 1, tj);
      s0 = fma(a, a, s0);
      s1 = fma(b, b, s1);
    }
    if (r < N) s0 = fma(at(X, ld, r, tj), at(X, ld, r, tj), s0);
    vn1[tj] = vn2[tj] = sqrt(s0 + s1);
    perm[tj] = tj;
  }
  __syncthreads();

  const double tol3z = 1.4901161193847656e-08;  // sqrt(eps), LAPACK dlaqp2
  for (int k = 0; k < N; ++k) {
    // ---- pivot: largest remaining column norm
    const int pv = block64_argmax(own ? vn1[tj] : 0.0, tj, own && tj >= k, s_i, s_k);
    if (pv != k) {
      if (own) {
        const double a = at(X, ld, tj, k);
        at(X, ld, tj, k) = at(X, ld, tj, pv);
        at(X, ld, tj, pv) = a;
      }
      if (tj == 0) {
        const int tp = perm[k]; perm[k] = perm[pv]; perm[pv] = tp;
        double tv = vn1[k]; vn1[k] = vn1[pv]; vn1[pv] = tv;
        tv = vn2[k]; vn2[k] = vn2[pv]; vn2[pv] = tv;
      }
      __syncthreads();
    }
    // ---- Householder reflector of X[k:,k]: row r > k held by thread r
    const double xr = (own && tj > k) ? at(X, ld, tj, k) : 0.0;
    const double xnorm2 = block64_sum(xr * xr, s_d);
    if (tj == 0) {
      const double alpha = at(X, ld, k, k);
      double t = 0.0, beta = alpha, scal = 1.0;
      if (xnorm2 != 0.0) {
        const double nrm = sqrt(alpha * alpha + xnorm2);
        beta = alpha >= 0 ? -nrm : nrm;
        t = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      s_tau = t; s_scal = scal; s_beta = beta;
      tau[k] = t;
    }
    __syncthreads();
    if (own && tj > k) at(X, ld, tj, k) *= s_scal;
    if (tj == 0) at(X, ld, k, k) = s_beta;
    __syncthreads();
    // ---- trailing update of column tj > k, then its norm downdate
    const double tk = s_tau;
    if (own && tj > k && tk != 0.0) {
      double a0 = at(X, ld, k, tj), a1 = 0.0;
      int r = k + 1;
      for (; r + 1 < N; r += 2) {
        a0 = fma(at(X, ld, r, k), at(X, ld, r, tj), a0);
        a1 = fma(at(X, ld, r + 1, k), at(X, ld, r + 1, tj), a1);
      }
      if (r < N) a0 = fma(at(X, ld, r, k), at(X, ld, r, tj), a0);
      const double wv = (a0 + a1) * tk;
      at(X, ld, k, tj) -= wv;
      for (r = k + 1; r < N; ++r) at(X, ld, r, tj) = fma(-wv, at(X, ld, r, k), at(X, ld, r, tj));
    }
    if (own && tj > k) {
      const double v1 = vn1[tj];
      if (v1 != 0.0) {
        double tmp = fabs(at(X, ld, k, tj)) / v1;
        tmp = fmax(0.0, 1.0 - tmp * tmp);
        const double r2 = v1 / vn2[tj];
        if (tmp * r2 * r2 <= tol3z) {
          double q0 = 0, q1 = 0;
          int r = k + 1;
          for (; r + 1 < N; r += 2) {
            q0 = fma(at(X, ld, r, tj), at(X, ld, r, tj), q0);
            q1 = fma(at(X, ld, r + 1, tj), at(X, ld, r + 1, tj), q1);
          }
          if (r < N) q0 = fma(at(X, ld, r, tj), at(X, ld, r, tj), q0);
          vn1[tj] = vn2[tj] = sqrt(q0 + q1);
        } else {
          vn1[tj] = v1 * sqrt(tmp);
        }
      }
    }
    __syncthreads();
  }

  // ---- D = |diag R| and the right factor F = (D^-1 R P^T) F_prev
  double* lv = stack_level(w, side, sp, j);
  double* Uo = lv;
  double* Fo = lv + (long long)N * N;
  double* Do = lv + 2LL * N * N;
  if (own) {
    const double d = fabs(at(X, ld, tj, tj));
    Do[tj] = d;
    invd[tj] = (d != 0.0) ? 1.0 / d : 0.0;
    if (d == 0.0 || !isfinite(d)) atomicOr(w.status, ST_SINGULAR);
  }
  __syncthreads();
  if (j == 0) {
    // F = T: column perm[c] of T holds R(:,c)/D for rows i <= c
    if (own) {
      const int c = tj;
      double* fc = Fo + (long long)perm[c] * N;
      for (int i = 0; i < N; ++i) fc[i] = (i <= c) ? at(X, ld, i, c) * invd[i] : 0.0;
    }
  } else if (own) {
    // thread c: F_new(i,c) = sum_{k>=i} (R(i,k)/D(i)) F_prev(perm[k], c)
    const int c = tj;
    const double* fp = stack_level(w, side, sp, j - 1) + (long long)N * N + (long long)c * N;
    double* fo = Fo + (long long)c * N;
    for (int i = 0; i < N; ++i) {
      double a0 = 0.0, a1 = 0.0;
      int k = i;
      for (; k + 1 < N; k += 2) {
        a0 = fma(at(X, ld, i, k), __ldg(fp + perm[k]), a0);
        a1 = fma(at(X, ld, i, k + 1), __ldg(fp + perm[k + 1]), a1);
      }
      if (k < N) a0 = fma(at(X, ld, i, k), __ldg(fp + perm[k]), a0);
      fo[i] = (a0 + a1) * invd[i];
    }
  }
  __syncthreads();

  // ---- Q = H_0 H_1 ... H_{N-1}, formed in place (dorg2r order)
  for (int i = N - 1; i >= 0; --i) {
    const double ti = tau[i];
    if (i < N - 1 && own && tj > i) {
      // apply H_i to column tj (rows i..N-1), v = [1; X(i+1:,i)]
      double a0 = at(X, ld, i, tj), a1 = 0.0;
      int r = i + 1;
      for (; r + 1 < N; r += 2) {
        a0 = fma(at(X, ld, r, i), at(X, ld, r, tj), a0);
        a1 = fma(at(X, ld, r + 1, i), at(X, ld, r + 1, tj), a1);
      }
      if (r < N) a0 = fma(at(X, ld, r, i), at(X, ld, r, tj), a0);
      const double wv = (a0 + a1) * ti;
      at(X, ld, i, tj) -= wv;
      for (r = i + 1; r < N; ++r) at(X, ld, r, tj) = fma(-wv, at(X, ld, r, i), at(X, ld, r, tj));
    }
    __syncthreads();
    if (own) {  // column i of Q: thread tj handles row tj
      const int r = tj;
      if (r > i) at(X, ld, r, i) *= -ti;
      else if (r == i) at(X, ld, r, i) = 1.0 - ti;
      else at(X, ld, r, i) = 0.0;
    }
    __syncthreads();
  }
  for (int c = 0; c < N; ++c)
    if (own) Uo[(long long)c * N + tj] = at(X, ld, tj, c);
}

// --------------------------------------------------------------------------
// In-SMEM LU with partial pivoting of M, applied on the fly to the right-hand
// sides Y (forward substitution fused), then back substitution: Y <- M^-1 Y.
// Returns false if a zero pivot was met.
// --------------------------------------------------------------------------
__device__ bool lu_solve_smem(double* M, double* Y, int N, int ld, double* red) {
  __shared__ int s_p;
  __shared__ int s_bad;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  if (threadIdx.x == 0) s_bad = 0;
  for (int k = 0; k < N; ++k) {
    if (wid == 0) {
      double best = -1.0;
      int bi = k;
      for (int r = k + lane; r < N; r += 32) {
        const double a = fabs(at(M, ld, r, k));
        if (a > best) { best = a; bi = r; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
      }
      if (lane == 0) { s_p = bi; if (best == 0.0) s_bad = 1; }
    }
    __syncthreads();
    const int pr = s_p;
    if (pr != k) {
      for (int c = threadIdx.x; c < 2 * N; c += kThreads) {
        double* m = (c < N) ? M : Y;
        const int cc = (c < N) ? c : c - N;
        const double tmp = at(m, ld, k, cc);
        at(m, ld, k, cc) = at(m, ld, pr, cc);
        at(m, ld, pr, cc) = tmp;
      }
      __syncthreads();
    }
    const double piv = at(M, ld, k, k);
    const double inv = (piv != 0.0) ? 1.0 / piv : 0.0;
    for (int r = k + 1 + threadIdx.x; r < N; r += kThreads) at(M, ld, r, k) *= inv;
    __syncthreads();
    const int nr = N - k - 1;
    // trailing update of M (cols k+1..N-1) and of Y (all cols)
    for (int e = threadIdx.x; e < nr * (nr + N); e += kThreads) {
      const int r = k + 1 + e % nr, cc = e / nr;
      const double l = at(M, ld, r, k);
      if (cc < nr) {
        const int c = k + 1 + cc;
        at(M, ld, r, c) = fma(-l, at(M, ld, k, c), at(M, ld, r, c));
      } else {
        const int c = cc - nr;
        at(Y, ld, r, c) = fma(-l, at(Y, ld, k, c), at(Y, ld, r, c));
      }
    }
    __syncthreads();
  }
  for (int k = N - 1; k >= 0; --k) {
    const double inv = 1.0 / at(M, ld, k, k);
    for (int c = threadIdx.x; c < N; c += kThreads) at(Y, ld, k, c) *= inv;
    __syncthreads();
    for (int e = threadIdx.x; e < k * N; e += kThreads) {
      const int r = e % k, c = e / k;
      at(Y, ld, r, c) = fma(-at(M, ld, r, k), at(Y, ld, k, c), at(Y, ld, r, c));
    }
    __syncthreads();
  }
  (void)red;
  return s_bad == 0;
}

// --------------------------------------------------------------------------
// Fresh equal-time G from the two stacks (numerical_stable.hpp:186-239):
//   general:  G = (U_R Drmax^-1) [ Dlmax^-1 U_L^T U_R Drmax^-1 + Dlmin F_L F_R^T Drmin ]^-1 (Dlmax^-1 U_L^T)
//   right empty (t = Lt): G = (Dmax^-1 U^T + Dmin F)^-1 Dmax^-1 U^T  of the left stack
//   left  empty (t = 0):  G = [same of the right stack]^T
// Also the wrap error max|G_fresh - G| (matrix_compare_error, :34-47) and the trace.
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) greens_kernel(const WalkerDev* __restrict__ W, int mode, int j,
                                                          int check_error, int trace_slot) {
  const int wi = blockIdx.x >> 1, sp = blockIdx.x & 1;
  const WalkerDev& w = W[wi];
  if (j >= w.nstack || sp >= w.S || w.path != 0) return;
  extern __shared__ double smem[];
  const int N = w.N, ld = N + 1, ns = w.nstack;
  double* Ms = smem;
  double* Ys = Ms + (long long)N * ld;
  double* dl_max = Ys + (long long)N * ld;
  double* dl_min = dl_max + N;
  double* dr_max = dl_min + N;
  double* dr_min = dr_max + N;
  double* red = dr_min + N;  // 64

  // the final stabilization of the backward sweep (t = 0) and the initial G
  // are not compared with a wrapped G (dqmc_walker.cpp:399-405, :137-147)
  if (mode == MODE_INIT || (mode == MODE_BWD && j == ns - 1)) check_error = 0;
  int nl, nr;  // stack lengths after this step's push/pop
  if (mode == MODE_FWD) { nl = j + 1; nr = ns - 1 - j; }
  else if (mode == MODE_BWD) { nl = ns - 1 - j; nr = j + 1; }
  else { nl = 0; nr = ns; }

  const double* UL = nullptr; const double* FL = nullptr; const double* DL = nullptr;
  const double* UR = nullptr; const double* FR = nullptr; const double* DR = nullptr;
  if (nl > 0) {
    const double* lv = stack_level(w, 0, sp, nl - 1);
    UL = lv; FL = lv + (long long)N * N; DL = lv + 2LL * N * N;
  }
  if (nr > 0) {
    const double* lv = stack_level(w, 1, sp, nr - 1);
    UR = lv; FR = lv + (long long)N * N; DR = lv + 2LL * N * N;
  }
  auto split = [&](const double* D, double* mx, double* mn) {
    for (int i = threadIdx.x; i < N; i += kThreads) {
      const double d = D[i];
      if (d >= 1.0) { mx[i] = d; mn[i] = 1.0; } else { mx[i] = 1.0; mn[i] = d; }
    }
  };
  bool transpose_out = false;
  if (nl > 0 && nr > 0) {
    split(DL, dl_max, dl_min);
    split(DR, dr_max, dr_min);
    __syncthreads();
    // M = Dlmax^-1 (U_L^T U_R) Drmax^-1 + Dlmin (F_L F_R^T) Drmin
    block_gemm(N, [&](int r, int k) { return __ldg(UL + (long long)r * N + k); },
               [&](int k, int c) { return __ldg(UR + (long long)c * N + k); },
               [&](int r, int c, double v) { at(Ms, ld, r, c) = v / (dl_max[r] * dr_max[c]); });
    block_gemm(N, [&](int r, int k) { return __ldg(FL + (long long)k * N + r); },
               [&](int k, int c) { return __ldg(FR + (long long)k * N + c); },
               [&](int r, int c, double v) { at(Ms, ld, r, c) += v * dl_min[r] * dr_min[c]; });
    for (int e = threadIdx.x; e < N * N; e += kThreads) {
      const int r = e % N, c = e / N;  // Y = Dlmax^-1 U_L^T
      at(Ys, ld, r, c) = UL[(long long)r * N + c] / dl_max[r];
    }
  } else {
    const double* U = (nl > 0) ? UL : UR;
    const double* F = (nl > 0) ? FL : FR;
    const double* D = (nl > 0) ? DL : DR;
    transpose_out = (nl == 0);
    split(D, dl_max, dl_min);
    __syncthreads();
    for (int e = threadIdx.x; e < N * N; e += kThreads) {
      const int r = e % N, c = e / N;
      const double y = U[(long long)r * N + c] / dl_max[r];
      at(Ys, ld, r, c) = y;
      at(Ms, ld, r, c) = y + dl_min[r] * F[(long long)c * N + r];
    }
  }
  __syncthreads();
  const bool ok = lu_solve_smem(Ms, Ys, N, ld, red);
  if (!ok && threadIdx.x == 0) atomicOr(w.status, ST_SINGULAR);

  double* G = w.G + (long long)sp * N * N;
  double* tr = (w.trace && trace_slot >= 0 && trace_slot < w.trace_cap)
                   ? w.trace + ((long long)trace_slot * 2 + sp) * N * N : nullptr;
  double err = 0.0;
  bool finite = true;
  if (nl > 0 && nr > 0) {
    for (int i = threadIdx.x; i < N; i += kThreads) dr_min[i] = 1.0 / dr_max[i];
    __syncthreads();
    // G = (U_R Drmax^-1) Y; the product is formed in registers, compared, stored
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    block_gemm(N, [&](int r, int k) { return __ldg(UR + (long long)k * N + r) * dr_min[k]; },
               [&](int k, int c) { return at(Ys, ld, k, c); },
               [&](int r, int c, double v) {
                 const long long o = (long long)c * N + r;
                 if (check_error) err = fmax(err, fabs(v - G[o]));
                 if (!isfinite(v)) finite = false;
                 G[o] = v;
                 if (tr) tr[o] = v;
               });
    (void)tx; (void)ty;
  } else {
    for (int e = threadIdx.x; e < N * N; e += kThreads) {
      const int r = e % N, c = e / N;
      const double v = transpose_out ? at(Ys, ld, c, r) : at(Ys, ld, r, c);
      if (check_error) err = fmax(err, fabs(v - G[e]));
      if (!isfinite(v)) finite = false;
      G[e] = v;
      if (tr) tr[e] = v;
    }
  }
  if (!finite) atomicOr(w.status, ST_NONFINITE_G);
  if (check_error) {
    const double m = block_max(err, red);
    if (threadIdx.x == 0) atomicMax(w.wrap_bits, (unsigned long long)__double_as_longlong(m));
  }
  // attractive: spin down mirrors spin up
  if (w.S == 1) {
    __syncthreads();
    double* Gd = w.G + (long long)N * N;
    for (int e = threadIdx.x; e < N * N; e += kThreads) Gd[e] = G[e];
    if (tr) {
      double* trd = tr + (long long)N * N;
      for (int e = threadIdx.x; e < N * N; e += kThreads) trd[e] = G[e];
    }
  }
}

// Measurement of a slot whose recorded G is the fresh one (after greens_kernel).
__global__ void __launch_bounds__(kThreads) measure_kernel(const WalkerDev* __restrict__ W, int mode, int j) {
  const WalkerDev& w = W[blockIdx.x];
  if (j >= w.nstack || w.path != 0) return;
  if (mode == MODE_BWD && j != w.nstack - 1) return;
  extern __shared__ double smem[];
  const int N = w.N, ld = N + 1;
  double* gu = smem;
  double* gd = (w.S == 2) ? smem + (long long)N * ld : smem;
  double* red = smem + 2LL * N * ld;
  double* scratch = red + 64;
  for (int sp = 0; sp < w.S; ++sp) {
    const double* Gg = w.G + (long long)sp * N * N;
    double* d = sp ? gd : gu;
    for (int e = threadIdx.x; e < N * N; e += kThreads) at(d, ld, e % N, e / N) = Gg[e];
  }
  __syncthreads();
  const double sg = (mode == MODE_BWD) ? *w.sign_Lt : *w.sign;
  measure_slice(w, gu, gd, ld, sg, scratch, red);
}

// sign(det G_up det G_dn) (dqmc_walker.cpp:150-163) via in-SMEM LU.
__global__ void __launch_bounds__(kThreads) sign_kernel(const WalkerDev* __restrict__ W) {
  const WalkerDev& w = W[blockIdx.x];
  if (w.path != 0) return;
  extern __shared__ double smem[];
  const int N = w.N, ld = N + 1;
  double* M = smem;
  __shared__ int s_neg;
  if (threadIdx.x == 0) s_neg = 0;
  int total_neg = 0;
  for (int sp = 0; sp < 2; ++sp) {
    const double* Gg = w.G + (long long)sp * N * N;
    for (int e = threadIdx.x; e < N * N; e += kThreads) at(M, ld, e % N, e / N) = Gg[e];
    __syncthreads();
    // LU with partial pivoting, counting swaps and negative pivots
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    __shared__ int s_p;
    for (int k = 0; k < N; ++k) {
      if (wid == 0) {
        double best = -1.0;
        int bi = k;
        for (int r = k + lane; r < N; r += 32) {
          const double a = fabs(at(M, ld, r, k));
          if (a > best) { best = a; bi = r; }
        }
        for (int o = 16; o > 0; o >>= 1) {
          const double ob = __shfl_xor_sync(0xffffffffu, best, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (lane == 0) s_p = bi;
      }
      __syncthreads();
      const int pr = s_p;
      if (pr != k) {
        for (int c = threadIdx.x; c < N; c += kThreads) {
          const double tmp = at(M, ld, k, c);
          at(M, ld, k, c) = at(M, ld, pr, c);
          at(M, ld, pr, c) = tmp;
        }
        if (threadIdx.x == 0) ++s_neg;
      }
      __syncthreads();
      const double piv = at(M, ld, k, k);
      if (threadIdx.x == 0 && piv < 0) ++s_neg;
      const double inv = (piv != 0.0) ? 1.0 / piv : 0.0;
      for (int r = k + 1 + threadIdx.x; r < N; r += kThreads) at(M, ld, r, k) *= inv;
      __syncthreads();
      const int nr = N - k - 1;
      for (int e = threadIdx.x; e < nr * nr; e += kThreads) {
        const int r = k + 1 + e % nr, c = k + 1 + e / nr;
        at(M, ld, r, c) = fma(-at(M, ld, r, k), at(M, ld, k, c), at(M, ld, r, c));
      }
      __syncthreads();
    }
    total_neg = s_neg;
  }
  if (threadIdx.x == 0) *w.sign = (total_neg % 2 == 0) ? 1.0 : -1.0;
}

// half-sweep counter of the Philox stream (a kernel, so a captured graph advances it)
__global__ void bump_counter_kernel(unsigned long long* ctr) { *ctr += 1ULL; }
void launch_bump(unsigned long long* ctr, cudaStream_t st) { bump_counter_kernel<<<1, 1, 0, st>>>(ctr); }

// MeasureHandler::normalize_stats + write_stats_to_bins + clear_temporary
// (src/measure/measure_handler.cpp:170-277) for every walker on the device:
// bin = sum / (count <sign>), the sign bin |<sign>|, accumulators cleared.
// bins: [walker][nbins][kNumObs].
__global__ void bin_close_kernel(const WalkerDev* __restrict__ W, int nw, double* bins, int nbins, int bin) {
  const int w = blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= nw) return;
  const WalkerDev& h = W[w];
  const double sign = h.obs[kNumObs - 1] / (double)h.obs_cnt[kNumObs - 1];
  double* out = bins + ((long long)w * nbins + bin) * kNumObs;
  for (int k = 0; k < kNumObs - 1; ++k) out[k] = h.obs[k] / ((double)h.obs_cnt[k] * sign);
  out[kNumObs - 1] = fabs(sign);
  for (int k = 0; k < kNumObs; ++k) {
    h.obs[k] = 0.0;
    h.obs_cnt[k] = 0;
  }
}
void launch_bin_close(const WalkerDev* W, int nw, double* bins, int nbins, int bin, cudaStream_t st) {
  bin_close_kernel<<<(nw + 127) / 128, 128, 0, st>>>(W, nw, bins, nbins, bin);
}

// --------------------------------------------------------------------------
// FP64 FMA throughput probe: 8 independent register FMA chains per thread.
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads) fp64_fma_probe(double* out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-3 + k;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 12345.678) out[blockIdx.x] = s;  // keeps the chains live
}

double run_fp64_probe(cudaError_t* err) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  double* d = nullptr;
  *err = cudaMalloc(&d, sizeof(double) * sms * 8);
  if (*err) return 0;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int iters = 4096, blocks = sms * 8;
  fp64_fma_probe<<<blocks, kThreads>>>(d, iters, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0);
  fp64_fma_probe<<<blocks, kThreads>>>(d, iters, 0.999999, 1e-7);
  cudaEventRecord(e1);
  *err = cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(d);
  if (*err == cudaSuccess) *err = cudaGetLastError();
  return 2.0 * 8.0 * iters * (double)blocks * kThreads / (ms * 1e-3) / 1e9;
}

// --------------------------------------------------------------------------
// host-side launch helpers
// --------------------------------------------------------------------------
size_t segment_smem_bytes(int N, int S) { return sizeof(double) * ((size_t)S * N * (N + 1) + 8 * N + 64 + 2 * N); }
size_t push_smem_bytes(int N) { return sizeof(double) * ((size_t)N * (N + 1) + 4 * N) + sizeof(int) * N; }
size_t greens_smem_bytes(int N) { return sizeof(double) * (2 * (size_t)N * (N + 1) + 4 * N + 64); }
size_t measure_smem_bytes(int N) { return sizeof(double) * (2 * (size_t)N * (N + 1) + 64 + 2 * N); }

cudaError_t configure_fp64_kernels(int maxN) {
  const size_t s1 = segment_smem_bytes(maxN, 2), s2 = push_smem_bytes(maxN), s3 = greens_smem_bytes(maxN),
               s4 = measure_smem_bytes(maxN);
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(segment_kernel<MODE_INIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1))) return e;
  if ((e = cudaFuncSetAttribute(segment_kernel<MODE_FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1))) return e;
  if ((e = cudaFuncSetAttribute(segment_kernel<MODE_BWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1))) return e;
  if ((e = cudaFuncSetAttribute(push_kernel<MODE_INIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2))) return e;
  if ((e = cudaFuncSetAttribute(push_kernel<MODE_FWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2))) return e;
  if ((e = cudaFuncSetAttribute(push_kernel<MODE_BWD>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2))) return e;
  if ((e = cudaFuncSetAttribute(greens_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s3))) return e;
  if ((e = cudaFuncSetAttribute(measure_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s4))) return e;
  if ((e = cudaFuncSetAttribute(sign_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s3))) return e;
  return cudaSuccess;
}

void launch_segment(int mode, const WalkerDev* W, int nw, int j, int measure, int maxN, cudaStream_t st) {
  const size_t sm = segment_smem_bytes(maxN, 2);
  if (mode == MODE_INIT) segment_kernel<MODE_INIT><<<nw, kThreads, sm, st>>>(W, j, 0);
  else if (mode == MODE_FWD) segment_kernel<MODE_FWD><<<nw, kThreads, sm, st>>>(W, j, measure);
  else segment_kernel<MODE_BWD><<<nw, kThreads, sm, st>>>(W, j, measure);
}
void launch_push(int mode, const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st) {
  const size_t sm = push_smem_bytes(maxN);
  if (mode == MODE_INIT) push_kernel<MODE_INIT><<<2 * nw, kPushThreads, sm, st>>>(W, j);
  else if (mode == MODE_FWD) push_kernel<MODE_FWD><<<2 * nw, kPushThreads, sm, st>>>(W, j);
  else push_kernel<MODE_BWD><<<2 * nw, kPushThreads, sm, st>>>(W, j);
}
void launch_greens(int mode, const WalkerDev* W, int nw, int j, int check, int trace_slot, int maxN, cudaStream_t st) {
  greens_kernel<<<2 * nw, kThreads, greens_smem_bytes(maxN), st>>>(W, mode, j, check, trace_slot);
}
void launch_measure(int mode, const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st) {
  measure_kernel<<<nw, kThreads, measure_smem_bytes(maxN), st>>>(W, mode, j);
}
void launch_sign(const WalkerDev* W, int nw, int maxN, cudaStream_t st) {
  sign_kernel<<<nw, kThreads, greens_smem_bytes(maxN), st>>>(W);
}

}  // namespace dqmc
