// kernels_general.cu — FP64 plain-method kernels for walkers whose G does not
// fit in shared memory (N > 64, up to 1024).
//
// G, the B-chain and the stacks stay in HBM/L2; a half-sweep runs slice by
// slice as a short sequence of batched launches:
//   wrap (two batched GEMMs with the diagonal exp(+/-alpha s) fused, or
//   checkerboard passes) -> Metropolis (one CTA per walker, rank-1 updates,
//   look-ahead decisions) -> measurement -> B-chain step (GEMM, ping-pong).
// Stabilization: column-pivoted QR with one thread per column (row-major copy,
// coalesced across threads), Green's assembly by batched GEMMs and an LU solve
// with one thread per column of [M | Y].
//
// Reference behaviour is the same as kernels_fp64.cu (src/dqmc_walker.cpp,
// src/model/*.cpp, src/svd_stack.cpp, include/utils/numerical_stable.hpp,
// src/measure/measure_methods.cpp); only the data placement differs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "dqmc_device.cuh"

namespace dqmc {

namespace {

__device__ __forceinline__ double warp_sum_g(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ bool is_general(const WalkerDev& w) { return w.path != 0; }

// Slice t handled at step j, in-segment index q (false when q is past the segment).
__device__ __forceinline__ bool slice_of(const WalkerDev& w, int mode, int j, int q, int& t, int& nsl, int& t_hi) {
  if (j >= w.nstack) return false;
  const int k = (mode == MODE_FWD) ? j : (w.nstack - 1 - j);
  const int t_lo = k * w.pace + 1;
  t_hi = min((k + 1) * w.pace, w.Lt);
  nsl = t_hi - t_lo + 1;
  if (q >= nsl) return false;
  t = (mode == MODE_FWD) ? t_lo + q : t_hi - q;
  return true;
}

// exp(sgn * spin_factor * alpha * s(t-1, i))
__device__ __forceinline__ double bscale(const WalkerDev& w, int t, int spin, int sgn, int i) {
  const int sf = (w.model == 0 && spin == 1) ? -1 : 1;
  const int s = w.fields[(long long)(t - 1) * w.N + i];
  return (sgn * sf * s > 0) ? w.e_pa : w.e_ma;
}

__device__ __forceinline__ double* chain_buf(const WalkerDev& w, int spin, int which) {
  return w.chain + ((long long)which * w.S + spin) * w.N * w.N;
}

}  // namespace

// --------------------------------------------------------------------------
// Batched FP64 GEMM, 64x64 output tile per CTA, 16-deep K steps staged in
// SMEM, 4x4 register tile per thread.  The operation (operands, transposes,
// fused diagonal scalings, epilogue) is selected by OP; each CTA finds its
// walker, spin and slice from the descriptors.
// --------------------------------------------------------------------------
enum GemmOp {
  OP_WL_FWD = 0,   // work = diag(e^{+}) expK G          (mult_B_from_left)
  OP_WR_FWD = 1,   // G    = work expK^-1 diag(e^{-})    (mult_invB_from_right)
  OP_WR_BWD = 2,   // work = G diag(e^{+}) expK          (mult_B_from_right)
  OP_WL_BWD = 3,   // G    = expK^-1 diag(e^{-}) work    (mult_invB_from_left)
  OP_CH_FWD = 4,   // chain' = diag(e^{+}) expK chain    (B-chain, forward)
  OP_CH_BWD = 5,   // chain' = expK^T diag(e^{+}) chain  (B-chain, backward / init)
  OP_GA = 6,       // M  = Dlmax^-1 (U_L^T U_R) Drmax^-1
  OP_GB = 7,       // M += Dlmin (F_L F_R^T) Drmin
  OP_GG = 8,       // G  = (U_R Drmax^-1) X, wrap error, trace
  // dynamic half-sweep (sweep_for_dynamic_greens, src/dqmc_walker.cpp:424-524)
  OP_DT0 = 9,      // G(t,0) = diag(e+) expK G(t-1,0)          (mult_B_from_left)
  OP_D0T = 10,     // G(0,t) = G(0,t-1) expK^-1 diag(e-)       (mult_invB_from_right)
  OP_DT0_OUT = 11, // G(t,0) = (U_R Drmax^-1) X1, X1 = M^-1 Dlmin F_L; wrap error
  OP_D0T_OUT = 12, // G(0,t) = -(F_R^T Drmin) X, X = M^-1 Dlmax^-1 U_L^T; wrap error
};

constexpr int kTile = 64, kTk = 16;

template <int OP>
__global__ void __launch_bounds__(256) gemm_op_kernel(const WalkerDev* __restrict__ W, int mode, int j, int q,
                                                      int trace_slot) {
  const int wi = blockIdx.z >> 1, sp = blockIdx.z & 1;
  const WalkerDev& w = W[wi];
  if (!is_general(w) || sp >= w.S) return;
  const int N = w.N;
  const int r0 = blockIdx.y * kTile, c0 = blockIdx.x * kTile;
  if (r0 >= N || c0 >= N) return;
  int t = 0, nsl = 0, t_hi = 0;
  constexpr bool dyn_prop = OP == OP_DT0 || OP == OP_D0T;
  constexpr bool dyn_out = OP == OP_DT0_OUT || OP == OP_D0T_OUT;
  const bool slice_op = OP <= OP_CH_BWD || dyn_prop;
  if ((dyn_prop || dyn_out) && !w.gt0) return;
  if (slice_op && w.cb) return;  // checkerboard walkers take cb_general_kernel (expK is null for them)
  if (slice_op && w.path == 2) return;  // mixed walkers take the tensor-core products
  if (slice_op && !slice_of(w, mode, j, q, t, nsl, t_hi)) return;
  if (!slice_op && j >= w.nstack) return;
  if (!slice_op && w.ozstab) return;  // stabilized by kernels_stab_oz.cu

  const long long NN = (long long)N * N;
  double* G = w.G + sp * NN;
  double* work = w.work + sp * NN;
  const double* A = nullptr;
  const double* B = nullptr;
  double* C = nullptr;
  // stack tops for the Green's assembly (lengths after this step's push)
  int nl = 0, nr = 0;
  if (!slice_op) {
    if (mode == MODE_FWD) { nl = j + 1; nr = w.nstack - 1 - j; }
    else if (mode == MODE_BWD) { nl = w.nstack - 1 - j; nr = j + 1; }
    else { nl = 0; nr = w.nstack; }
  }
  if (!slice_op && !(nl > 0 && nr > 0)) return;  // boundary steps: prep/out kernels
  const double* UL = nl ? stack_level(w, 0, sp, nl - 1) : nullptr;
  const double* UR = nr ? stack_level(w, 1, sp, nr - 1) : nullptr;
  const double* DL = UL ? UL + 2 * NN : nullptr;
  const double* DR = UR ? UR + 2 * NN : nullptr;
  double* scr = w.scr + sp * 2 * NN;  // M (col-major), Y/X (row-major)
  // dynamic buffers: [2][S][N*N], slot = parity of the slice
  const int t_end = min((j + 1) * w.pace, w.Lt);  // forward step j ends at this slice
  auto dbuf = [&](double* base, int par) { return base + ((long long)(par & 1) * w.S + sp) * NN; };
  switch (OP) {
    case OP_WL_FWD: A = w.expK; B = G; C = work; break;
    case OP_WR_FWD: A = work; B = w.invK; C = G; break;
    case OP_WR_BWD: A = G; B = w.expK; C = work; break;
    case OP_WL_BWD: A = w.invK; B = work; C = G; break;
    case OP_CH_FWD:
    case OP_CH_BWD: A = w.expK; B = chain_buf(w, sp, q & 1); C = chain_buf(w, sp, (q + 1) & 1); break;
    case OP_GA: A = UL; B = UR; C = scr; break;
    case OP_GB: A = UL + NN; B = UR + NN; C = scr; break;      // F_L, F_R
    case OP_GG: A = UR; B = scr + NN; C = G; break;           // U_R, X (row-major)
    case OP_DT0: A = w.expK; B = dbuf(w.gt0, t - 1); C = dbuf(w.gt0, t); break;
    case OP_D0T: A = dbuf(w.g0t, t - 1); B = w.invK; C = dbuf(w.g0t, t); break;
    case OP_DT0_OUT: A = UR; B = w.dynx + sp * NN; C = dbuf(w.gt0, t_end); break;   // X1 row-major
    case OP_D0T_OUT: A = UR + NN; B = scr + NN; C = dbuf(w.g0t, t_end); break;      // F_R, X row-major
  }

  __shared__ double As[kTk][kTile + 1];
  __shared__ double Bs[kTk][kTile + 1];
  __shared__ double s_red[8];
  __shared__ double s_inv[(OP == OP_GG || dyn_out) ? kMaxN : 1];  // 1 / max(D_R, 1) or min(D_R, 1) along k
  const int tid = threadIdx.x, tx = tid & 15, ty = tid >> 4;
  if (OP == OP_GG || OP == OP_DT0_OUT) {
    for (int k = tid; k < N; k += 256) s_inv[k] = 1.0 / fmax(DR[k], 1.0);
    __syncthreads();
  } else if (OP == OP_D0T_OUT) {
    for (int k = tid; k < N; k += 256) s_inv[k] = fmin(DR[k], 1.0);
    __syncthreads();
  }
  double acc[4][4];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;

  for (int k0 = 0; k0 < N; k0 += kTk) {
    // A tile: rows r0..r0+63, k k0..k0+15 -> As[kk][rr]
#pragma unroll
    for (int e = tid; e < kTile * kTk; e += 256) {
      const int rr = e % kTile, kk = e / kTile;
      const int r = r0 + rr, k = k0 + kk;
      double v = 0.0;
      if (r < N && k < N) {
        switch (OP) {
          case OP_WL_FWD: v = A[(long long)k * N + r] * bscale(w, t, sp, +1, r); break;
          case OP_WR_FWD: v = A[(long long)k * N + r]; break;
          case OP_WR_BWD: v = A[(long long)k * N + r] * bscale(w, t, sp, +1, k); break;
          case OP_WL_BWD: v = A[(long long)k * N + r]; break;
          case OP_CH_FWD: v = A[(long long)k * N + r] * bscale(w, t, sp, +1, r); break;
          case OP_CH_BWD: v = A[(long long)r * N + k] * bscale(w, t, sp, +1, k); break;  // expK^T
          case OP_GA: v = A[(long long)r * N + k]; break;  // U_L^T (r,k) = U_L(k,r)
          case OP_GB: v = A[(long long)k * N + r]; break;
          case OP_GG: v = A[(long long)k * N + r] * s_inv[k]; break;  // U_R(r,k) / drmax_k
          case OP_DT0: v = A[(long long)k * N + r] * bscale(w, t, sp, +1, r); break;
          case OP_D0T: v = A[(long long)k * N + r]; break;
          case OP_DT0_OUT: v = A[(long long)k * N + r] * s_inv[k]; break;
          case OP_D0T_OUT: v = A[(long long)r * N + k] * s_inv[k]; break;  // F_R^T(r,k) drmin_k
        }
      }
      As[kk][rr] = v;
    }
    // B tile: k k0..k0+15, cols c0..c0+63 -> Bs[kk][cc]
#pragma unroll
    for (int e = tid; e < kTile * kTk; e += 256) {
      const int kk = e % kTk, cc = e / kTk;
      const int k = k0 + kk, c = c0 + cc;
      double v = 0.0;
      if (k < N && c < N) {
        switch (OP) {
          case OP_WL_FWD: v = B[(long long)c * N + k]; break;
          case OP_WR_FWD: v = B[(long long)c * N + k]; break;
          case OP_WR_BWD: v = B[(long long)c * N + k]; break;
          case OP_WL_BWD: v = B[(long long)c * N + k] * bscale(w, t, sp, -1, k); break;
          case OP_CH_FWD: v = B[(long long)c * N + k]; break;
          case OP_CH_BWD: v = B[(long long)c * N + k]; break;
          case OP_GA: v = B[(long long)c * N + k]; break;
          case OP_GB: v = B[(long long)k * N + c]; break;  // F_R^T(k,c) = F_R(c,k)
          case OP_GG: v = B[(long long)k * N + c]; break;                     // X row-major
          case OP_DT0: v = B[(long long)c * N + k]; break;
          case OP_D0T: v = B[(long long)c * N + k]; break;
          case OP_DT0_OUT: v = B[(long long)k * N + c]; break;  // X1 row-major
          case OP_D0T_OUT: v = B[(long long)k * N + c]; break;  // X row-major
        }
      }
      Bs[kk][cc] = v;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTk; ++kk) {
      double av[4], bv[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) av[a] = As[kk][ty + 16 * a];
#pragma unroll
      for (int b = 0; b < 4; ++b) bv[b] = Bs[kk][tx + 16 * b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = fma(av[a], bv[b], acc[a][b]);
    }
    __syncthreads();
  }

  // epilogue
  double err = 0.0;
  bool finite = true;
  double* tr = (OP == OP_GG && w.trace && trace_slot >= 0 && trace_slot < w.trace_cap)
                   ? w.trace + ((long long)trace_slot * 2 + sp) * NN : nullptr;
  const bool check = (OP == OP_GG) && !(mode == MODE_INIT || (mode == MODE_BWD && j == w.nstack - 1));
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) {
      const int r = r0 + ty + 16 * a, c = c0 + tx + 16 * b;
      if (r >= N || c >= N) continue;
      double v = acc[a][b];
      const long long o = (long long)c * N + r;
      switch (OP) {
        case OP_WR_FWD: v *= bscale(w, t, sp, -1, c); break;
        case OP_D0T: v *= bscale(w, t, sp, -1, c); break;
        case OP_D0T_OUT: v = -v; break;
        case OP_GA: v /= fmax(DL[r], 1.0) * fmax(DR[c], 1.0); break;
        case OP_GB: v *= fmin(DL[r], 1.0) * fmin(DR[c], 1.0); break;
        default: break;
      }
      if (OP == OP_GB) {
        C[o] += v;
      } else if (dyn_out) {
        err = fmax(err, fabs(v - C[o]));
        if (!isfinite(v)) finite = false;
        C[o] = v;
      } else if (OP == OP_GG) {
        if (check) err = fmax(err, fabs(v - C[o]));
        if (!isfinite(v)) finite = false;
        C[o] = v;
        if (tr) tr[o] = v;
        if (w.S == 1) {
          C[NN + o] = v;
          if (tr) tr[NN + o] = v;
        }
      } else {
        C[o] = v;
      }
    }
  if (OP == OP_GG || dyn_out) {
    if (!finite) atomicOr(w.status, ST_NONFINITE_G);
    if (check || dyn_out) {
      for (int o = 16; o > 0; o >>= 1) err = fmax(err, __shfl_xor_sync(0xffffffffu, err, o));
      if ((tid & 31) == 0) s_red[tid >> 5] = err;
      __syncthreads();
      if (tid == 0) {
        double m = 0;
        for (int k = 0; k < 8; ++k) m = fmax(m, s_red[k]);
        atomicMax(w.wrap_bits, (unsigned long long)__double_as_longlong(m));
      }
    }
  }
}

// --------------------------------------------------------------------------
// Checkerboard on global matrices (general N): one CTA per (walker, spin).
//   kind 0: wrap fwd  G <- P_A P_B G (scale rows e^+) ; G <- G P_B^-1 P_A^-1 (scale cols e^-)
//   kind 1: wrap bwd  G <- G diag(e^+) P_A P_B ; G <- P_B^-1 P_A^-1 diag(e^-) G
//   kind 2: chain fwd C <- diag(e^+) P_A P_B C
//   kind 3: chain bwd C <- P_B P_A diag(e^+) C
//   kind 4: time-displaced steps of the dynamic half-sweep (mult_B_from_left and
//           mult_invB_from_right, src/dqmc_walker.cpp:455-466):
//           G(t,0) <- diag(e^+) P_A P_B G(t-1,0),  G(0,t) <- G(0,t-1) P_B^-1 P_A^-1 diag(e^-)
// --------------------------------------------------------------------------
__device__ void cbg_pass(double* M, int N, int L, int parity, const double* P, bool left, const double* pre,
                         const double* post) {
  const int nq = (L >> 1) * (L >> 1), half = L >> 1;
  for (int it = threadIdx.x; it < nq * N; it += blockDim.x) {
    int q, x2;
    if (left) { q = it % nq; x2 = it / nq; } else { x2 = it % N; q = it / N; }
    const int x = 2 * (q % half) + parity, y = 2 * (q / half) + parity;
    const int x1 = (x + 1) % L, y1 = (y + 1) % L;
    const int idx[4] = {x + L * y, x1 + L * y, x + L * y1, x1 + L * y1};
    double v[4];
    for (int a = 0; a < 4; ++a) {
      v[a] = left ? M[(long long)x2 * N + idx[a]] : M[(long long)idx[a] * N + x2];
      if (pre) v[a] *= pre[idx[a]];
    }
    for (int a = 0; a < 4; ++a) {
      double o = 0.0;
      for (int b = 0; b < 4; ++b) o = left ? fma(P[a * 4 + b], v[b], o) : fma(v[b], P[b * 4 + a], o);
      if (post) o *= post[idx[a]];
      if (left) M[(long long)x2 * N + idx[a]] = o; else M[(long long)idx[a] * N + x2] = o;
    }
  }
}

__global__ void __launch_bounds__(256) cb_general_kernel(const WalkerDev* __restrict__ W, int mode, int j, int q,
                                                         int kind) {
  const int wi = blockIdx.x >> 1, sp = blockIdx.x & 1;
  const WalkerDev& w = W[wi];
  if (!is_general(w) || !w.cb || sp >= w.S) return;
  int t, nsl, t_hi;
  if (!slice_of(w, mode, j, q, t, nsl, t_hi)) return;
  extern __shared__ double sh[];
  const int N = w.N, L = w.L;
  double* dpos = sh;
  double* dneg = sh + N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    dpos[i] = bscale(w, t, sp, +1, i);
    dneg[i] = bscale(w, t, sp, -1, i);
  }
  __syncthreads();
  double* G = w.G + (long long)sp * N * N;
  double* C = chain_buf(w, sp, 0);
  switch (kind) {
    case 0:
      cbg_pass(G, N, L, 1, w.cbP, true, nullptr, nullptr); __syncthreads();
      cbg_pass(G, N, L, 0, w.cbP, true, nullptr, dpos); __syncthreads();
      cbg_pass(G, N, L, 1, w.cbI, false, nullptr, nullptr); __syncthreads();
      cbg_pass(G, N, L, 0, w.cbI, false, nullptr, dneg); __syncthreads();
      break;
    case 1:
      cbg_pass(G, N, L, 0, w.cbP, false, dpos, nullptr); __syncthreads();
      cbg_pass(G, N, L, 1, w.cbP, false, nullptr, nullptr); __syncthreads();
      cbg_pass(G, N, L, 0, w.cbI, true, dneg, nullptr); __syncthreads();
      cbg_pass(G, N, L, 1, w.cbI, true, nullptr, nullptr); __syncthreads();
      break;
    case 2:
      cbg_pass(C, N, L, 1, w.cbP, true, nullptr, nullptr); __syncthreads();
      cbg_pass(C, N, L, 0, w.cbP, true, nullptr, dpos); __syncthreads();
      break;
    case 3:
      cbg_pass(C, N, L, 0, w.cbP, true, dpos, nullptr); __syncthreads();
      cbg_pass(C, N, L, 1, w.cbP, true, nullptr, nullptr); __syncthreads();
      break;
    case 4: {
      if (!w.gt0) return;
      // ping-pong slots [parity][S][N*N]: read slice t - 1's, write slice t's, then in place
      const long long NN = (long long)N * N;
      const double* a0 = w.gt0 + ((long long)((t - 1) & 1) * w.S + sp) * NN;
      double* a1 = w.gt0 + ((long long)(t & 1) * w.S + sp) * NN;
      const double* b0 = w.g0t + ((long long)((t - 1) & 1) * w.S + sp) * NN;
      double* b1 = w.g0t + ((long long)(t & 1) * w.S + sp) * NN;
      for (long long e = threadIdx.x; e < NN; e += blockDim.x) {
        a1[e] = a0[e];
        b1[e] = b0[e];
      }
      __syncthreads();
      cbg_pass(a1, N, L, 1, w.cbP, true, nullptr, nullptr); __syncthreads();
      cbg_pass(a1, N, L, 0, w.cbP, true, nullptr, dpos); __syncthreads();
      cbg_pass(b1, N, L, 1, w.cbI, false, nullptr, nullptr); __syncthreads();
      cbg_pass(b1, N, L, 0, w.cbI, false, nullptr, dneg); __syncthreads();
      break;
    }
  }
}

// --------------------------------------------------------------------------
// Chain start of step j: chain <- U_top diag(D_top) or I (general walkers).
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(256) chain_init_general_kernel(const WalkerDev* __restrict__ W, int mode, int j) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!is_general(w) || sp >= w.S || j >= w.nstack) return;
  const int N = w.N;
  const int side = (mode == MODE_FWD) ? 0 : 1;
  const double* lv = j ? stack_level(w, side, sp, j - 1) : nullptr;
  double* C = chain_buf(w, sp, 0);
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < (long long)N * N;
       e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e % N), c = (int)(e / N);
    C[e] = lv ? lv[e] * lv[2LL * N * N + c] : ((r == c) ? 1.0 : 0.0);
  }
}

// --------------------------------------------------------------------------
// Metropolis on global G (general N), one CTA of 512 threads per walker.
// Warp 0 decides with look-ahead (as in the SMEM kernel), warps 1..15 apply
// the rank-1 update of the previous accepted site.
// --------------------------------------------------------------------------
constexpr int kMetroThreads = 512;

__global__ void __launch_bounds__(kMetroThreads) metropolis_general_kernel(const WalkerDev* __restrict__ W, int mode,
                                                                          int j, int q) {
  const WalkerDev& w = W[blockIdx.x];
  if (!is_general(w)) return;
  int t, nsl, t_hi;
  if (!slice_of(w, mode, j, q, t, nsl, t_hi)) return;
  extern __shared__ double sh[];
  const int N = w.N, S = w.S, Lt = w.Lt;
  double* vec = sh;             // [4][N]: f u (2 spins), e_i - G(i,:) (2 spins)
  double* diag_pre = sh + 4 * N;  // [2][N]
  int8_t* s_field = (int8_t*)(sh + 6 * N);
  __shared__ int s_next;
  __shared__ double s_f[2];
  const long long NN = (long long)N * N;
  double* Gs[2] = {w.G, (S == 2) ? w.G + NN : w.G};
  const int eff = t - 1;
  for (int i = threadIdx.x; i < N; i += blockDim.x) s_field[i] = w.fields[(long long)eff * N + i];
  double sign = *w.sign;
  long long acc_count = 0;
  const unsigned long long sweep = (w.rng == 1) ? *w.sweep_ctr : 0ULL;
  __syncthreads();

  auto decide_from = [&](int i0, bool pending) {
    for (int i = i0; i < N; ++i) {
      const int s = s_field[i];
      const int si = s > 0 ? 0 : 1;
      double gu, gd;
      if (pending) {
        gu = fma(-vec[2 * N + i], vec[i], diag_pre[i]);
        gd = (S == 2) ? fma(-vec[3 * N + i], vec[N + i], diag_pre[N + i]) : gu;
      } else {
        gu = Gs[0][(long long)i * N + i];
        gd = Gs[1][(long long)i * N + i];
      }
      const FlipRatio q = flip_ratio(w, si, gu, gd);  // reference operation order
      const double r = q.r;
      const int attempt = (mode == MODE_FWD) ? (eff * N + i) : ((Lt - t) * N + i);
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
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
  while (s_next < N) {
    const int i = s_next;
    for (int r = threadIdx.x; r < N; r += blockDim.x) {
      for (int sp = 0; sp < S; ++sp) {
        const double* g = Gs[sp];
        vec[sp * N + r] = s_f[sp] * g[(long long)i * N + r];
        vec[(2 + sp) * N + r] = ((r == i) ? 1.0 : 0.0) - g[(long long)r * N + i];
        diag_pre[sp * N + r] = g[(long long)r * N + r];
      }
    }
    __syncthreads();
    if (wid == 0) {
      if (lane == 0) s_next = decide_from(i + 1, true);
    } else {
      for (int sp = 0; sp < S; ++sp) {
        double* g = Gs[sp];
        const double* wv = vec + (2 + sp) * N;
        const double* uv = vec + sp * N;
        for (int c = wid - 1; c < N; c += nwarp - 1) {
          const double wc = -wv[c];
          double* gc = g + (long long)c * N;
          for (int r = lane; r < N; r += 32) gc[r] = fma(wc, uv[r], gc[r]);
        }
      }
    }
    __syncthreads();
  }
  int8_t* frw = w.fields + (long long)eff * N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) frw[i] = s_field[i];
  if (threadIdx.x == 0) {
    *w.sign = sign;
    *w.accepts += acc_count;
    if (mode == MODE_BWD && t == Lt) *w.sign_Lt = sign;
  }
}

// --------------------------------------------------------------------------
// Equal-time measurement on global G (general N); mode/j/q select the slot as
// in the SMEM kernels.  after_stab = 1 measures the slot closing the step
// with the fresh G (forward) or slot Lt-1 with the final G(0) (backward).
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(256) measure_general_kernel(const WalkerDev* __restrict__ W, int mode, int j, int q,
                                                              int after_stab) {
  const WalkerDev& w = W[blockIdx.x];
  if (!is_general(w)) return;
  double sg;
  if (after_stab) {
    if (j >= w.nstack) return;
    if (mode == MODE_BWD && j != w.nstack - 1) return;
    sg = (mode == MODE_BWD) ? *w.sign_Lt : *w.sign;
  } else {
    int t, nsl, t_hi;
    if (!slice_of(w, mode, j, q, t, nsl, t_hi)) return;
    const bool here = (mode == MODE_FWD) ? (t != t_hi) : (t != w.Lt);
    if (!here) return;
    sg = *w.sign;
  }
  const int N = w.N, L = w.L;
  const long long NN = (long long)N * N;
  const double* gu = w.G;
  const double* gd = (w.S == 2) ? w.G + NN : w.G;
  extern __shared__ double sh[];
  double* du = sh;
  double* dd = sh + N;
  __shared__ double red[8 * 8];
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    du[i] = 1.0 - gu[(long long)i * N + i];
    dd[i] = 1.0 - gd[(long long)i * N + i];
  }
  __syncthreads();
  // The pair sums run with the separable parts factored out (per column jj the lane
  // sums c_u = sum_i ff(jj - i) du_i and c_d) and the i = jj terms corrected in the
  // site loop, so a pair costs 8 FP64 operations (5 with one spin matrix) instead of 14:
  //   v4 = sum ff (Gu_ji + Gd_ji),  v5 = sum ff (du_i du_j + dd_i dd_j + guc Gu_ij + gdc Gd_ij),
  //   v6 = sum ff (dd_i du_j + du_i dd_j),  v7 = sum guc gdc,  guc = delta_ij - Gu_ji.
  const bool one = (w.S == 1);
  const double ff0 = w.ff[0];
  double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const double a = 1.0 - du[i], b = 1.0 - dd[i];
    v[0] += a + b;
    v[1] += du[i] * dd[i];
    v[2] += a + b - 2 * a * b;
    // bonds to the +x, +y (, +z) neighbours (measure_methods.cpp:87-95)
    const int jx = site_nn(L, i, 0), jy = site_nn(L, i, 1);
    double kin = gu[(long long)jx * N + i] + gd[(long long)jx * N + i] + gu[(long long)jy * N + i] + gd[(long long)jy * N + i];
    if (w.dim == 3) {
      const int jz = site_nn(L, i, 2);
      kin += gu[(long long)jz * N + i] + gd[(long long)jz * N + i];
    }
    v[3] += kin;
    // i = jj: the pair loop's off-diagonal forms give -ff0 (Gu_ii^2 + Gd_ii^2) and Gu_ii Gd_ii
    v[5] += ff0 * (a + b);
    v[7] += du[i] * dd[i] - a * b;
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  double p4 = 0.0, p5 = 0.0;  // pair parts of v4 and v5 (one spin matrix: doubled below)
  const int dim = w.dim;
  for (int jj = wid; jj < N; jj += blockDim.x >> 5) {
    const int xj = jj % L, yj = jj / L;
    double cu = 0.0, cd = 0.0;
    for (int i = lane; i < N; i += 32) {
      int r;
      if (dim == 2) {
        int dx = xj - i % L, dy = yj - i / L;
        dx += (dx < 0) ? L : 0;
        dy += (dy < 0) ? L : 0;
        r = dx + dy * L;
      } else {
        r = site_disp(L, 3, i, jj);
      }
      const double ff = w.ff[r];
      const double gu_ij = gu[(long long)jj * N + i], gu_ji = gu[(long long)i * N + jj];
      cu = fma(ff, du[i], cu);
      if (one) {
        p4 = fma(ff, gu_ji, p4);
        p5 = fma(-ff, gu_ji * gu_ij, p5);
        v[7] = fma(gu_ji, gu_ji, v[7]);
      } else {
        const double gd_ij = gd[(long long)jj * N + i], gd_ji = gd[(long long)i * N + jj];
        cd = fma(ff, dd[i], cd);
        p4 = fma(ff, gu_ji + gd_ji, p4);
        p5 = fma(-ff, fma(gd_ji, gd_ij, gu_ji * gu_ij), p5);
        v[7] = fma(gu_ji, gd_ji, v[7]);
      }
    }
    if (one) {
      v[5] = fma(2.0 * du[jj], cu, v[5]);
      v[6] = fma(2.0 * du[jj], cu, v[6]);
    } else {
      v[5] += du[jj] * cu + dd[jj] * cd;
      v[6] += du[jj] * cd + dd[jj] * cu;
    }
  }
  v[4] += one ? 2.0 * p4 : p4;
  v[5] += one ? 2.0 * p5 : p5;
  for (int k = 0; k < 8; ++k) {
    const double s = warp_sum_g(v[k]);
    if (lane == 0) red[k * 8 + wid] = s;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot[8];
    for (int k = 0; k < 8; ++k) {
      tot[k] = 0;
      for (int q2 = 0; q2 < (int)(blockDim.x >> 5); ++q2) tot[k] += red[k * 8 + q2];
    }
    const double n = (double)N;
    double* o = w.obs;
    o[0] += sg * (2.0 - tot[0] / n);
    o[1] += sg * tot[1] / n;
    o[2] += sg * (2.0 * w.hop_t) * tot[3] / n;
    o[3] += sg * (1.0 - 0.5 * tot[4] / n);
    o[4] += sg * tot[2] / n;
    o[5] += sg * (tot[5] - tot[6]) / (n * n);
    o[6] += sg * (tot[5] + tot[6]) / (n * n);
    o[7] += sg * tot[7] / n;
    o[8] += sg;
    for (int k = 0; k < kNumObs; ++k) w.obs_cnt[k] += 1;
  }
}

// --------------------------------------------------------------------------
// Column-pivoted QR push, general N: one CTA per (walker, spin), thread per
// column, matrix in a row-major HBM/L2 scratch (coalesced across threads).
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(1024) push_general_kernel(const WalkerDev* __restrict__ W, int mode, int j) {
  const int wi = blockIdx.x >> 1, sp = blockIdx.x & 1;
  const WalkerDev& w = W[wi];
  if (!is_general(w) || w.ozstab || sp >= w.S || j >= w.nstack) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  const int side = (mode == MODE_FWD) ? 0 : 1;
  int nsl = 0;
  {
    const int k = (mode == MODE_FWD) ? j : (w.nstack - 1 - j);
    nsl = min((k + 1) * w.pace, w.Lt) - k * w.pace;
  }
  const double* Cin = w.cb ? chain_buf(w, sp, 0) : chain_buf(w, sp, nsl & 1);
  double* X = w.scr + sp * 2 * NN;  // row-major: X[r*N + c]
  extern __shared__ double sh[];
  double* v = sh;          // reflector / scratch column [N]
  double* vn1 = sh + N;
  double* vn2 = sh + 2 * N;
  double* tau = sh + 3 * N;
  double* invd = sh + 4 * N;
  int* perm = (int*)(sh + 5 * N);
  __shared__ int s_piv;
  __shared__ double s_tau, s_scal;
  __shared__ long long s_key[32];
  __shared__ int s_idx[32];
  const int tj = threadIdx.x;
  const bool own = tj < N;
  auto Xat = [&](int r, int c) -> double& { return X[(long long)r * N + c]; };

  if (own) {
    double s0 = 0, s1 = 0;
    for (int r = 0; r < N; ++r) {
      const double a = Cin[(long long)tj * N + r];
      Xat(r, tj) = a;
      if (r & 1) s1 = fma(a, a, s1); else s0 = fma(a, a, s0);
    }
    vn1[tj] = vn2[tj] = sqrt(s0 + s1);
    perm[tj] = tj;
  }
  __syncthreads();
  const double tol3z = 1.4901161193847656e-08;
  const int nwarps = (blockDim.x + 31) >> 5;
  for (int k = 0; k < N; ++k) {
    // pivot
    long long key = (own && tj >= k) ? __double_as_longlong(vn1[tj]) : -1LL;
    int bi = tj;
    for (int o = 16; o > 0; o >>= 1) {
      const long long ok = __shfl_xor_sync(0xffffffffu, key, o);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
      if (ok > key || (ok == key && oi < bi)) { key = ok; bi = oi; }
    }
    if ((tj & 31) == 0) { s_key[tj >> 5] = key; s_idx[tj >> 5] = bi; }
    __syncthreads();
    if (tj == 0) {
      long long bk = s_key[0];
      int b = s_idx[0];
      for (int q = 1; q < nwarps; ++q)
        if (s_key[q] > bk || (s_key[q] == bk && s_idx[q] < b)) { bk = s_key[q]; b = s_idx[q]; }
      s_piv = b;
    }
    __syncthreads();
    const int pv = s_piv;
    if (pv != k) {
      if (own) {  // thread tj swaps row tj of columns k and pv
        const double a = Xat(tj, k);
        Xat(tj, k) = Xat(tj, pv);
        Xat(tj, pv) = a;
      }
      if (tj == 0) {
        const int tp = perm[k]; perm[k] = perm[pv]; perm[pv] = tp;
        double tv = vn1[k]; vn1[k] = vn1[pv]; vn1[pv] = tv;
        tv = vn2[k]; vn2[k] = vn2[pv]; vn2[pv] = tv;
      }
      __syncthreads();
    }
    // reflector: column k rows > k into v (SMEM), norm by block reduction
    double xr = 0.0;
    if (own && tj > k) { xr = Xat(tj, k); v[tj] = xr; }
    double s = warp_sum_g(xr * xr);
    if ((tj & 31) == 0) s_key[tj >> 5] = __double_as_longlong(s);
    __syncthreads();
    if (tj == 0) {
      double xn2 = 0;
      for (int q = 0; q < nwarps; ++q) xn2 += __longlong_as_double(s_key[q]);
      const double alpha = Xat(k, k);
      double t2 = 0.0, beta = alpha, scal = 1.0;
      if (xn2 != 0.0) {
        const double nrm = sqrt(alpha * alpha + xn2);
        beta = alpha >= 0 ? -nrm : nrm;
        t2 = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      s_tau = t2; s_scal = scal;
      tau[k] = t2;
      Xat(k, k) = beta;
    }
    __syncthreads();
    if (own && tj > k) {
      const double vv = v[tj] * s_scal;
      v[tj] = vv;
      Xat(tj, k) = vv;
    }
    __syncthreads();
    const double tk = s_tau;
    if (own && tj > k) {
      if (tk != 0.0) {
        double a0 = Xat(k, tj), a1 = 0.0;
        int r = k + 1;
        for (; r + 1 < N; r += 2) {
          a0 = fma(v[r], Xat(r, tj), a0);
          a1 = fma(v[r + 1], Xat(r + 1, tj), a1);
        }
        if (r < N) a0 = fma(v[r], Xat(r, tj), a0);
        const double wv = (a0 + a1) * tk;
        Xat(k, tj) -= wv;
        for (r = k + 1; r < N; ++r) Xat(r, tj) = fma(-wv, v[r], Xat(r, tj));
      }
      const double v1 = vn1[tj];
      if (v1 != 0.0) {
        double tmp = fabs(Xat(k, tj)) / v1;
        tmp = fmax(0.0, 1.0 - tmp * tmp);
        const double r2 = v1 / vn2[tj];
        if (tmp * r2 * r2 <= tol3z) {
          double q0 = 0, q1 = 0;
          int r = k + 1;
          for (; r + 1 < N; r += 2) {
            q0 = fma(Xat(r, tj), Xat(r, tj), q0);
            q1 = fma(Xat(r + 1, tj), Xat(r + 1, tj), q1);
          }
          if (r < N) q0 = fma(Xat(r, tj), Xat(r, tj), q0);
          vn1[tj] = vn2[tj] = sqrt(q0 + q1);
        } else {
          vn1[tj] = v1 * sqrt(tmp);
        }
      }
    }
    __syncthreads();
  }
  // D and F = (D^-1 R P^T) F_prev
  double* lv = stack_level(w, side, sp, j);
  double* Uo = lv;
  double* Fo = lv + NN;
  double* Do = lv + 2 * NN;
  if (own) {
    const double d = fabs(Xat(tj, tj));
    Do[tj] = d;
    invd[tj] = (d != 0.0) ? 1.0 / d : 0.0;
    if (d == 0.0 || !isfinite(d)) atomicOr(w.status, ST_SINGULAR);
  }
  __syncthreads();
  if (own) {
    const int c = tj;
    if (j == 0) {
      double* fc = Fo + (long long)perm[c] * N;
      for (int i = 0; i < N; ++i) fc[i] = (i <= c) ? Xat(i, c) * invd[i] : 0.0;
    } else {
      const double* fp = stack_level(w, side, sp, j - 1) + NN + (long long)c * N;
      double* fo = Fo + (long long)c * N;
      for (int i = 0; i < N; ++i) {
        double a0 = 0.0, a1 = 0.0;
        int k = i;
        for (; k + 1 < N; k += 2) {
          a0 = fma(Xat(i, k), fp[perm[k]], a0);
          a1 = fma(Xat(i, k + 1), fp[perm[k + 1]], a1);
        }
        if (k < N) a0 = fma(Xat(i, k), fp[perm[k]], a0);
        fo[i] = (a0 + a1) * invd[i];
      }
    }
  }
  __syncthreads();
  // Q in place (dorg2r order); reflector i staged into v
  for (int i = N - 1; i >= 0; --i) {
    const double ti = tau[i];
    if (own && tj > i) v[tj] = Xat(tj, i);
    __syncthreads();
    if (i < N - 1 && own && tj > i && ti != 0.0) {
      double a0 = Xat(i, tj), a1 = 0.0;
      int r = i + 1;
      for (; r + 1 < N; r += 2) {
        a0 = fma(v[r], Xat(r, tj), a0);
        a1 = fma(v[r + 1], Xat(r + 1, tj), a1);
      }
      if (r < N) a0 = fma(v[r], Xat(r, tj), a0);
      const double wv = (a0 + a1) * ti;
      Xat(i, tj) -= wv;
      for (r = i + 1; r < N; ++r) Xat(r, tj) = fma(-wv, v[r], Xat(r, tj));
    }
    __syncthreads();
    if (own) {
      const int r = tj;
      if (r > i) Xat(r, i) = v[r] * -ti;
      else if (r == i) Xat(r, i) = 1.0 - ti;
      else Xat(r, i) = 0.0;
    }
    __syncthreads();
  }
  if (own)
    for (int r = 0; r < N; ++r) Uo[(long long)tj * N + r] = Xat(r, tj);
}

// --------------------------------------------------------------------------
// Green's assembly support (general N).
//   prep: boundary cases build M and Y; general case builds Y = Dlmax^-1 U_L^T
//         (M comes from OP_GA/OP_GB).  M col-major in scr, Y row-major in scr+NN.
//   lu:   solve M X = Y (partial pivoting), thread per column of [M | Y], X in Y.
//   out:  boundary cases write G = X (or X^T) with wrap error and trace.
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(256) greens_prep_general_kernel(const WalkerDev* __restrict__ W, int mode, int j) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!is_general(w) || w.ozstab || sp >= w.S || j >= w.nstack) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  int nl, nr;
  if (mode == MODE_FWD) { nl = j + 1; nr = w.nstack - 1 - j; }
  else if (mode == MODE_BWD) { nl = w.nstack - 1 - j; nr = j + 1; }
  else { nl = 0; nr = w.nstack; }
  double* M = w.scr + sp * 2 * NN;
  double* Y = M + NN;
  const bool both = nl > 0 && nr > 0;
  const double* lv = (nl > 0) ? stack_level(w, 0, sp, nl - 1) : stack_level(w, 1, sp, nr - 1);
  const double* U = lv;
  const double* F = lv + NN;
  const double* D = lv + 2 * NN;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < NN; e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e / N), c = (int)(e % N);   // Y row-major: Y[r*N + c]
    const double y = U[(long long)r * N + c] / fmax(D[r], 1.0);  // (Dmax^-1 U^T)(r,c)
    Y[e] = y;
    if (!both) M[(long long)c * N + r] = y + fmin(D[r], 1.0) * F[(long long)c * N + r];
  }
}

__global__ void __launch_bounds__(1024) lu_solve_general_kernel(const WalkerDev* __restrict__ W, int mode, int j) {
  const int wi = blockIdx.x >> 1, sp = blockIdx.x & 1;
  const WalkerDev& w = W[wi];
  if (!is_general(w) || w.ozstab || sp >= w.S || j >= w.nstack) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  double* M = w.scr + sp * 2 * NN;  // col-major
  double* Y = M + NN;               // row-major
  extern __shared__ double sh[];
  double* l = sh;  // multipliers of the current step
  __shared__ int s_p;
  __shared__ int s_bad;
  const int tid = threadIdx.x, nt = blockDim.x;
  if (tid == 0) s_bad = 0;
  for (int k = 0; k < N; ++k) {
    if (tid < 32) {  // pivot: warp argmax of |M(r,k)|, r >= k, on the integer bit patterns
      long long key = -1;
      int bi = k;
      for (int r = k + tid; r < N; r += 32) {
        const long long a = __double_as_longlong(M[(long long)k * N + r]) & 0x7fffffffffffffffLL;
        if (a > key) { key = a; bi = r; }
      }
      for (int o = 16; o > 0; o >>= 1) {
        const long long ok = __shfl_xor_sync(0xffffffffu, key, o);
        const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
        if (ok > key || (ok == key && oi < bi)) { key = ok; bi = oi; }
      }
      if (tid == 0) { s_p = bi; if (key == 0) s_bad = 1; }
    }
    __syncthreads();
    const int p = s_p;
    if (w.dpiv && tid == 0) w.dpiv[sp * N + k] = p;  // kept for a second right-hand side
    if (p != k) {  // swap rows k and p of M (all columns) and Y
      for (int c = tid; c < N; c += nt) {
        double* mc = M + (long long)c * N;
        const double a = mc[k]; mc[k] = mc[p]; mc[p] = a;
        const double b = Y[(long long)k * N + c]; Y[(long long)k * N + c] = Y[(long long)p * N + c];
        Y[(long long)p * N + c] = b;
      }
      __syncthreads();
    }
    const double piv = M[(long long)k * N + k];
    const double inv = (piv != 0.0) ? 1.0 / piv : 0.0;
    for (int r = k + 1 + tid; r < N; r += nt) {
      const double lr = M[(long long)k * N + r] * inv;
      M[(long long)k * N + r] = lr;
      l[r] = lr;
    }
    __syncthreads();
    // columns of M right of k, then all columns of Y (row-major: thread per column c)
    for (int c = k + 1 + tid; c < N; c += nt) {
      double* mc = M + (long long)c * N;
      const double mk = mc[k];
      if (mk != 0.0)
        for (int r = k + 1; r < N; ++r) mc[r] = fma(-l[r], mk, mc[r]);
    }
    for (int c = tid; c < N; c += nt) {
      const double yk = Y[(long long)k * N + c];
      if (yk != 0.0)
        for (int r = k + 1; r < N; ++r) Y[(long long)r * N + c] = fma(-l[r], yk, Y[(long long)r * N + c]);
    }
    __syncthreads();
  }
  // back substitution, thread per column of Y (reciprocal diagonal staged in l)
  for (int k = tid; k < N; k += nt) l[k] = 1.0 / M[(long long)k * N + k];
  __syncthreads();
  for (int c = tid; c < N; c += nt) {
    for (int k = N - 1; k >= 0; --k) {
      const double yk = Y[(long long)k * N + c] * l[k];
      Y[(long long)k * N + c] = yk;
      for (int r = 0; r < k; ++r) Y[(long long)r * N + c] = fma(-M[(long long)k * N + r], yk, Y[(long long)r * N + c]);
    }
  }
  if (tid == 0 && s_bad) atomicOr(w.status, ST_SINGULAR);
}

__global__ void __launch_bounds__(256) greens_out_general_kernel(const WalkerDev* __restrict__ W, int mode, int j,
                                                                 int trace_slot) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!is_general(w) || w.ozstab || sp >= w.S || j >= w.nstack) return;
  int nl, nr;
  if (mode == MODE_FWD) { nl = j + 1; nr = w.nstack - 1 - j; }
  else if (mode == MODE_BWD) { nl = w.nstack - 1 - j; nr = j + 1; }
  else { nl = 0; nr = w.nstack; }
  if (nl > 0 && nr > 0) return;  // general case finished by OP_GG
  const int N = w.N;
  const long long NN = (long long)N * N;
  const double* X = w.scr + sp * 2 * NN + NN;  // row-major
  double* G = w.G + sp * NN;
  double* tr = (w.trace && trace_slot >= 0 && trace_slot < w.trace_cap) ? w.trace + ((long long)trace_slot * 2 + sp) * NN
                                                                       : nullptr;
  const bool transpose_out = (nl == 0);
  const bool check = !(mode == MODE_INIT || (mode == MODE_BWD && j == w.nstack - 1));
  double err = 0.0;
  bool finite = true;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < NN; e += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(e % N), c = (int)(e / N);  // G col-major (r, c)
    const double v = transpose_out ? X[(long long)c * N + r] : X[(long long)r * N + c];
    if (check) err = fmax(err, fabs(v - G[e]));
    if (!isfinite(v)) finite = false;
    G[e] = v;
    if (tr) tr[e] = v;
    if (w.S == 1) {
      G[NN + e] = v;
      if (tr) tr[NN + e] = v;
    }
  }
  if (!finite) atomicOr(w.status, ST_NONFINITE_G);
  if (check) {
    for (int o = 16; o > 0; o >>= 1) err = fmax(err, __shfl_xor_sync(0xffffffffu, err, o));
    if ((threadIdx.x & 31) == 0) atomicMax(w.wrap_bits, (unsigned long long)__double_as_longlong(err));
  }
}

// sign(det G_up det G_dn) for general walkers: LU of a copy in scr (col-major)
__global__ void __launch_bounds__(1024) sign_general_kernel(const WalkerDev* __restrict__ W) {
  const WalkerDev& w = W[blockIdx.x];
  if (!is_general(w)) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  __shared__ int s_p, s_neg;
  extern __shared__ double sh[];
  double* l = sh;
  if (threadIdx.x == 0) s_neg = 0;
  for (int sp = 0; sp < 2; ++sp) {
    double* M = w.scr;  // spin 0 scratch reused sequentially
    const double* Gg = w.G + sp * NN;
    for (long long e = threadIdx.x; e < NN; e += blockDim.x) M[e] = Gg[e];
    __syncthreads();
    for (int k = 0; k < N; ++k) {
      if (threadIdx.x == 0) {
        int p = k;
        double m = fabs(M[(long long)k * N + k]);
        for (int r = k + 1; r < N; ++r) {
          const double a = fabs(M[(long long)k * N + r]);
          if (a > m) { m = a; p = r; }
        }
        s_p = p;
        if (p != k) ++s_neg;
        if (M[(long long)k * N + p] < 0) ++s_neg;
      }
      __syncthreads();
      const int p = s_p;
      if (p != k)
        for (int c = threadIdx.x; c < N; c += blockDim.x) {
          double* mc = M + (long long)c * N;
          const double a = mc[k]; mc[k] = mc[p]; mc[p] = a;
        }
      __syncthreads();
      const double inv = 1.0 / M[(long long)k * N + k];
      for (int r = k + 1 + threadIdx.x; r < N; r += blockDim.x) l[r] = M[(long long)k * N + r] * inv;
      __syncthreads();
      for (int c = k + 1 + threadIdx.x; c < N; c += blockDim.x) {
        double* mc = M + (long long)c * N;
        const double mk = mc[k];
        for (int r = k + 1; r < N; ++r) mc[r] = fma(-l[r], mk, mc[r]);
      }
      __syncthreads();
    }
  }
  if (threadIdx.x == 0) *w.sign = (s_neg % 2 == 0) ? 1.0 : -1.0;
}

// --------------------------------------------------------------------------
// Dynamic half-sweep (sweep_for_dynamic_greens, src/dqmc_walker.cpp:424-524):
// the forward half-sweep with the fields fixed, carrying G(t,0) and G(0,t)
// besides G(t,t).  At each stabilization, with M and X = M^-1 Dlmax^-1 U_L^T of
// the equal-time assembly (LU pivots kept):
//   G(t,0) = U_R Drmax^-1 M^-1 (Dlmin F_L)     (compute_dynamic_greens, :246-325)
//   G(0,t) = -F_R^T Drmin X                     (push-through form of the second
//            formula, exact for any right factor F; the reference's form needs an
//            orthogonal V)
// and at t = beta (right stack empty, H = Dmax^-1 U^T + Dmin F):
//   G(beta,0) = H^-1 Dmin F,  G(0,beta) = -H^-1 Dmax^-1 U^T = -G(beta,beta).
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(256) dyn_init_kernel(const WalkerDev* __restrict__ W) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!w.gt0 || sp >= w.S) return;
  const long long NN = (long long)w.N * w.N;
  const double* G = w.G + sp * NN;
  double* t0 = w.gt0 + sp * NN;  // parity slot 0 (t = 0)
  double* ot = w.g0t + sp * NN;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < NN; e += (long long)gridDim.x * 256) {
    const int r = (int)(e % w.N), c = (int)(e / w.N);
    t0[e] = G[e];
    ot[e] = G[e] - ((r == c) ? 1.0 : 0.0);
  }
}

// X1 = M^-1 (Dlmin F_L) with the LU factors and pivots left by lu_solve_general_kernel;
// thread per column of the right-hand side (row-major, coalesced across threads)
__global__ void __launch_bounds__(1024) dyn_resolve_kernel(const WalkerDev* __restrict__ W, int j) {
  const int wi = blockIdx.x >> 1, sp = blockIdx.x & 1;
  const WalkerDev& w = W[wi];
  if (!w.gt0 || w.ozstab || sp >= w.S || j >= w.nstack) return;  // tensor-core walkers: oz_greens
  const int N = w.N;
  const long long NN = (long long)N * N;
  const int nl = j + 1;  // forward step j: left stack holds j + 1 levels
  const double* lv = stack_level(w, 0, sp, nl - 1);
  const double* F = lv + NN;
  const double* D = lv + 2 * NN;
  const double* M = w.scr + sp * 2 * NN;  // LU factors, col-major
  const int* piv = w.dpiv + sp * N;
  double* X = w.dynx + sp * NN;  // row-major
  for (int c = threadIdx.x; c < N; c += blockDim.x) {
    for (int r = 0; r < N; ++r) X[(long long)r * N + c] = fmin(D[r], 1.0) * F[(long long)c * N + r];
    // the factorization swapped whole rows (multipliers included): all swaps first, then L and U
    for (int k = 0; k < N; ++k) {
      const int p = piv[k];
      if (p != k) {
        const double a = X[(long long)k * N + c];
        X[(long long)k * N + c] = X[(long long)p * N + c];
        X[(long long)p * N + c] = a;
      }
    }
    for (int k = 0; k < N; ++k) {
      const double yk = X[(long long)k * N + c];
      if (yk != 0.0)
        for (int r = k + 1; r < N; ++r) X[(long long)r * N + c] = fma(-M[(long long)k * N + r], yk, X[(long long)r * N + c]);
    }
    for (int k = N - 1; k >= 0; --k) {
      const double yk = X[(long long)k * N + c] / M[(long long)k * N + k];
      X[(long long)k * N + c] = yk;
      for (int r = 0; r < k; ++r) X[(long long)r * N + c] = fma(-M[(long long)k * N + r], yk, X[(long long)r * N + c]);
    }
  }
}

// t = beta (forward step nstack - 1): G(beta,0) = X1, G(0,beta) = -X, with their wrap errors
__global__ void __launch_bounds__(256) dyn_boundary_kernel(const WalkerDev* __restrict__ W, int j) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!w.gt0 || w.ozstab || sp >= w.S || j != w.nstack - 1) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  const int par = w.Lt & 1;
  double* t0 = w.gt0 + ((long long)par * w.S + sp) * NN;
  double* ot = w.g0t + ((long long)par * w.S + sp) * NN;
  const double* X1 = w.dynx + sp * NN;        // row-major
  const double* X = w.scr + sp * 2 * NN + NN;  // row-major
  double err = 0.0;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < NN; e += (long long)gridDim.x * 256) {
    const int r = (int)(e % N), c = (int)(e / N);
    const double a = X1[(long long)r * N + c], b = -X[(long long)r * N + c];
    err = fmax(err, fmax(fabs(a - t0[e]), fabs(b - ot[e])));
    t0[e] = a;
    ot[e] = b;
  }
  for (int o = 16; o > 0; o >>= 1) err = fmax(err, __shfl_xor_sync(0xffffffffu, err, o));
  if ((threadIdx.x & 31) == 0) atomicMax(w.wrap_bits, (unsigned long long)__double_as_longlong(err));
}

// G(k,tau) += sign / N sum_ij FF(r_j - r_i) (G_up(t,0)(j,i) + G_dn(t,0)(j,i)) / 2 at the listed tau
// (measure_greens_functions, src/measure/measure_methods.cpp:278-308).  phase 0: slices inside
// the interval (after propagation); 1: the interval's last slice (after stabilization);
// 2: tau = 0 from G(beta,beta) after the sweep.
__global__ void __launch_bounds__(256) dyn_measure_kernel(const WalkerDev* __restrict__ W, int j, int q, int phase) {
  const WalkerDev& w = W[blockIdx.x];
  if (!w.gt0 || j >= w.nstack) return;
  int t;
  if (phase == 2) {
    t = 0;
  } else {
    const int t_lo = j * w.pace + 1, t_hi = min((j + 1) * w.pace, w.Lt);
    if (phase == 0) {
      if (q >= t_hi - t_lo) return;  // the last slice of the interval is measured after stabilization
      t = t_lo + q;
    } else {
      t = t_hi;
    }
    if (t >= w.Lt) return;  // tau = beta is not measured
  }
  int slot = -1;
  for (int k = 0; k < w.dyn_ntau; ++k)
    if (w.dyn_taus[k] == t) slot = k;
  const int N = w.N, L = w.L, S = w.S;
  const long long NN = (long long)N * N;
  const double sg = *w.sign;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  extern __shared__ double dsh[];  // [L] cos(-r kx1), phase 2 also [N] e_i and [N] B_i
  __shared__ double red[8][4];
  // FourierFactor(r, 1) of the reference's k-star 1 = (2 pi / L, 0) on the site (r, 0)
  const double kx1 = (double)((L + 1) / 2 + 1) / L * 2 * M_PI - M_PI;
  for (int r = threadIdx.x; r < L; r += blockDim.x) dsh[r] = cos(-r * kx1);
  __syncthreads();
  if (slot >= 0) {
    // G(t,t), G(t,0), G(0,t); at tau = 0 the reference's index Lt-1: G(beta,beta), G(beta,0), G(0,beta)
    const int tb = (phase == 2) ? (w.Lt & 1) : (t & 1);
    const double* gtt[2] = {w.G, w.G + (S == 2 ? NN : 0)};
    const double* gt0[2] = {w.gt0 + (long long)tb * S * NN, w.gt0 + ((long long)tb * S + (S == 2)) * NN};
    const double* g0t[2] = {w.g0t + (long long)tb * S * NN, w.g0t + ((long long)tb * S + (S == 2)) * NN};
    // G(k,tau) and the density of states read G(beta,beta) at tau = 0 (Greentt(Lt-1))
    const double* gk[2] = {phase == 2 ? gtt[0] : gt0[0], phase == 2 ? gtt[1] : gt0[1]};
    double v = 0.0, tr = 0.0, cpart = 0.0, rcor = 0.0;
    // cubic lattice: G(k,tau) only; the stiffness is a square-lattice observable
    // (dqmc_initializer.cpp:233-237, measure_methods.cpp:350)
    if (w.dim == 3)
      for (int jj = wid; jj < N; jj += 8)
        for (int i = lane; i < N; i += 32)
          v += w.ff[site_disp(L, 3, i, jj)] * (gk[0][(long long)i * N + jj] + gk[1][(long long)i * N + jj]);
    for (int jj = wid; jj < N && w.dim == 2; jj += 8) {
      const int xj = jj % L, yj = jj / L;
      const int jpx = (xj + 1) % L + L * yj;
      for (int i = lane; i < N; i += 32) {
        const int xi = i % L, yi = i / L;
        int dx = xj - xi, dy = yj - yi;
        dx += (dx < 0) ? L : 0;
        dy += (dy < 0) ? L : 0;
        v += w.ff[dx + dy * L] * (gk[0][(long long)i * N + jj] + gk[1][(long long)i * N + jj]);  // G(jj, i)
        // correlated current-current term of the stiffness (i, jj): measure_methods.cpp:400-407
        const int ipx = (xi + 1) % L + L * yi;
        const double fq = dsh[dx] - dsh[dy];
        double c = 0.0;
        for (int sp = 0; sp < S; ++sp) {
          const double* a = g0t[sp];
          const double* b = gt0[sp];
          c += -a[(long long)jpx * N + ipx] * b[(long long)i * N + jj] + a[(long long)jpx * N + i] * b[(long long)ipx * N + jj] +
               a[(long long)jj * N + ipx] * b[(long long)i * N + jpx] - a[(long long)jj * N + i] * b[(long long)ipx * N + jpx];
        }
        rcor += fq * ((S == 1) ? 2.0 * c : c);
      }
    }
    // per-displacement sums S(r) = sum_i G(i + r, i) (both spins): G(k,tau) = sum_r cos(k r) S(r)
    for (int r = wid; r < N; r += 8) {
      const int rx = r % L, ry = r / L;
      double sr = 0.0;
      for (int i = lane; i < N; i += 32) {
        const int jj = (w.dim == 2) ? (i % L + rx) % L + L * ((i / L + ry) % L) : site_shift(L, 3, i, r);
        sr += gk[0][(long long)i * N + jj] + gk[1][(long long)i * N + jj];
      }
      sr = warp_sum_g(sr);
      if (lane == 0) w.dyn_r[(long long)slot * N + r] += sg * 0.5 * sr / N;
    }
    for (int i = threadIdx.x; i < N; i += blockDim.x) {
      const long long d = (long long)i * N + i;
      const int ipx = site_nn(L, i, 0);
      tr += gk[0][d] + gk[1][d];
      cpart += g0t[0][d] * gt0[0][d] + g0t[1][d] * gt0[1][d];
      // parts that wait for G(beta,beta): d_i of the spin susceptibility, A_i of the stiffness
      double* dv = w.dyn_vec + (long long)slot * 2 * N;
      dv[i] = (1.0 - gtt[0][d]) - (1.0 - gtt[1][d]);
      dv[N + i] = (gtt[0][(long long)ipx * N + i] - gtt[0][(long long)i * N + ipx]) +
                  (gtt[1][(long long)ipx * N + i] - gtt[1][(long long)i * N + ipx]);
    }
    v = warp_sum_g(v);
    tr = warp_sum_g(tr);
    cpart = warp_sum_g(cpart);
    rcor = warp_sum_g(rcor);
    if (lane == 0) {
      red[wid][0] = v;
      red[wid][1] = tr;
      red[wid][2] = cpart;
      red[wid][3] = rcor;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double tot[4] = {0.0, 0.0, 0.0, 0.0};
      for (int k = 0; k < 8; ++k)
        for (int m = 0; m < 4; ++m) tot[m] += red[k][m];
      w.dyn_sum[slot] += sg * 0.5 * tot[0] / N;
      w.dyn_cnt[slot] += 1;
      w.dyn_obs[slot * 3 + 0] += sg * 0.5 * tot[1] / N;
      w.dyn_part[slot * 2 + 0] = tot[2];
      w.dyn_part[slot * 2 + 1] = tot[3];
    }
  }
  if (phase != 2) return;
  // end of the half-sweep: g00 = G(beta,beta) completes the spin susceptibility and the
  // uncorrelated stiffness term of every listed tau (measure_methods.cpp:345-461)
  __syncthreads();
  double* e = dsh + L;
  double* B = e + N;
  for (int i = threadIdx.x; i < N; i += blockDim.x) {
    const long long d = (long long)i * N + i;
    const int ipx = site_nn(L, i, 0);
    const double* g0 = w.G;
    const double* g1 = w.G + (S == 2 ? NN : 0);
    e[i] = (1.0 - g0[d]) - (1.0 - g1[d]);
    B[i] = (g0[(long long)ipx * N + i] - g0[(long long)i * N + ipx]) + (g1[(long long)ipx * N + i] - g1[(long long)i * N + ipx]);
  }
  __syncthreads();
  for (int k = 0; k < w.dyn_ntau; ++k) {
    const double* dv = w.dyn_vec + (long long)k * 2 * N;
    double ch = 0.0, un = 0.0;
    for (int i = threadIdx.x; i < N; i += blockDim.x) ch += dv[i] * e[i];
    for (int jj = wid; jj < N && w.dim == 2; jj += 8) {
      const int xj = jj % L, yj = jj / L;
      for (int i = lane; i < N; i += 32) {
        int dx = xj - i % L, dy = yj - i / L;
        dx += (dx < 0) ? L : 0;
        dy += (dy < 0) ? L : 0;
        un += (dsh[dx] - dsh[dy]) * dv[N + jj] * B[i];
      }
    }
    ch = warp_sum_g(ch);
    un = warp_sum_g(un);
    if (lane == 0) {
      red[wid][0] = ch;
      red[wid][1] = un;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double c2 = 0.0, u2 = 0.0;
      for (int q2 = 0; q2 < 8; ++q2) {
        c2 += red[q2][0];
        u2 += red[q2][1];
      }
      const double n = (double)N;
      w.dyn_obs[k * 3 + 1] += 0.25 * sg / n * (c2 - w.dyn_part[k * 2 + 0]);
      if (w.dim == 2) w.dyn_obs[k * 3 + 2] += 0.25 * w.hop_t * w.hop_t * sg * (w.dyn_part[k * 2 + 1] - u2) / (n * n);
    }
    __syncthreads();
  }
}

// --------------------------------------------------------------------------
// host-side launchers for general walkers
// --------------------------------------------------------------------------
static dim3 gemm_grid(int maxN, int nw) {
  const int t = (maxN + kTile - 1) / kTile;
  return dim3(t, t, 2 * nw);
}

void mixed_wrap_fwd(const WalkerDev* W, int nw, int maxN, int j, int q, cudaStream_t st);
void mixed_wrap_bwd(const WalkerDev* W, int nw, int maxN, int j, int q, cudaStream_t st);
void mixed_chain(const WalkerDev* W, int nw, int maxN, int mode, int j, int q, cudaStream_t st);
void mixed_dynamic_prop(const WalkerDev* W, int nw, int maxN, int j, int q, cudaStream_t st);

void launch_metropolis_delayed(bool mixed, const WalkerDev* W, int nw, int mode, int j, int q, int maxN, int S_max,
                               int KD, int tc_flush, cudaStream_t st);
void launch_metropolis_sub(const WalkerDev* W, int nw, int mode, int j, int q, int maxN, int S_max, cudaStream_t st);
void launch_metropolis_sub_split(const WalkerDev* W, int nw, int mode, int j, int q, int maxN, int S_max,
                                 cudaStream_t st);

// One slice of general walkers in three launch groups (timed separately by the
// host): the dense products before the updates (forward wrap), the Metropolis
// updates with the fused measurement, and the products after them (B-chain
// step and backward wrap).
void general_slice_pre(int mode, const WalkerDev* W, int nw, int j, int q, int maxN, bool any_dense, bool any_cb,
                       bool mixed, cudaStream_t st) {
  if (mode != MODE_FWD) return;
  // in a mixed batch the dense products go through the tensor cores (kernels_ozaki.cu)
  const bool fp64_dense = any_dense && !mixed;
  const dim3 g = gemm_grid(maxN, nw);
  if (fp64_dense) {
    gemm_op_kernel<OP_WL_FWD><<<g, 256, 0, st>>>(W, mode, j, q, -1);
    gemm_op_kernel<OP_WR_FWD><<<g, 256, 0, st>>>(W, mode, j, q, -1);
  }
  if (any_dense && mixed) mixed_wrap_fwd(W, nw, maxN, j, q, st);
  if (any_cb) cb_general_kernel<<<2 * nw, 256, sizeof(double) * 2 * maxN, st>>>(W, mode, j, q, 0);
}

void general_slice_metro(int mode, const WalkerDev* W, int nw, int j, int q, int maxN, int measure, bool mixed,
                         int kd, int smax, int tc_flush, cudaStream_t st) {
  if (mode == MODE_INIT) return;
  const size_t met_sm = sizeof(double) * 6 * maxN + maxN + 16;
  if (mixed && tc_flush == 2) launch_metropolis_sub(W, nw, mode, j, q, maxN, smax, st);
  else if (mixed && tc_flush == 3) launch_metropolis_sub_split(W, nw, mode, j, q, maxN, smax, st);
  else if (kd > 0) launch_metropolis_delayed(mixed, W, nw, mode, j, q, maxN, smax, kd, tc_flush, st);
  else metropolis_general_kernel<<<nw, kMetroThreads, met_sm, st>>>(W, mode, j, q);
  if (measure) measure_general_kernel<<<nw, 256, sizeof(double) * 2 * maxN, st>>>(W, mode, j, q, 0);
}

void general_slice_post(int mode, const WalkerDev* W, int nw, int j, int q, int maxN, bool any_dense, bool any_cb,
                        bool mixed, cudaStream_t st) {
  const bool fp64_dense = any_dense && !mixed;
  const bool mixed_dense = any_dense && mixed;
  const dim3 g = gemm_grid(maxN, nw);
  const size_t cb_sm = sizeof(double) * 2 * maxN;
  if (fp64_dense) {
    if (mode == MODE_FWD) gemm_op_kernel<OP_CH_FWD><<<g, 256, 0, st>>>(W, mode, j, q, -1);
    else gemm_op_kernel<OP_CH_BWD><<<g, 256, 0, st>>>(W, mode, j, q, -1);
  }
  if (mixed_dense) mixed_chain(W, nw, maxN, mode, j, q, st);
  if (any_cb) cb_general_kernel<<<2 * nw, 256, cb_sm, st>>>(W, mode, j, q, mode == MODE_FWD ? 2 : 3);
  if (mode == MODE_BWD) {
    if (fp64_dense) {
      gemm_op_kernel<OP_WR_BWD><<<g, 256, 0, st>>>(W, mode, j, q, -1);
      gemm_op_kernel<OP_WL_BWD><<<g, 256, 0, st>>>(W, mode, j, q, -1);
    }
    if (mixed_dense) mixed_wrap_bwd(W, nw, maxN, j, q, st);
    if (any_cb) cb_general_kernel<<<2 * nw, 256, cb_sm, st>>>(W, mode, j, q, 1);
  }
}

// One slice of the dynamic half-sweep in three launch groups (timed apart by the host):
// the wrap; the G(t,0) and G(0,t) steps with the G(k,tau) measurement; the B-chain step.
// Dense walkers through the products (on the tensor cores for mixed walkers),
// checkerboard walkers through the plaquette passes.
void general_dynamic_wrap(const WalkerDev* W, int nw, int j, int q, int maxN, bool mixed, bool any_dense,
                          bool any_cb, cudaStream_t st) {
  const dim3 g = gemm_grid(maxN, nw);
  if (any_dense) {
    if (mixed) {
      mixed_wrap_fwd(W, nw, maxN, j, q, st);
    } else {
      gemm_op_kernel<OP_WL_FWD><<<g, 256, 0, st>>>(W, MODE_FWD, j, q, -1);
      gemm_op_kernel<OP_WR_FWD><<<g, 256, 0, st>>>(W, MODE_FWD, j, q, -1);
    }
  }
  if (any_cb) cb_general_kernel<<<2 * nw, 256, sizeof(double) * 2 * maxN, st>>>(W, MODE_FWD, j, q, 0);
}

void general_dynamic_prop(const WalkerDev* W, int nw, int j, int q, int maxN, bool mixed, bool any_dense,
                          bool any_cb, cudaStream_t st) {
  const dim3 g = gemm_grid(maxN, nw);
  if (any_dense) {
    if (mixed) {
      mixed_dynamic_prop(W, nw, maxN, j, q, st);
    } else {
      gemm_op_kernel<OP_DT0><<<g, 256, 0, st>>>(W, MODE_FWD, j, q, -1);
      gemm_op_kernel<OP_D0T><<<g, 256, 0, st>>>(W, MODE_FWD, j, q, -1);
    }
  }
  if (any_cb) cb_general_kernel<<<2 * nw, 256, sizeof(double) * 2 * maxN, st>>>(W, MODE_FWD, j, q, 4);
  dyn_measure_kernel<<<nw, 256, sizeof(double) * 32, st>>>(W, j, q, 0);
}

void general_dynamic_chain(const WalkerDev* W, int nw, int j, int q, int maxN, bool mixed, bool any_dense,
                           bool any_cb, cudaStream_t st) {
  const dim3 g = gemm_grid(maxN, nw);
  if (any_dense) {
    if (mixed) mixed_chain(W, nw, maxN, MODE_FWD, j, q, st);
    else gemm_op_kernel<OP_CH_FWD><<<g, 256, 0, st>>>(W, MODE_FWD, j, q, -1);
  }
  if (any_cb) cb_general_kernel<<<2 * nw, 256, sizeof(double) * 2 * maxN, st>>>(W, MODE_FWD, j, q, 2);
}

// stabilization of the dynamic pieces after general_greens of forward step j (walkers
// stabilized by the tensor-core blocked QR get theirs from oz_greens)
void general_dynamic_stab(const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st) {
  const dim3 g = gemm_grid(maxN, nw);
  const int threads = std::min(1024, ((maxN + 31) / 32) * 32);
  dyn_resolve_kernel<<<2 * nw, threads, 0, st>>>(W, j);
  gemm_op_kernel<OP_DT0_OUT><<<g, 256, 0, st>>>(W, MODE_FWD, j, 0, -1);
  gemm_op_kernel<OP_D0T_OUT><<<g, 256, 0, st>>>(W, MODE_FWD, j, 0, -1);
  dyn_boundary_kernel<<<dim3(64, 2 * nw), 256, 0, st>>>(W, j);
}
// G(k,tau) measurement at the stabilization slice of forward step j (after both paths)
void general_dynamic_stab_measure(const WalkerDev* W, int nw, int j, cudaStream_t st) {
  dyn_measure_kernel<<<nw, 256, sizeof(double) * 32, st>>>(W, j, 0, 1);
}

void general_dynamic_begin(const WalkerDev* W, int nw, cudaStream_t st) {
  dyn_init_kernel<<<dim3(64, 2 * nw), 256, 0, st>>>(W);
}
void general_dynamic_end(const WalkerDev* W, int nw, int maxN, cudaStream_t st) {
  dyn_measure_kernel<<<nw, 256, sizeof(double) * (32 + 2 * maxN), st>>>(W, 0, 0, 2);
}

cudaError_t configure_general_kernels() {
  cudaError_t e;
  const int met = (int)(sizeof(double) * 6 * kMaxN + kMaxN + 16);
  if ((e = cudaFuncSetAttribute(metropolis_general_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, met))) return e;
  return cudaSuccess;
}

void general_chain_init(int mode, const WalkerDev* W, int nw, int j, cudaStream_t st) {
  chain_init_general_kernel<<<dim3(64, 2 * nw), 256, 0, st>>>(W, mode, j);
}

void general_push(int mode, const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st) {
  const int threads = ((maxN + 31) / 32) * 32;
  push_general_kernel<<<2 * nw, threads, sizeof(double) * 5 * maxN + sizeof(int) * maxN, st>>>(W, mode, j);
}

void general_greens(int mode, const WalkerDev* W, int nw, int j, int trace_slot, int maxN, cudaStream_t st) {
  const dim3 g = gemm_grid(maxN, nw);
  // general case needs M from the two GEMMs; boundary cases skip them (kernels exit)
  if (mode != MODE_INIT) {
    gemm_op_kernel<OP_GA><<<g, 256, 0, st>>>(W, mode, j, 0, -1);
    gemm_op_kernel<OP_GB><<<g, 256, 0, st>>>(W, mode, j, 0, -1);
  }
  greens_prep_general_kernel<<<dim3(64, 2 * nw), 256, 0, st>>>(W, mode, j);
  const int threads = std::min(1024, ((maxN + 31) / 32) * 32);
  lu_solve_general_kernel<<<2 * nw, threads, sizeof(double) * maxN, st>>>(W, mode, j);
  if (mode != MODE_INIT) gemm_op_kernel<OP_GG><<<g, 256, 0, st>>>(W, mode, j, 0, trace_slot);
  greens_out_general_kernel<<<dim3(64, 2 * nw), 256, 0, st>>>(W, mode, j, trace_slot);
}

void general_measure_after(int mode, const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st) {
  measure_general_kernel<<<nw, 256, sizeof(double) * 2 * maxN, st>>>(W, mode, j, 0, 1);
}

void general_sign(const WalkerDev* W, int nw, int maxN, cudaStream_t st) {
  sign_general_kernel<<<nw, 1024, sizeof(double) * maxN, st>>>(W);
}

}  // namespace dqmc
