// kernels_delayed.cu — Metropolis with delayed rank-k updates for walkers
// whose G lives in HBM/L2 (the HBM FP64 path and the mixed path).
//
// The reference applies each accepted flip at once as a rank-1 update
// (update_greens_function, src/model/repulsive_hubbard.cpp:127-155):
//     G <- G - u w^T,  u = f G(:,i),  w = e_i - G(i,:)^T.
// Here G0 (HBM) is held fixed while up to k accepted flips accumulate as
// columns of U and V in shared memory, G_cur = G0 - U V^T:
//     u = f (G0(:,i) - U V(i,:)^T),  w = e_i - (G0(i,:) - U(i,:) V^T)^T,
// the corrected diagonal is kept up to date per accept (one FMA per site),
// and every k accepts (and at the end of the slice) G0 <- G0 - U V^T is
// applied as one dense product: register-light FP64 on the plain path, the
// exact-slice BF16 tensor-core product on the mixed path.  The decisions are
// the reference's (same ratio, same uniform per site); only the order in which
// the flips reach G changes, so G agrees with sequential rank-1 updates to
// rounding.
#include <cuda_runtime.h>

#include <cstdint>

#include "dqmc_device.cuh"
#include "ozaki.cuh"

namespace dqmc {

namespace {

__device__ __forceinline__ bool d_slice_of(const WalkerDev& w, int mode, int j, int q, int& t) {
  if (j >= w.nstack) return false;
  const int k = (mode == MODE_FWD) ? j : (w.nstack - 1 - j);
  const int t_lo = k * w.pace + 1, t_hi = min((k + 1) * w.pace, w.Lt);
  if (q >= t_hi - t_lo + 1) return false;
  t = (mode == MODE_FWD) ? t_lo + q : t_hi - q;
  return true;
}

constexpr int kDelThreads = 256;
constexpr int kTileRow = 64;  // flush tile edge

}  // namespace

// shared-memory bytes of the delayed kernel for (N, S, KD)
__host__ __device__ inline size_t delayed_smem_bytes(int N, int S, int KD) {
  const size_t uv = 2ull * S * N * (KD + 1) * sizeof(double);
  const size_t dc = (size_t)S * N * sizeof(double);
  const size_t tiles = 2ull * 6 * kTileRow * (KD + 8) * sizeof(unsigned short);
  return uv + dc + tiles + (size_t)N + 64;
}

// largest k in {32, 16, 8} that fits the shared-memory budget
int delayed_pick_kd(int N, int S) {
  for (int kd : {32, 16, 8})
    if (delayed_smem_bytes(N, S, kd) <= 200 * 1024) return kd;
  return 0;
}

// ---- the G0 -= U V^T flush ---------------------------------------------------
__device__ void flush_fp64(double* G0, int N, const double* U, const double* V, int ldu, int M) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c = wid; c < N; c += kDelThreads / 32) {
    const double* vc = V + (long long)c * ldu;
    double* gc = G0 + (long long)c * N;
    for (int r = lane; r < N; r += 32) {
      const double* ur = U + (long long)r * ldu;
      double a0 = 0.0, a1 = 0.0;
      int m = 0;
      for (; m + 1 < M; m += 2) {
        a0 = fma(ur[m], vc[m], a0);
        a1 = fma(ur[m + 1], vc[m + 1], a1);
      }
      if (m < M) a0 = fma(ur[m], vc[m], a0);
      gc[r] -= a0 + a1;
    }
  }
}

// tensor-core flush: 64 x 64 tiles, K = KD (stale columns m >= M are zeroed by the caller)
__device__ void flush_ozaki(double* G0, int N, const double* U, const double* V, int ldu, int KD,
                            unsigned short* tA, unsigned short* tB, int* eA, int* eB) {
  constexpr int S = 6, B = 7;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int wm = wid >> 2, wn = wid & 3, g = lane >> 2, t4 = lane & 3;
  const int ldt = KD + 8;  // padded tile row (BF16)
  for (int r0 = 0; r0 < N; r0 += kTileRow)
    for (int c0 = 0; c0 < N; c0 += kTileRow) {
      // exponents of the 64 rows of U (A operand) and 64 rows of V (columns of V^T, B operand)
      if (tid < 2 * kTileRow) {
        const int op = tid >> 6, l = tid & 63;
        const int row = (op == 0 ? r0 : c0) + l;
        int e = -1100;
        if (row < N) {
          const double* src = (op == 0 ? U : V) + (long long)row * ldu;
          for (int m = 0; m < KD; ++m) e = max(e, ozaki::exp_bound(src[m]));
        }
        (op == 0 ? eA : eB)[l] = e;
      }
      __syncthreads();
      for (int e2 = tid; e2 < 2 * kTileRow * KD; e2 += kDelThreads) {
        const int op = e2 / (kTileRow * KD), rem = e2 % (kTileRow * KD);
        const int l = rem / KD, m = rem % KD;
        const int row = (op == 0 ? r0 : c0) + l;
        const double x = (row < N) ? (op == 0 ? U : V)[(long long)row * ldu + m] : 0.0;
        bool neg;
        const unsigned long long qv = ozaki::fixed42(x, (op == 0 ? eA : eB)[l], neg);
        unsigned short* dst = (op == 0 ? tA : tB);
        for (int s = 0; s < S; ++s) dst[(s * kTileRow + l) * ldt + m] = ozaki::slice_bf16(qv, s, B, neg);
      }
      __syncthreads();
      float acc[S][2][2][4];
#pragma unroll
      for (int m = 0; m < S; ++m)
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
          for (int b = 0; b < 2; ++b)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[m][a][b][v] = 0.f;
      for (int k0 = 0; k0 < KD; k0 += 16) {
#pragma unroll
        for (int i = 0; i < S; ++i) {
          unsigned a[2][4];
#pragma unroll
          for (int mt = 0; mt < 2; ++mt) {
            const unsigned short* p = tA + (i * kTileRow + wm * 32 + mt * 16 + g) * ldt + k0 + 2 * t4;
            a[mt][0] = *(const unsigned*)(p);
            a[mt][1] = *(const unsigned*)(p + 8 * ldt);
            a[mt][2] = *(const unsigned*)(p + 8);
            a[mt][3] = *(const unsigned*)(p + 8 * ldt + 8);
          }
#pragma unroll
          for (int jj = 0; jj < S - i; ++jj) {
            unsigned b[2][2];
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
              const unsigned short* p = tB + (jj * kTileRow + wn * 16 + nt * 8 + g) * ldt + k0 + 2 * t4;
              b[nt][0] = *(const unsigned*)(p);
              b[nt][1] = *(const unsigned*)(p + 8);
            }
#pragma unroll
            for (int mt = 0; mt < 2; ++mt)
#pragma unroll
              for (int nt = 0; nt < 2; ++nt)
                ozaki::mma16816(acc[i + jj][mt][nt], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b[nt][0], b[nt][1]);
          }
        }
      }
#pragma unroll
      for (int mt = 0; mt < 2; ++mt)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
          for (int v = 0; v < 4; ++v) {
            const int rl = wm * 32 + mt * 16 + g + ((v >> 1) << 3), cl = wn * 16 + nt * 8 + 2 * t4 + (v & 1);
            const int r = r0 + rl, c = c0 + cl;
            if (r >= N || c >= N) continue;
            long long s = 0;
#pragma unroll
            for (int m = 0; m < S; ++m) s = (s << B) + (long long)ozaki::f2i_small(acc[m][mt][nt][v]);
            if (s != 0) G0[(long long)c * N + r] -= ozaki::ldexp_i64(s, eA[rl] + eB[cl] - B * (S + 1));
          }
      __syncthreads();
    }
}

// --------------------------------------------------------------------------
// One slice of Metropolis for general walkers.  One CTA per walker.
// --------------------------------------------------------------------------
template <bool MIXED>
__global__ void __launch_bounds__(kDelThreads) metropolis_delayed_kernel(const WalkerDev* __restrict__ W, int mode,
                                                                        int j, int q, int KD, int tc_flush) {
  const WalkerDev& w = W[blockIdx.x];
  if (w.path == 0 || (MIXED != (w.path == 2))) return;
  int t;
  if (!d_slice_of(w, mode, j, q, t)) return;
  const int N = w.N, S = w.S, Lt = w.Lt, ldu = KD + 1;
  const long long NN = (long long)N * N;
  extern __shared__ double sh[];
  double* U = sh;                                   // [S][N][ldu]
  double* V = U + (long long)S * N * ldu;           // [S][N][ldu]
  double* dcur = V + (long long)S * N * ldu;        // [S][N] diagonal of G_cur
  unsigned short* tA = (unsigned short*)(dcur + (long long)S * N);
  unsigned short* tB = tA + 6 * kTileRow * (KD + 8);
  int8_t* s_field = (int8_t*)(tB + 6 * kTileRow * (KD + 8));
  __shared__ int s_next;
  __shared__ double s_f[2];
  __shared__ int eA[kTileRow], eB[kTileRow];
  double* G0[2] = {w.G, (S == 2) ? w.G + NN : w.G};
  const int eff = t - 1;
  for (int i = threadIdx.x; i < N; i += kDelThreads) {
    s_field[i] = w.fields[(long long)eff * N + i];
    for (int sp = 0; sp < S; ++sp) dcur[sp * N + i] = G0[sp][(long long)i * N + i];
  }
  double sign = *w.sign;
  long long acc_count = 0;
  const unsigned long long sweep = (w.rng == 1) ? *w.sweep_ctr : 0ULL;
  __syncthreads();

  int M = 0;  // pending columns of U, V
  auto flush = [&]() {
    if (M == 0) return;
    if (MIXED && tc_flush && KD >= 16) {
      // zero the stale columns m >= M so the K = KD product sees only the pending block
      for (int sp = 0; sp < S; ++sp)
        for (int e = threadIdx.x; e < N * (KD - M); e += kDelThreads) {
          const int r = e / (KD - M), m = M + e % (KD - M);
          U[((long long)sp * N + r) * ldu + m] = 0.0;
          V[((long long)sp * N + r) * ldu + m] = 0.0;
        }
      __syncthreads();
      for (int sp = 0; sp < S; ++sp)
        flush_ozaki(G0[sp], N, U + (long long)sp * N * ldu, V + (long long)sp * N * ldu, ldu, KD, tA, tB, eA, eB);
    } else {
      for (int sp = 0; sp < S; ++sp)
        flush_fp64(G0[sp], N, U + (long long)sp * N * ldu, V + (long long)sp * N * ldu, ldu, M);
    }
    __syncthreads();
    M = 0;
  };

  auto decide_from = [&](int i0) {
    for (int i = i0; i < N; ++i) {
      const int s = s_field[i];
      const int si = s > 0 ? 0 : 1;
      const double gu = dcur[i];
      const double gd = (S == 2) ? dcur[N + i] : gu;
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

  int cur = 0;
  while (true) {
    if (threadIdx.x == 0) s_next = decide_from(cur);
    __syncthreads();
    const int i = s_next;
    if (i >= N) break;
    // new columns u (of U) and w (of V) from G_cur = G0 - U V^T
    for (int r = threadIdx.x; r < N; r += kDelThreads) {
      for (int sp = 0; sp < S; ++sp) {
        const double* Us = U + (long long)sp * N * ldu;
        const double* Vs = V + (long long)sp * N * ldu;
        double gri = G0[sp][(long long)i * N + r];  // G0(r, i)
        double gir = G0[sp][(long long)r * N + i];  // G0(i, r)
        const double* ur = Us + (long long)r * ldu;
        const double* ui = Us + (long long)i * ldu;
        const double* vr = Vs + (long long)r * ldu;
        const double* vi = Vs + (long long)i * ldu;
        for (int m = 0; m < M; ++m) {
          gri = fma(-ur[m], vi[m], gri);
          gir = fma(-ui[m], vr[m], gir);
        }
        const double uu = s_f[sp] * gri;
        const double ww = ((r == i) ? 1.0 : 0.0) - gir;
        // column M is written here; rows i of U/V are read above only for m < M
        dcur[sp * N + r] = fma(-uu, ww, dcur[sp * N + r]);
        ((double*)Us)[(long long)r * ldu + M] = uu;
        ((double*)Vs)[(long long)r * ldu + M] = ww;
      }
    }
    __syncthreads();
    ++M;
    cur = i + 1;
    if (M == KD) flush();
  }
  flush();

  int8_t* frw = w.fields + (long long)eff * N;
  for (int i = threadIdx.x; i < N; i += kDelThreads) frw[i] = s_field[i];
  if (threadIdx.x == 0) {
    *w.sign = sign;
    *w.accepts += acc_count;
    if (mode == MODE_BWD && t == Lt) *w.sign_Lt = sign;
  }
}

// dynamic shared memory limit = device opt-in maximum minus the kernel's static part
template <class K>
static cudaError_t allow_max_smem(K kernel) {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa{};
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, kernel);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - (int)fa.sharedSizeBytes);
  return e;
}

cudaError_t configure_delayed_kernels() {
  cudaError_t e;
  if ((e = allow_max_smem(metropolis_delayed_kernel<false>))) return e;
  if ((e = allow_max_smem(metropolis_delayed_kernel<true>))) return e;
  return cudaSuccess;
}

void launch_metropolis_delayed(bool mixed, const WalkerDev* W, int nw, int mode, int j, int q, int maxN, int S_max,
                               int KD, int tc_flush, cudaStream_t st) {
  const size_t sm = delayed_smem_bytes(maxN, S_max, KD);
  if (mixed) metropolis_delayed_kernel<true><<<nw, kDelThreads, sm, st>>>(W, mode, j, q, KD, tc_flush);
  else metropolis_delayed_kernel<false><<<nw, kDelThreads, sm, st>>>(W, mode, j, q, KD, 0);
}

}  // namespace dqmc
