// kernels_submatrix.cu — Metropolis of one time slice for walkers on the
// tensor-core path, by submatrix updates.
//
// The reference visits the N sites of slice t in order (metropolis_update,
// src/dqmc_walker.cpp:173-197) and applies every accepted flip at once to the
// whole N x N Green's function as a rank-1 update (update_greens_function,
// src/model/repulsive_hubbard.cpp:127-155, attractive_hubbard.cpp:128-157):
//     G <- G - u w^T,   u = f G(:,i),   w = e_i - G(i,:)^T,   f = Delta / ratio.
// On GB300 that costs 2 N^2 FP64 operations per accepted flip on a pipe that
// runs at 1/64 of the FP32 rate.  Here the sites are taken in blocks I of 32.
// Inside a block the decisions need only the 32 x 32 diagonal block G(I,I),
// which is kept current flip by flip with the same rank-1 formula.  The m
// accepted flips of the block (positions l_1 < ... < l_m) are recorded in
// coefficient form, u_q = G0(:,I_A) a_q and w_q = R_A^T b_q with
//     a_q = f_q (e_q - sum_{p<q} w~_p(l_q) a_p),   b_q = e_q + sum_{p<q} u~_p(l_q) b_p,
// where u~_p, w~_p are u_p, w_p on the block and R_A = E_A^T - G0(I_A,:).
// After the block
//     G = G0 - G0(:,I_A) Gamma R_A,   Gamma = sum_q a_q b_q^T   (m x m),
// the Sherman-Morrison-Woodbury form of the m flips, applied as two products
// on the BF16 tensor cores through exact 42-bit integer slices (ozaki.cuh; K <= 32 per flush):
// T = Gamma R_A (m x N), then G -= G0(:,I_A) T (N x N, K = m).
//
// The decisions use the reference's ratio formula, evaluated with the same
// rounded operations, and the same uniform per site; G reaches them through
// a different but equivalent sequence of updates, so they agree with the
// reference's unless a ratio lies within rounding of its uniform.
#include <cuda_runtime.h>

#include <cstdint>

#include "dqmc_device.cuh"
#include "ozaki.cuh"

namespace dqmc {

namespace {

constexpr int kSubThreads = 256;
constexpr int KB = 32;           // sites per block
constexpr int KK = KB * KB;
constexpr int KP = KB + 8;       // padded BF16 row of a slice tile (80 bytes)
constexpr int OZS = 6, OZB = 7;  // 6 slices of 7 bits; group sums < 2^22 for K <= 32

__host__ __device__ inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// per-spin scratch in HBM (WalkerDev::msub)
struct SubOff {
  size_t T, sT, sG, eT, eG, total;
};
__host__ __device__ inline SubOff sub_offsets(int N) {
  SubOff o;
  o.T = 0;                                                          // T(x, c) at c * KB + x
  o.sT = al256((size_t)N * KB * sizeof(double));                    // slices of T, lines = columns c
  o.sG = o.sT + al256((size_t)OZS * N * KP * sizeof(unsigned short));  // slices of G0(:, I_A), lines = rows
  o.eT = o.sG + al256((size_t)OZS * N * KP * sizeof(unsigned short));
  o.eG = o.eT + al256((size_t)N * sizeof(int));
  o.total = o.eG + al256((size_t)N * sizeof(int));
  return o;
}

__device__ __forceinline__ bool sub_slice_of(const WalkerDev& w, int mode, int j, int q, int& t) {
  if (j >= w.nstack) return false;
  const int k = (mode == MODE_FWD) ? j : (w.nstack - 1 - j);
  const int t_lo = k * w.pace + 1, t_hi = min((k + 1) * w.pace, w.Lt);
  if (q >= t_hi - t_lo + 1) return false;
  t = (mode == MODE_FWD) ? t_lo + q : t_hi - q;
  return true;
}

__device__ __forceinline__ void cp16(void* dst, const void* src, bool pred) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  const int n = pred ? 16 : 0;  // 0: zero-fill, nothing is read
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(n));
}

// Slices nlines lines x K (<= KB) of an operand into dst[s][line][KP] with one
// exponent per line (ex[line]); get(line, k) is the FP64 element.  Lines of a
// 64-line chunk past nlines (up to dst_lines) are written as zeros.  All
// threads take part; 4 threads per line, 8 k each.
template <class Get>
__device__ void slice_lines(Get get, int nlines, int K, unsigned short* dst, int dst_lines, int* ex, int* etmp) {
  const int tid = threadIdx.x, ll = tid & 63, part = tid >> 6;
  for (int l0 = 0; l0 < nlines; l0 += 64) {
    const int line = l0 + ll;
    double v[8];
    int e = -1100;
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int k = part * 8 + u;
      v[u] = (line < nlines && k < K) ? get(line, k) : 0.0;
      e = max(e, ozaki::exp_bound(v[u]));
    }
    etmp[part * 64 + ll] = e;
    __syncthreads();
    e = max(max(etmp[ll], etmp[64 + ll]), max(etmp[128 + ll], etmp[192 + ll]));
    if (line < dst_lines) {
      if (part == 0) ex[line] = e;
      unsigned pk[OZS][4];
#pragma unroll
      for (int u = 0; u < 8; u += 2) {
        bool n0, n1;
        const unsigned long long q0 = ozaki::fixed42(v[u], e, n0), q1 = ozaki::fixed42(v[u + 1], e, n1);
#pragma unroll
        for (int s = 0; s < OZS; ++s)
          pk[s][u >> 1] = (unsigned)ozaki::slice_bf16(q0, s, OZB, n0) |
                          ((unsigned)ozaki::slice_bf16(q1, s, OZB, n1) << 16);
      }
#pragma unroll
      for (int s = 0; s < OZS; ++s)
        *reinterpret_cast<uint4*>(dst + ((long long)s * dst_lines + line) * KP + part * 8) =
            make_uint4(pk[s][0], pk[s][1], pk[s][2], pk[s][3]);
    }
    __syncthreads();
  }
}

// 64 x 64 product tile, K = 32, from sa[s][row][KP] and sb[s][col][KP]: weight groups in acc
__device__ __forceinline__ void mma_tile(const unsigned short* sa, const unsigned short* sb,
                                         float (&acc)[OZS][2][2][4]) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int wm = wid >> 2, wn = wid & 3, g = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int m = 0; m < OZS; ++m)
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[m][a][b][v] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < KB; k0 += 16) {
#pragma unroll
    for (int i = 0; i < OZS; ++i) {
      unsigned a[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const unsigned short* p = sa + (i * 64 + wm * 32 + mt * 16 + g) * KP + k0 + 2 * t4;
        a[mt][0] = *(const unsigned*)(p);
        a[mt][1] = *(const unsigned*)(p + 8 * KP);
        a[mt][2] = *(const unsigned*)(p + 8);
        a[mt][3] = *(const unsigned*)(p + 8 * KP + 8);
      }
#pragma unroll
      for (int jj = 0; jj < OZS - i; ++jj) {
        unsigned b[2][2];
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
          const unsigned short* p = sb + (jj * 64 + wn * 16 + nt * 8 + g) * KP + k0 + 2 * t4;
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
}

// calls f(rl, cl, v, e_offset) for this thread's 16 elements of a 64 x 64 tile;
// value = v * 2^(eA[rl] + eB[cl] + e_offset)
template <class F>
__device__ __forceinline__ void tile_epilogue(const float (&acc)[OZS][2][2][4], F f) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int wm = wid >> 2, wn = wid & 3, g = lane >> 2, t4 = lane & 3;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int rl = wm * 32 + mt * 16 + g + ((v >> 1) << 3), cl = wn * 16 + nt * 8 + 2 * t4 + (v & 1);
        long long s = 0;
#pragma unroll
        for (int m = 0; m < OZS; ++m) s = (s << OZB) + (long long)ozaki::f2i_small(acc[m][mt][nt][v]);
        f(rl, cl, s);
      }
}

constexpr int kEOff = -OZB * (OZS + 1);

}  // namespace

size_t submatrix_scratch_bytes(int N) { return sub_offsets(N).total; }

// nbuf: flush tile buffers (2 overlaps the copies of tile i+1 with tile i)
size_t submatrix_smem_bytes(int N, int S, int nbuf) {
  const size_t Nu = (size_t)((N + 1) & ~1);
  return sizeof(double) * (Nu + 6ull * S * KK) + 2ull * nbuf * OZS * 64 * KP * sizeof(unsigned short) +
         256 * sizeof(int) + (size_t)N;
}

__global__ void __launch_bounds__(kSubThreads) metropolis_sub_kernel(const WalkerDev* __restrict__ W, int mode, int j,
                                                                     int q, int nbuf) {
  const WalkerDev& w = W[blockIdx.x];
  if (w.path != 2) return;
  int t;
  if (!sub_slice_of(w, mode, j, q, t)) return;
  const int N = w.N, S = w.S, Lt = w.Lt, tid = threadIdx.x;
  const long long NN = (long long)N * N;
  extern __shared__ __align__(16) double sh[];
  double* uni = sh;                      // [N] uniforms of the slice
  double* Gb = uni + ((N + 1) & ~1);     // [S][KK] diagonal block, (r, c) at c * KB + r
  double* Ac = Gb + S * KK;              // [S][q][x] a_q at compact index x
  double* Bc = Ac + S * KK;              // [S][q][x] b_q
  double* Ut = Bc + S * KK;              // [S][q][l] u~_q at block position l
  double* Wt = Ut + S * KK;              // [S][q][l] w~_q
  double* Gam = Wt + S * KK;             // [S][KK] Gamma(x, y) at y * KB + x
  unsigned short* sa = reinterpret_cast<unsigned short*>(Gam + S * KK);  // [nbuf][6][64][KP] left operand tiles
  unsigned short* sb = sa + nbuf * OZS * 64 * KP;                         // [nbuf][6][64][KP] right operand tiles
  int* etmp = reinterpret_cast<int*>(sb + nbuf * OZS * 64 * KP);  // [256]
  int8_t* s_field = reinterpret_cast<int8_t*>(etmp + 256);  // [N]
  __shared__ int eA[64], eB[64];
  __shared__ int fA[2][64], fB[2][64];  // exponents of the flush tiles (per buffer)
  __shared__ int s_next, s_pos[KB];
  __shared__ double s_f[2];

  const SubOff so = sub_offsets(N);
  double* G[2] = {w.G, (S == 2) ? w.G + NN : w.G};
  const int eff = t - 1;
  const unsigned long long sweep = (w.rng == 1) ? *w.sweep_ctr : 0ULL;
  for (int i = tid; i < N; i += kSubThreads) {
    s_field[i] = w.fields[(long long)eff * N + i];
    const int attempt = (mode == MODE_FWD) ? (eff * N + i) : ((Lt - t) * N + i);
    uni[i] = (w.rng == 0) ? w.uni[attempt] : philox_uniform(w.seed, blockIdx.x, sweep, (unsigned)(eff * N + i));
  }
  double sign = 0.0;
  long long acc_count = 0;
  if (tid == 0) sign = *w.sign;
  __syncthreads();

  for (int i0 = 0; i0 < N; i0 += KB) {
    const int kb = min(KB, N - i0);
    for (int e = tid; e < S * KK; e += kSubThreads) {
      const int sp = e / KK, c = (e % KK) / KB, r = e % KB;
      Gb[e] = (r < kb && c < kb) ? G[sp][(long long)(i0 + c) * N + i0 + r] : 0.0;
    }
    __syncthreads();

    // ---- decisions, flip by flip, on the diagonal block
    int m = 0, cur = 0;
    while (true) {
      if (tid == 0) {
        int l = cur;
        for (; l < kb; ++l) {
          const int i = i0 + l;
          const int s = s_field[i];
          const int si = s > 0 ? 0 : 1;
          const double gu = Gb[l * KB + l];
          const double gd = (S == 2) ? Gb[KK + l * KB + l] : gu;
          const double cu = w.cm[si];
          const double cd = (w.model == 0) ? w.cp[si] : w.cm[si];
          const double ru = __dadd_rn(1.0, __dmul_rn(__dsub_rn(1.0, gu), cu));
          const double rd = __dadd_rn(1.0, __dmul_rn(__dsub_rn(1.0, gd), cd));
          const double r = (w.model == 0) ? __dmul_rn(ru, rd) : __dmul_rn(__dmul_rn(w.ex2[si], ru), rd);
          const double prob = fmin(1.0, fabs(r));
          if (!isfinite(r)) atomicOr(w.status, ST_NONFINITE_RATIO);
          if (uni[i] < prob) {
            s_f[0] = __ddiv_rn(cu, ru);
            s_f[1] = (w.model == 0) ? __ddiv_rn(cd, rd) : s_f[0];
            s_field[i] = (int8_t)(-s);
            sign = (r >= 0) ? sign : -sign;
            ++acc_count;
            break;
          }
        }
        s_next = l;
      }
      __syncthreads();
      const int l = s_next;
      if (l >= kb) break;
      // u~, w~ of accept m on the block, and its coefficients a_m, b_m
      for (int e = tid; e < S * 4 * KB; e += kSubThreads) {
        const int sp = e / (4 * KB), role = (e / KB) & 3, x = e % KB;
        const double f = s_f[sp];
        const double* gb = Gb + sp * KK;
        double* ut = Ut + sp * KK;
        double* wt = Wt + sp * KK;
        double* ac = Ac + sp * KK;
        double* bc = Bc + sp * KK;
        if (role == 0) {
          ut[m * KB + x] = f * gb[l * KB + x];  // f G(x, l)
        } else if (role == 1) {
          wt[m * KB + x] = ((x == l) ? 1.0 : 0.0) - gb[x * KB + l];  // delta - G(l, x)
        } else if (role == 2) {
          double a = (x == m) ? 1.0 : 0.0;
          for (int p = x; p < m; ++p) a = fma(-wt[p * KB + l], ac[p * KB + x], a);
          ac[m * KB + x] = (x <= m) ? f * a : 0.0;
        } else {
          double b = (x == m) ? 1.0 : 0.0;
          for (int p = x; p < m; ++p) b = fma(ut[p * KB + l], bc[p * KB + x], b);
          bc[m * KB + x] = (x <= m) ? b : 0.0;
        }
      }
      if (tid == 0) s_pos[m] = l;
      __syncthreads();
      // rank-1 update of the part of the block later decisions read
      for (int e = tid; e < S * KK; e += kSubThreads) {
        const int sp = e / KK, c = (e % KK) / KB, r = e % KB;
        if (r > l && c > l && r < kb && c < kb)
          Gb[e] = fma(-Ut[sp * KK + m * KB + r], Wt[sp * KK + m * KB + c], Gb[e]);
      }
      ++m;
      cur = l + 1;
      __syncthreads();
    }
    if (m == 0) continue;

    // ---- Gamma = sum_q a_q b_q^T
    for (int e = tid; e < S * KK; e += kSubThreads) {
      const int sp = e / KK, y = (e % KK) / KB, x = e % KB;
      double gsum = 0.0;
      if (x < m && y < m) {
        const double* ac = Ac + sp * KK;
        const double* bc = Bc + sp * KK;
        for (int p = max(x, y); p < m; ++p) gsum = fma(ac[p * KB + x], bc[p * KB + y], gsum);
      }
      Gam[e] = gsum;
    }
    __syncthreads();

    for (int sp = 0; sp < S; ++sp) {
      unsigned char* ms = w.msub + (size_t)sp * so.total;
      double* Tg = reinterpret_cast<double*>(ms + so.T);
      unsigned short* sT = reinterpret_cast<unsigned short*>(ms + so.sT);
      unsigned short* sG = reinterpret_cast<unsigned short*>(ms + so.sG);
      int* eT = reinterpret_cast<int*>(ms + so.eT);
      int* eG = reinterpret_cast<int*>(ms + so.eG);
      const double* gam = Gam + sp * KK;
      double* Gs = G[sp];
      // Gamma as the left operand (lines = rows x, k = y)
      slice_lines([&](int line, int k) { return gam[k * KB + line]; }, m, m, sa, 64, eA, etmp);
      // G0(:, I_A) as the left operand of the flush, taken before G changes
      slice_lines([&](int line, int k) { return Gs[(long long)(i0 + s_pos[k]) * N + line]; }, N, m, sG, N, eG,
                  etmp);
      // T = Gamma R_A, 64 columns at a time
      for (int c0 = 0; c0 < N; c0 += 64) {
        slice_lines(
            [&](int line, int k) {
              const int c = c0 + line, i = i0 + s_pos[k];
              return ((c == i) ? 1.0 : 0.0) - Gs[(long long)c * N + i];
            },
            min(64, N - c0), m, sb, 64, eB, etmp);
        float acc[OZS][2][2][4];
        mma_tile(sa, sb, acc);
        tile_epilogue(acc, [&](int rl, int cl, long long v) {
          const int c = c0 + cl;
          if (rl < m && c < N) Tg[(long long)c * KB + rl] = ozaki::ldexp_i64(v, eA[rl] + eB[cl] + kEOff);
        });
        __syncthreads();
      }
      // T as the right operand (lines = columns c, k = x)
      slice_lines([&](int line, int k) { return Tg[(long long)line * KB + k]; }, N, m, sT, N, eT, etmp);
      // G -= G0(:, I_A) T, tile by tile: the slices of tile i+1 are copied (cp.async) while
      // tile i multiplies, and each tile's G values are loaded before its MMAs
      const int ntl = (N + 63) / 64, ntiles = ntl * ntl;
      auto issue = [&](int ti, int b) {
        const int r0 = (ti / ntl) * 64, c0 = (ti % ntl) * 64;
        unsigned short* ta = sa + b * OZS * 64 * KP;
        unsigned short* tb = sb + b * OZS * 64 * KP;
        for (int e = tid; e < 2 * OZS * 64 * 4; e += kSubThreads) {
          const int ch = e & 3, line = (e >> 2) & 63, s = (e >> 8) % OZS, op = (e >> 8) / OZS;
          const int gl = (op == 0 ? r0 : c0) + line;
          const unsigned short* src = (op == 0 ? sG : sT) + ((long long)s * N + min(gl, N - 1)) * KP + ch * 8;
          cp16((op == 0 ? ta : tb) + (s * 64 + line) * KP + ch * 8, src, gl < N);
        }
        if (tid < 128) {
          const int op = tid >> 6, l = tid & 63, gl = (op ? c0 : r0) + l;
          (op ? fB : fA)[b][l] = (gl < N) ? (op ? eT : eG)[gl] : -1100;
        }
        asm volatile("cp.async.commit_group;\n" ::);
      };
      issue(0, 0);
      for (int ti = 0; ti < ntiles; ++ti) {
        const int b = (nbuf == 2) ? (ti & 1) : 0;
        const int r0 = (ti / ntl) * 64, c0 = (ti % ntl) * 64;
        if (nbuf == 2 && ti + 1 < ntiles) {
          issue(ti + 1, b ^ 1);
          asm volatile("cp.async.wait_group 1;\n" ::: "memory");
        } else {
          asm volatile("cp.async.wait_group 0;\n" ::: "memory");
        }
        __syncthreads();
        double gv[2][2][4];
        {
          const int lane = tid & 31, wid = tid >> 5;
          const int wm = wid >> 2, wn = wid & 3, g = lane >> 2, t4 = lane & 3;
#pragma unroll
          for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
              for (int v = 0; v < 4; ++v) {
                const int r = r0 + wm * 32 + mt * 16 + g + ((v >> 1) << 3);
                const int c = c0 + wn * 16 + nt * 8 + 2 * t4 + (v & 1);
                gv[mt][nt][v] = (r < N && c < N) ? Gs[(long long)c * N + r] : 0.0;
              }
        }
        float acc[OZS][2][2][4];
        mma_tile(sa + b * OZS * 64 * KP, sb + b * OZS * 64 * KP, acc);
        {
          const int lane = tid & 31, wid = tid >> 5;
          const int wm = wid >> 2, wn = wid & 3, g = lane >> 2, t4 = lane & 3;
#pragma unroll
          for (int mt = 0; mt < 2; ++mt)
#pragma unroll
            for (int nt = 0; nt < 2; ++nt)
#pragma unroll
              for (int v = 0; v < 4; ++v) {
                const int rl = wm * 32 + mt * 16 + g + ((v >> 1) << 3), cl = wn * 16 + nt * 8 + 2 * t4 + (v & 1);
                const int r = r0 + rl, c = c0 + cl;
                long long sv = 0;
#pragma unroll
                for (int m = 0; m < OZS; ++m) sv = (sv << OZB) + (long long)ozaki::f2i_small(acc[m][mt][nt][v]);
                if (sv != 0 && r < N && c < N)
                  Gs[(long long)c * N + r] = gv[mt][nt][v] - ozaki::ldexp_i64(sv, fA[b][rl] + fB[b][cl] + kEOff);
              }
        }
        __syncthreads();
        if (nbuf == 1 && ti + 1 < ntiles) issue(ti + 1, 0);
      }
    }
  }

  int8_t* frw = w.fields + (long long)eff * N;
  for (int i = tid; i < N; i += kSubThreads) frw[i] = s_field[i];
  if (tid == 0) {
    *w.sign = sign;
    *w.accepts += acc_count;
    if (mode == MODE_BWD && t == Lt) *w.sign_Lt = sign;
  }
}

static size_t g_sub_smem_limit = 0;  // dynamic shared memory the kernel may use

cudaError_t configure_submatrix_kernel() {
  int dev = 0, optin = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  cudaFuncAttributes fa{};
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&fa, metropolis_sub_kernel);
  if (e == cudaSuccess) {
    g_sub_smem_limit = (size_t)(optin - (int)fa.sharedSizeBytes);
    e = cudaFuncSetAttribute(metropolis_sub_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)g_sub_smem_limit);
  }
  return e;
}

void launch_metropolis_sub(const WalkerDev* W, int nw, int mode, int j, int q, int maxN, int S_max, cudaStream_t st) {
  const int nbuf = submatrix_smem_bytes(maxN, S_max, 2) <= g_sub_smem_limit ? 2 : 1;
  metropolis_sub_kernel<<<nw, kSubThreads, submatrix_smem_bytes(maxN, S_max, nbuf), st>>>(W, mode, j, q, nbuf);
}

}  // namespace dqmc
