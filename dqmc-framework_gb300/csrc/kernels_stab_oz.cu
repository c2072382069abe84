// kernels_stab_oz.cu — stabilization of tensor-core-path walkers (N >= 128):
// the UDT push and the Green's assembly as blocked Householder factorizations
// whose matrix products run on the BF16 tensor cores at FP64 accuracy.
//
// Reference: SvdStack::push (src/svd_stack.cpp:34-87) factors the B-chain with
// MKL dgesvd and compute_equaltime_greens (include/utils/numerical_stable.hpp:
// 186-239) assembles G through an LU inverse.  The plain path restates them
// with column-pivoted QR (kernels_general.cu), a latency-bound FP64 loop.  Here
//   push:   the columns of the chain are ordered once by norm (pre-pivoting,
//           Bai, Lee, Li and Xu, Linear Algebra Appl. 435 (2011) 659) and
//           factored by blocked Householder QR with 32-column panels.  Each
//           panel is factored in FP64 in shared memory (LAPACK dgeqr2 and
//           dlarft order); the trailing update A -= V T^T (V^T A), the formation
//           of Q and F = D^-1 R P^T F_prev are products.
//   greens: M = Dlmax^-1 U_L^T U_R Drmax^-1 + Dlmin F_L F_R^T Drmin and
//           Y = Dlmax^-1 U_L^T; M = QR by the same blocked Householder; X =
//           R^-1 Q^T Y by blocked reflector application and blocked back
//           substitution (FP64 diagonal blocks); G = U_R Drmax^-1 X.  Boundary
//           steps (one stack empty) form M = Y + Dmin F and G = X or X^T.
//   dynamic half-sweep (compute_dynamic_greens, include/utils/numerical_stable.hpp:
//           246-325): the same factorization of M also solves the second
//           right-hand side Y2 = Dlmin F_L, X2 = M^-1 Y2; then G(t,0) = U_R
//           Drmax^-1 X2 and G(0,t) = -F_R^T Drmin X (at t = beta, right stack
//           empty: G(beta,0) = X2, G(0,beta) = -X).
// Every product slices its two FP64 operands once (zslice_kernel, tensor-core
// images) into 8 integer slices of 7 bits (56 significant bits, K <= 256) or 9
// of 6 (54 bits, K <= 1024) and multiplies them on the BF16 tensor cores with
// FP32 accumulation (exact for the leading weight groups; zgemm_tc_kernel
// streams the slices through oztc::mainloop): an FP64-class GEMM.  The panel
// folds its T factor into the reflectors (Vt = V T, or V T^T when forming Q),
// so applying a block reflector is two products.  Panels, diagonal solves,
// reflectors and reductions are native FP64.  G equals the pivoted-QR path's
// mathematically; the UDT factors differ only in the column order of the QR.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "dqmc_device.cuh"
#include "ozaki.cuh"
#include "oz_tc.cuh"
#include "tcgen05.cuh"

namespace dqmc {

namespace {

constexpr int TB = 32;           // Householder panel width

__device__ __forceinline__ double zwarp_sum(double v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ void zstack_tops(const WalkerDev& w, int mode, int j, int& nl, int& nr) {
  if (mode == MODE_FWD) { nl = j + 1; nr = w.nstack - 1 - j; }
  else if (mode == MODE_BWD) { nl = w.nstack - 1 - j; nr = j + 1; }
  else { nl = 0; nr = w.nstack; }
}

// per-spin scratch: scr = X (matrix being factored) | Y (right-hand sides);
// work = Wb [TB N] | W2 [TB N] | T factors [ceil(N/TB) TB TB] | invd | four
// diagonal scale vectors | perm | line exponents of the two operands of the
// current product: 2 TB N + TB (N + TB) + 6.5 N <= N^2 for N >= 110
struct ZScr {
  double *X, *Y, *Wb, *W2, *Tb, *invd, *dlmaxi, *drmaxi, *dlmin, *drmin;
  int *perm, *expA, *expB;
};
__device__ __forceinline__ ZScr zscr(const WalkerDev& w, int sp) {
  const long long NN = (long long)w.N * w.N;
  const long long TN = (long long)TB * w.N;
  const long long TT = (long long)TB * TB * ((w.N + TB - 1) / TB);
  ZScr z;
  z.X = w.scr + sp * 2 * NN;
  z.Y = z.X + NN;
  double* wk = w.work + sp * NN;
  z.Wb = wk;
  z.W2 = wk + TN;
  z.Tb = wk + 2 * TN;
  z.invd = wk + 2 * TN + TT;
  z.dlmaxi = z.invd + w.N;
  z.drmaxi = z.dlmaxi + w.N;
  z.dlmin = z.drmaxi + w.N;
  z.drmin = z.dlmin + w.N;
  z.perm = reinterpret_cast<int*>(z.drmin + w.N);
  z.expA = z.perm + w.N;
  z.expB = z.expA + w.N;
  return z;
}

// An operand of C = op(A) op(B).  Element (row, col) of the stored block sits at
// p[col * ld + row'] with row' = rowmap ? rowmap[row] : row.  For A the logical
// element (i, k) is stored (i, k), or (k, i) when tr; for B the logical (k, i)
// is stored (k, i), or (i, k) when tr (i: output row of A / column of B).
struct ZOpnd {
  const double* p;
  long long ld;
  int tr;
  int kind;            // 0 full, 1 unit lower (Householder vectors), 2 upper with diagonal
  const int* rowmap;
  const double* ks;    // multiplier along k, or null
};
struct ZJob {
  ZOpnd a, b;
  double* c;
  long long ldc;
  int M, N, K;
  int beta;            // 1: C += (-1)^neg AB
  int neg;             // 1: the product enters negated (an operand modifier, no FP64 multiply)
  const double* rs;    // row multiplier of the product, or null
  const double* cs;    // column multiplier, or null
  int out;             // 1: Green's function output (wrap error, trace, spin copy);
                       // 2: time-displaced output (wrap error against the propagated value)
};

// the ping-pong slot of G(t,0) or G(0,t) at slice t ([parity][S][N*N])
__device__ __forceinline__ double* zdyn_slot(double* base, const WalkerDev& w, int sp, int t) {
  return base + ((long long)(t & 1) * w.S + sp) * w.N * w.N;
}

__device__ __forceinline__ double zel(const ZOpnd& o, int i, int k, bool isB) {
  const int row = (o.tr != (int)isB) ? k : i;
  const int col = (o.tr != (int)isB) ? i : k;
  double v;
  if (o.kind == 1 && row <= col) v = (row == col) ? 1.0 : 0.0;
  else if (o.kind == 2 && row > col) v = 0.0;
  else v = o.p[(long long)col * o.ld + (o.rowmap ? o.rowmap[row] : row)];
  if (o.ks) v *= o.ks[k];
  return v;
}

// The block reflector of panel p is I - V_p T_p V_p^T.  Its T factor is folded
// into the reflectors once per panel in FP64, Vt = V_p T_p (applying Q_p^T:
// T_p^T V_p^T A = Vt^T A) or Vt = V_p T_p^T (applying Q_p), so that every
// application is two products: Wb = Vt^T A, A -= V_p Wb.
enum ZOp {
  Z_QR_W = 0,    // Wb = (V_p T_p)^T X(j0:, j0+pb:)
  Z_QR_UPD,      // X(j0:, j0+pb:) -= V_p Wb
  Z_Q_W,         // Wb = (V_p T_p^T)^T U(j0:, j0:)   (forming Q, backward)
  Z_Q_UPD,       // U(j0:, j0:) -= V_p Wb
  Z_F,           // F = D^-1 R P^T F_prev
  Z_GA,          // M = Dlmax^-1 U_L^T U_R Drmax^-1
  Z_GB,          // M += Dlmin F_L F_R^T Drmin
  Z_AQ_W,        // Wb = (V_p T_p)^T Y(j0:, :)
  Z_AQ_UPD,      // Y(j0:, :) -= V_p Wb
  Z_TR_UPD,      // Y(j0:j0+pb, :) -= R(j0:j0+pb, j0+pb:) Y(j0+pb:, :)
  Z_GG,          // G = U_R Drmax^-1 X
  Z_GRAM,        // Zg = V_p^T V_p (pb x pb, into Wb): the Gram matrix of the panel's reflectors
  Z_VT,          // Vt = V_p T_p (m x pb, into W2), T_p from ztfac_kernel
  // the dynamic half-sweep's second right-hand side Y2 (dynx) and outputs
  Z_AQ2_W,       // Wb = (V_p T_p)^T Y2(j0:, :)
  Z_AQ2_UPD,     // Y2(j0:, :) -= V_p Wb
  Z_TR2_UPD,     // Y2(j0:j0+pb, :) -= R(j0:j0+pb, j0+pb:) Y2(j0+pb:, :)
  Z_DT0_OUT,     // G(t,0) = U_R Drmax^-1 X2
  Z_D0T_OUT,     // G(0,t) = -F_R^T Drmin X
};

__device__ bool zjob(const WalkerDev& w, int op, int mode, int j, int p, int sp, ZJob& jb) {
  if (j >= w.nstack) return false;
  const int N = w.N;
  const long long NN = (long long)N * N;
  const ZScr z = zscr(w, sp);
  const int j0 = p * TB;
  const int m = N - j0, pb = min(TB, m);
  jb = ZJob{};
  const bool panel_op = op != Z_F && op != Z_GA && op != Z_GB && op != Z_GG;
  if (panel_op && j0 >= N) return false;
  const ZOpnd Vp{z.X + (long long)j0 * N + j0, N, 0, 1, nullptr, nullptr};
  const ZOpnd VtT{z.W2, N, 1, 0, nullptr, nullptr};  // Vt^T (Vt: m x pb, ld N, in W2)
  const ZOpnd Wbo{z.Wb, TB, 0, 0, nullptr, nullptr};
  int nl = 0, nr = 0;
  zstack_tops(w, mode, j, nl, nr);
  const int side = (mode == MODE_FWD) ? 0 : 1;
  switch (op) {
    case Z_QR_W:
    case Z_QR_UPD: {
      const int nt = m - pb;
      if (nt <= 0) return false;
      if (op == Z_QR_W) {
        jb.a = VtT;
        jb.b = ZOpnd{z.X + (long long)(j0 + pb) * N + j0, N, 0, 0, nullptr, nullptr};
        jb.c = z.Wb; jb.ldc = TB; jb.M = pb; jb.N = nt; jb.K = m;
      } else {
        jb.a = Vp;
        jb.b = Wbo;
        jb.c = z.X + (long long)(j0 + pb) * N + j0; jb.ldc = N; jb.M = m; jb.N = nt; jb.K = pb;
        jb.beta = 1; jb.neg = 1;
      }
      return true;
    }
    case Z_Q_W:
    case Z_Q_UPD: {
      double* Uo = stack_level(w, side, sp, j);
      if (op == Z_Q_W) {
        jb.a = VtT;
        jb.b = ZOpnd{Uo + (long long)j0 * N + j0, N, 0, 0, nullptr, nullptr};
        jb.c = z.Wb; jb.ldc = TB; jb.M = pb; jb.N = m; jb.K = m;
      } else {
        jb.a = Vp;
        jb.b = Wbo;
        jb.c = Uo + (long long)j0 * N + j0; jb.ldc = N; jb.M = m; jb.N = m; jb.K = pb;
        jb.beta = 1; jb.neg = 1;
      }
      return true;
    }
    case Z_F: {
      if (j == 0) return false;
      double* lv = stack_level(w, side, sp, j);
      const double* fp = stack_level(w, side, sp, j - 1) + NN;
      jb.a = ZOpnd{z.X, N, 0, 2, nullptr, nullptr};
      jb.b = ZOpnd{fp, N, 0, 0, z.perm, nullptr};
      jb.rs = z.invd;
      jb.c = lv + NN; jb.ldc = N; jb.M = N; jb.N = N; jb.K = N;
      return true;
    }
    case Z_GA:
    case Z_GB:
    case Z_GG: {
      if (!(nl > 0 && nr > 0)) return false;
      const double* UL = stack_level(w, 0, sp, nl - 1);
      const double* UR = stack_level(w, 1, sp, nr - 1);
      if (op == Z_GA) {
        jb.a = ZOpnd{UL, N, 1, 0, nullptr, nullptr};
        jb.b = ZOpnd{UR, N, 0, 0, nullptr, nullptr};
        jb.rs = z.dlmaxi; jb.cs = z.drmaxi;
        jb.c = z.X; jb.ldc = N; jb.M = N; jb.N = N; jb.K = N;
      } else if (op == Z_GB) {
        jb.a = ZOpnd{UL + NN, N, 0, 0, nullptr, nullptr};
        jb.b = ZOpnd{UR + NN, N, 1, 0, nullptr, nullptr};
        jb.rs = z.dlmin; jb.cs = z.drmin;
        jb.c = z.X; jb.ldc = N; jb.M = N; jb.N = N; jb.K = N; jb.beta = 1;
      } else {
        jb.a = ZOpnd{UR, N, 0, 0, nullptr, z.drmaxi};
        jb.b = ZOpnd{z.Y, N, 0, 0, nullptr, nullptr};
        jb.c = w.G + sp * NN; jb.ldc = N; jb.M = N; jb.N = N; jb.K = N; jb.out = 1;
      }
      return true;
    }
    case Z_AQ_W:
    case Z_AQ_UPD: {
      if (op == Z_AQ_W) {
        jb.a = VtT;
        jb.b = ZOpnd{z.Y + j0, N, 0, 0, nullptr, nullptr};
        jb.c = z.Wb; jb.ldc = TB; jb.M = pb; jb.N = N; jb.K = m;
      } else {
        jb.a = Vp;
        jb.b = Wbo;
        jb.c = z.Y + j0; jb.ldc = N; jb.M = m; jb.N = N; jb.K = pb;
        jb.beta = 1; jb.neg = 1;
      }
      return true;
    }
    case Z_TR_UPD:
    case Z_TR2_UPD: {
      if (j0 + pb >= N) return false;
      if (op == Z_TR2_UPD && !w.dynx) return false;
      double* Yr = (op == Z_TR_UPD) ? z.Y : w.dynx + sp * NN;
      jb.a = ZOpnd{z.X + (long long)(j0 + pb) * N + j0, N, 0, 0, nullptr, nullptr};
      jb.b = ZOpnd{Yr + j0 + pb, N, 0, 0, nullptr, nullptr};
      jb.c = Yr + j0; jb.ldc = N; jb.M = pb; jb.N = N; jb.K = N - j0 - pb;
      jb.beta = 1; jb.neg = 1;
      return true;
    }
    case Z_GRAM:
      jb.a = ZOpnd{z.X + (long long)j0 * N + j0, N, 1, 1, nullptr, nullptr};  // V_p^T
      jb.b = Vp;
      jb.c = z.Wb; jb.ldc = TB; jb.M = pb; jb.N = pb; jb.K = m;
      return true;
    case Z_VT:
      jb.a = Vp;
      jb.b = ZOpnd{z.Tb + (long long)p * TB * TB, TB, 0, 2, nullptr, nullptr};  // T_p, upper with diagonal
      jb.c = z.W2; jb.ldc = N; jb.M = m; jb.N = pb; jb.K = pb;
      return true;
    case Z_AQ2_W:
    case Z_AQ2_UPD: {
      if (!w.dynx) return false;
      double* Y2 = w.dynx + sp * NN;
      if (op == Z_AQ2_W) {
        jb.a = VtT;
        jb.b = ZOpnd{Y2 + j0, N, 0, 0, nullptr, nullptr};
        jb.c = z.Wb; jb.ldc = TB; jb.M = pb; jb.N = N; jb.K = m;
      } else {
        jb.a = Vp;
        jb.b = Wbo;
        jb.c = Y2 + j0; jb.ldc = N; jb.M = m; jb.N = N; jb.K = pb;
        jb.beta = 1; jb.neg = 1;
      }
      return true;
    }
    case Z_DT0_OUT:
    case Z_D0T_OUT: {
      // forward step j of the dynamic half-sweep, both stacks present
      if (!w.gt0 || !w.dynx || mode != MODE_FWD || !(nl > 0 && nr > 0)) return false;
      const int t_end = min((j + 1) * w.pace, w.Lt);
      const double* UR = stack_level(w, 1, sp, nr - 1);
      if (op == Z_DT0_OUT) {
        jb.a = ZOpnd{UR, N, 0, 0, nullptr, z.drmaxi};
        jb.b = ZOpnd{w.dynx + sp * NN, N, 0, 0, nullptr, nullptr};
        jb.c = zdyn_slot(w.gt0, w, sp, t_end);
      } else {
        jb.a = ZOpnd{UR + NN, N, 1, 0, nullptr, z.drmin};  // F_R^T, times Drmin along k
        jb.b = ZOpnd{z.Y, N, 0, 0, nullptr, nullptr};
        jb.c = zdyn_slot(w.g0t, w, sp, t_end);
        jb.neg = 1;
      }
      jb.ldc = N; jb.M = N; jb.N = N; jb.K = N; jb.out = 2;
      return true;
    }
  }
  return false;
}

// fixed-point magnitude |x| / 2^e with Q fraction bits (e >= exp_bound(x), Q <= 62)
__device__ __forceinline__ unsigned long long zfixed(double x, int e, int Q, bool& neg) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex == 0) return 0ULL;
  const unsigned long long mant = (b & 0xFFFFFFFFFFFFFULL) | 0x10000000000000ULL;
  const int s = ex - 1075 - e + Q;  // |x| 2^{Q-e} = mant 2^s
  if (s >= 0) return mant << s;     // s <= Q - 53 here
  if (s <= -64) return 0ULL;
  return mant >> (-s);
}

}  // namespace

// --------------------------------------------------------------------------
// Slicing of both operands of a product, once per product: blockIdx.y = 0 the
// rows of op(A), 1 the columns of op(B); 32 lines per CTA.  Pass 1: the line
// exponents (8 k groups per line); pass 2: 32 x 32 tiles staged through
// shared memory so that loads run along the stored matrix.  Output: per
// operand S slices of tc_lines(N) x zld in the tensor core's shared-memory
// image (ozaki::tc_index), zero past K up to a multiple of 32.
// --------------------------------------------------------------------------
template <int S, int B>
__global__ void __launch_bounds__(256) zslice_kernel(const WalkerDev* __restrict__ W, int op, int mode, int j, int p) {
  const int wi = blockIdx.z >> 1, sp = blockIdx.z & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || sp >= w.S) return;
  ZJob jb;
  if (!zjob(w, op, mode, j, p, sp, jb)) return;
  if ((jb.K <= 256) != (B == 7)) return;
  const bool isB = blockIdx.y == 1;
  const ZOpnd& o = isB ? jb.b : jb.a;
  const int nlines = isB ? jb.N : jb.M;
  const int l0 = blockIdx.x * 32;
  if (l0 >= nlines) return;
  constexpr int Q = S * B;
  const int N = w.N, Kp = (jb.K + 31) / 32 * 32, nlb = ozaki::tc_lines(N) / 8;
  const long long sst = (long long)ozaki::tc_lines(N) * w.zld;
  const ZScr z = zscr(w, sp);
  unsigned short* out = w.zsl + ((long long)(sp * 2 + (isB ? 1 : 0)) * 9) * sst;
  // lines contiguous in memory when the stored row index runs along the line
  const bool line_fast = (o.tr == (int)isB);
  __shared__ int s_e[8][32];
  __shared__ double s_t[32][33];
  {
    const int ll = line_fast ? (threadIdx.x & 31) : (threadIdx.x >> 3);
    const int kg = line_fast ? (threadIdx.x >> 5) : (threadIdx.x & 7);
    const int line = l0 + ll;
    int e = -1100;
    if (line < nlines)
      for (int k0 = kg; k0 < jb.K; k0 += 64) {
        double x[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
          const int k = k0 + 8 * u;
          x[u] = (k < jb.K) ? zel(o, line, k, isB) : 0.0;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) e = max(e, ozaki::exp_bound(x[u]));
      }
    s_e[kg][ll] = e;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    int m = s_e[0][threadIdx.x];
#pragma unroll
    for (int q = 1; q < 8; ++q) m = max(m, s_e[q][threadIdx.x]);
    s_e[0][threadIdx.x] = m;
    if (l0 + threadIdx.x < nlines) (isB ? z.expB : z.expA)[l0 + threadIdx.x] = m;
  }
  __syncthreads();
  for (int k0 = 0; k0 < Kp; k0 += 32) {
    for (int e = threadIdx.x; e < 32 * 32; e += 256) {
      const int ll = line_fast ? (e & 31) : (e >> 5), kk = line_fast ? (e >> 5) : (e & 31);
      const int line = l0 + ll, k = k0 + kk;
      s_t[ll][kk] = (line < nlines && k < jb.K) ? zel(o, line, k, isB) : 0.0;
    }
    __syncthreads();
    {  // one line and 4 consecutive k per thread: one 8-byte store per slice
      const int kq = threadIdx.x & 7, ll = threadIdx.x >> 3, line = l0 + ll;
      if (line < nlines) {
        unsigned long long q[4];
        bool ng[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) q[u] = zfixed(s_t[ll][kq * 4 + u], s_e[0][ll], Q, ng[u]);
        unsigned short* o = out + ozaki::tc_index(line, k0 + kq * 4, nlb);
#pragma unroll
        for (int s2 = 0; s2 < S; ++s2) {
          ushort4 v;
          v.x = ozaki::slice_bf16q(q[0], s2, B, Q, ng[0]);
          v.y = ozaki::slice_bf16q(q[1], s2, B, Q, ng[1]);
          v.z = ozaki::slice_bf16q(q[2], s2, B, Q, ng[2]);
          v.w = ozaki::slice_bf16q(q[3], s2, B, Q, ng[3]);
          *reinterpret_cast<ushort4*>(o + s2 * sst) = v;
        }
      }
    }
    __syncthreads();
  }
}

// --------------------------------------------------------------------------
// The product on the 5th-generation tensor cores (tcgen05): a 128 x NT output
// tile per CTA, the S weight groups accumulated in TMEM (S NT columns), the
// pre-sliced operands streamed by oztc::mainloop (bulk copies through a ring
// of NS stages of 16-deep k chunks).  The 56-bit configuration runs 128 x 32
// tiles with 2 stages so that two CTAs share an SM (256 TMEM columns, 80 KB of
// shared memory and at most 128 registers each): one CTA's epilogue overlaps
// the other's copies and MMAs.
// --------------------------------------------------------------------------
template <int S, int B, int NT, int NS, int MINB>
__global__ void __launch_bounds__(256, MINB) zgemm_tc_kernel(const WalkerDev* __restrict__ W, int op, int mode, int j,
                                                             int p, int trace_slot) {
  constexpr int MT = 128;
  constexpr int CW = (MINB > 1) ? 8 : 16;  // TMEM columns per load in the epilogue
  constexpr unsigned TCOLS = (S * NT <= 256) ? 256u : 512u;
  static_assert(MINB == 1 || S * NT <= 256, "two CTAs per SM need at most 256 TMEM columns each");
  const int wi = blockIdx.z >> 1, sp = blockIdx.z & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || sp >= w.S) return;
  ZJob jb;
  if (!zjob(w, op, mode, j, p, sp, jb)) return;
  if ((jb.K <= 256) != (B == 7)) return;
  const int r0 = blockIdx.y * MT, c0 = blockIdx.x * NT;
  if (r0 >= jb.M || c0 >= jb.N) return;
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ int eA[MT], eB[NT];
  __shared__ __align__(8) unsigned long long full[NS], done[NS];
  __shared__ unsigned tbase;
  __shared__ int s_fail, s_last;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const ZScr z = zscr(w, sp);
  const int N = w.N;
  if (tid < MT) eA[tid] = (r0 + tid < jb.M) ? z.expA[r0 + tid] : -1100;
  if (tid < NT) eB[tid] = (c0 + tid < jb.N) ? z.expB[c0 + tid] : -1100;
  if (tid == 0) {
    s_fail = 0;
    s_last = -1;
    for (int i = 0; i < NS; ++i) {
      tc::mbar_init(&full[i]);
      tc::mbar_init(&done[i]);
    }
    tc::mbar_fence_init();
  }
  if (warp == 0) tc::alloc(&tbase, TCOLS);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const unsigned taddr = tbase;
  if (tid == 0) {
    const long long sst = (long long)ozaki::tc_lines(N) * w.zld;
    const unsigned short* zA = w.zsl + (long long)(sp * 2) * 9 * sst;
    const unsigned short* zB = zA + 9 * sst;
    const long long cstep = (long long)(ozaki::tc_lines(N) / 8) * 128;
    bool ok;
    s_last = oztc::mainloop<S, MT, NT, NS>(tsm, full, done, taddr, zA + (long long)(r0 / 8) * 128,
                                            zB + (long long)(c0 / 8) * 128, sst, cstep, (jb.K + 15) / 16, ok);
    s_fail = ok ? 0 : 1;
  }
  __syncthreads();
  {
    const int last = s_last;
    const bool mma_done = last >= 0 && tc::mbar_wait(&done[last % NS], (last / NS) & 1);
    if (__syncthreads_or(!mma_done || s_fail) && tid == 0) s_fail = 1;
  }
  tc::fence_after();
  __syncthreads();

  // epilogue: warp w reads TMEM lanes 32 (w & 3) .. + 31 (rows), column half (w >> 2)
  const long long NN = (long long)w.N * w.N;
  double err = 0.0;
  bool finite = true;
  double* tr = (jb.out && w.trace && trace_slot >= 0 && trace_slot < w.trace_cap)
                   ? w.trace + ((long long)trace_slot * 2 + sp) * NN : nullptr;
  const bool check = (jb.out == 2) || (jb.out && !(mode == MODE_INIT || (mode == MODE_BWD && j == w.nstack - 1)));
  const int q4 = warp & 3, half = warp >> 2;
  const int rl = q4 * 32 + lane, r = r0 + rl;
  // K <= 32: every group sum is below 2^22 and converts with an FP32 add (the conversion
  // unit does ~15 per clock per SM); warps whose 32 rows are all past M skip the epilogue
  const bool small_k = jb.K <= 32;
  if (!s_fail && r0 + q4 * 32 < jb.M) {
    for (int cc = half * (NT / 2); cc < (half + 1) * (NT / 2); cc += CW) {
      uint32_t v[S][CW];
#pragma unroll
      for (int m = 0; m < S; ++m) tc::ldw<CW>(v[m], taddr + ((unsigned)(q4 * 32) << 16) + (unsigned)(m * NT + cc));
      tc::wait_ld();
#pragma unroll
      for (int u = 0; u < CW; ++u) {
        const int cl = cc + u, col = c0 + cl;
        if (r >= jb.M || col >= jb.N) continue;
        long long hi = 0, lo = 0;
        if (small_k) {
#pragma unroll
          for (int m = 0; m < 4; ++m) hi = (hi << B) + (long long)ozaki::f2i_small(__uint_as_float(v[m][u]));
#pragma unroll
          for (int m = 4; m < S; ++m) lo = (lo << B) + (long long)ozaki::f2i_small(__uint_as_float(v[m][u]));
        } else {
#pragma unroll
          for (int m = 0; m < 4; ++m) hi = (hi << B) + (long long)__float2int_rn(__uint_as_float(v[m][u]));
#pragma unroll
          for (int m = 4; m < S; ++m) lo = (lo << B) + (long long)__float2int_rn(__uint_as_float(v[m][u]));
        }
        const int e = eA[rl] + eB[cl];
        double val = ozaki::combine_hilo<S, B>(hi, lo, e);
        if (jb.rs) val *= jb.rs[r];
        if (jb.cs) val *= jb.cs[col];
        const long long o = (long long)col * jb.ldc + r;
        if (!jb.out) {
          if (jb.neg) val = -val;
          jb.c[o] = jb.beta ? jb.c[o] + val : val;
        } else if (jb.out == 2) {
          if (jb.neg) val = -val;
          err = fmax(err, fabs(val - jb.c[o]));
          if (!isfinite(val)) finite = false;
          jb.c[o] = val;
        } else {
          if (check) err = fmax(err, fabs(val - jb.c[o]));
          if (!isfinite(val)) finite = false;
          jb.c[o] = val;
          if (tr) tr[o] = val;
          if (w.S == 1) {
            jb.c[NN + o] = val;
            if (tr) tr[NN + o] = val;
          }
        }
      }
    }
  }
  if (s_fail && tid == 0) atomicOr(w.status, ST_TIMEOUT);
  if (jb.out) {
    if (!finite) atomicOr(w.status, ST_NONFINITE_G);
    if (check) {
      for (int o = 16; o > 0; o >>= 1) err = fmax(err, __shfl_xor_sync(0xffffffffu, err, o));
      if (lane == 0) atomicMax(w.wrap_bits, (unsigned long long)__double_as_longlong(err));
    }
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::dealloc(taddr, TCOLS);
}

// --------------------------------------------------------------------------
// Push preparation: column norms of the chain, order by decreasing norm
// (ties by index), X = chain(:, perm).  One CTA per (walker, spin).
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(256) zpush_prep_kernel(const WalkerDev* __restrict__ W, int mode, int j) {
  const int wi = blockIdx.x >> 1, sp = blockIdx.x & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || sp >= w.S || j >= w.nstack) return;
  const int N = w.N;
  int nsl;
  {
    const int k = (mode == MODE_FWD) ? j : (w.nstack - 1 - j);
    nsl = min((k + 1) * w.pace, w.Lt) - k * w.pace;
  }
  const long long NN = (long long)N * N;
  const double* Cin = w.chain + (long long)((w.cb ? 0 : (nsl & 1)) * w.S + sp) * NN;
  const ZScr z = zscr(w, sp);
  extern __shared__ long long zkey[];  // [N] norm bit patterns
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int c = wid; c < N; c += 8) {
    double s = 0.0;
    for (int r = lane; r < N; r += 32) {
      const double a = Cin[(long long)c * N + r];
      s = fma(a, a, s);
    }
    s = zwarp_sum(s);
    if (lane == 0) zkey[c] = __double_as_longlong(sqrt(s));  // >= 0 (or NaN): bit order = value order
  }
  for (int k = threadIdx.x; k < N; k += 256) z.perm[k] = k;
  __syncthreads();
  for (int c = threadIdx.x; c < N; c += 256) {
    const long long kc = zkey[c];
    int rank = 0;
    for (int c2 = 0; c2 < N; ++c2) {
      const long long k2 = zkey[c2];
      rank += (k2 > kc || (k2 == kc && c2 < c)) ? 1 : 0;
    }
    z.perm[rank] = c;
  }
  __syncthreads();
  for (int k = wid; k < N; k += 8) {
    const int c = z.perm[k];
    for (int r = lane; r < N; r += 32) z.X[(long long)k * N + r] = Cin[(long long)c * N + r];
  }
}

// --------------------------------------------------------------------------
// Householder panel p of X (rows j0:N, columns j0:j0+pb) in shared memory:
// reflectors into X below the diagonal, R on and above, T_p (dlarft) into the
// scratch; for the push also D = |diag R| into the stack level and 1/D.
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(256) zqr_panel_kernel(const WalkerDev* __restrict__ W, int mode, int j, int p,
                                                        int push) {
  const int wi = blockIdx.x >> 1, sp = blockIdx.x & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || sp >= w.S || j >= w.nstack) return;
  const int N = w.N, j0 = p * TB;
  if (j0 >= N) return;
  const int m = N - j0, pb = min(TB, m);
  const ZScr z = zscr(w, sp);
  extern __shared__ double psm[];
  double* P = psm;                // [TB][m], P[c * m + r]
  double* T = P + TB * m;         // [TB][TB], T[c * TB + r] (tau on the diagonal)
  __shared__ double s_red[8];
  __shared__ double s_tau, s_scal;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  for (int c = 0; c < pb; ++c)
    for (int r = tid; r < m; r += 256) P[c * m + r] = z.X[(long long)(j0 + c) * N + j0 + r];
  __syncthreads();
  for (int c = 0; c < pb; ++c) {
    double s = 0.0;
    for (int r = c + 1 + tid; r < m; r += 256) s = fma(P[c * m + r], P[c * m + r], s);
    s = zwarp_sum(s);
    if (lane == 0) s_red[wid] = s;
    __syncthreads();
    if (tid == 0) {
      double xn2 = 0.0;
      for (int q = 0; q < 8; ++q) xn2 += s_red[q];
      const double alpha = P[c * m + c];
      double tau = 0.0, beta = alpha, scal = 1.0;
      if (xn2 != 0.0) {
        const double nrm = sqrt(alpha * alpha + xn2);
        beta = alpha >= 0 ? -nrm : nrm;
        tau = (beta - alpha) / beta;
        scal = 1.0 / (alpha - beta);
      }
      s_tau = tau;
      s_scal = scal;
      P[c * m + c] = beta;
      T[c * TB + c] = tau;
    }
    __syncthreads();
    const double scal = s_scal, tau = s_tau;
    for (int r = c + 1 + tid; r < m; r += 256) P[c * m + r] *= scal;
    __syncthreads();
    if (tau != 0.0)
      for (int cc = c + 1 + wid; cc < pb; cc += 8) {
        double d = 0.0;
        for (int r = c + 1 + lane; r < m; r += 32) d = fma(P[c * m + r], P[cc * m + r], d);
        d = zwarp_sum(d) + P[cc * m + c];
        const double wv = tau * d;
        if (lane == 0) P[cc * m + c] -= wv;
        for (int r = c + 1 + lane; r < m; r += 32) P[cc * m + r] = fma(-wv, P[c * m + r], P[cc * m + r]);
      }
    __syncthreads();
  }
  for (int c = 0; c < pb; ++c)
    for (int r = tid; r < m; r += 256) z.X[(long long)(j0 + c) * N + j0 + r] = P[c * m + r];
  // the Gram matrix V^T V, the T factor and Vt = V T follow on the tensor cores (Z_GRAM,
  // ztfac_kernel, Z_VT); the panel leaves tau on the diagonal of its T slot
  double* Tg = z.Tb + (long long)p * TB * TB;
  for (int e = tid; e < TB * TB; e += 256) {
    const int r = e % TB, c = e / TB;
    Tg[e] = (r == c && c < pb) ? T[c * TB + c] : 0.0;
  }
  if (push && tid < pb) {
    const int side = (mode == MODE_FWD) ? 0 : 1;
    double* Do = stack_level(w, side, sp, j) + 2 * (long long)N * N;
    const double d = fabs(P[tid * m + tid]);
    Do[j0 + tid] = d;
    z.invd[j0 + tid] = (d != 0.0) ? 1.0 / d : 0.0;
    if (d == 0.0 || !isfinite(d)) atomicOr(w.status, ST_SINGULAR);
  }
}

// The T factor of panel p (LAPACK dlarft, forward, columnwise): T(c, c) = tau_c and
// T(0:c, c) = -tau_c T(0:c, 0:c) Zg(0:c, c), Zg = V^T V from the Z_GRAM product (in Wb).
// One warp per (walker, spin).
__global__ void __launch_bounds__(32) ztfac_kernel(const WalkerDev* __restrict__ W, int mode, int j, int p) {
  const int wi = blockIdx.x >> 1, sp = blockIdx.x & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || sp >= w.S || j >= w.nstack) return;
  const int N = w.N, j0 = p * TB;
  if (j0 >= N) return;
  const int pb = min(TB, N - j0), tid = threadIdx.x;
  const ZScr z = zscr(w, sp);
  __shared__ double T[TB * TB], Zg[TB * TB];
  double* Tg = z.Tb + (long long)p * TB * TB;
  for (int e = tid; e < TB * TB; e += 32) {
    T[e] = Tg[e];  // tau on the diagonal, zeros elsewhere
    const int i = e % TB, c = e / TB;
    Zg[e] = (i < pb && c < pb) ? z.Wb[(long long)c * TB + i] : 0.0;
  }
  __syncwarp();
  for (int c = 1; c < pb; ++c) {
    double s = 0.0;
    if (tid < c)
      for (int k = tid; k < c; ++k) s = fma(T[k * TB + tid], Zg[c * TB + k], s);
    __syncwarp();
    if (tid < c) T[c * TB + tid] = -T[c * TB + c] * s;
    __syncwarp();
  }
  for (int e = tid; e < TB * TB; e += 32) Tg[e] = T[e];
}

// Vt = V_p T_p^T (m x pb, ld N) for forming Q: Vt(r, c) = sum_{c <= q <= r} V(r, q) T(c, q).
// 32 rows per CTA, V and T staged in shared memory.
__global__ void __launch_bounds__(256) zvt_kernel(const WalkerDev* __restrict__ W, int mode, int j, int p) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || sp >= w.S || j >= w.nstack) return;
  const int N = w.N, j0 = p * TB;
  if (j0 >= N) return;
  const int m = N - j0, pb = min(TB, m), r0 = blockIdx.x * 32;
  if (r0 >= m) return;
  const ZScr z = zscr(w, sp);
  __shared__ double sV[TB][33], sT[TB][33];  // sV[q][rl] = V(r0 + rl, q), sT[q][c] = T(c, q)
  const double* Tg = z.Tb + (long long)p * TB * TB;
  for (int e = threadIdx.x; e < TB * TB; e += 256) {
    const int rl = e & 31, q = e >> 5, r = r0 + rl;
    double v = 0.0;
    if (q < pb && r < m) v = (r > q) ? z.X[(long long)(j0 + q) * N + j0 + r] : (r == q ? 1.0 : 0.0);
    sV[q][rl] = v;
    sT[q][rl] = (q < pb && rl < pb) ? Tg[q * TB + rl] : 0.0;  // T(rl, q), zero below the diagonal
  }
  __syncthreads();
  for (int e = threadIdx.x; e < 32 * pb; e += 256) {
    const int rl = e & 31, c = e >> 5, r = r0 + rl;
    if (r >= m) continue;
    double s = 0.0;
    for (int q = c; q < pb; ++q) s = fma(sV[q][rl], sT[q][c], s);
    z.W2[(long long)c * N + r] = s;
  }
}

// U = I before forming Q; at the first level F = D^-1 R P^T directly
__global__ void __launch_bounds__(256) zpush_fin_kernel(const WalkerDev* __restrict__ W, int mode, int j) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || sp >= w.S || j >= w.nstack) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  const int side = (mode == MODE_FWD) ? 0 : 1;
  double* Uo = stack_level(w, side, sp, j);
  double* Fo = Uo + NN;
  const ZScr z = zscr(w, sp);
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < NN; e += (long long)gridDim.x * 256) {
    const int r = (int)(e % N), c = (int)(e / N);
    Uo[e] = (r == c) ? 1.0 : 0.0;
    if (j == 0) Fo[(long long)z.perm[c] * N + r] = (r <= c) ? z.X[e] * z.invd[r] : 0.0;
  }
}

// --------------------------------------------------------------------------
// Green's preparation: scale vectors; Y = Dmax^-1 U^T (col-major); boundary
// steps also M = Y + Dmin F.  Grid over the N^2 elements.
// --------------------------------------------------------------------------
__global__ void __launch_bounds__(256) zgreens_prep_kernel(const WalkerDev* __restrict__ W, int mode, int j) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || sp >= w.S || j >= w.nstack) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  int nl, nr;
  zstack_tops(w, mode, j, nl, nr);
  const ZScr z = zscr(w, sp);
  const bool both = nl > 0 && nr > 0;
  const double* lv = (nl > 0) ? stack_level(w, 0, sp, nl - 1) : stack_level(w, 1, sp, nr - 1);
  const double* U = lv;
  const double* F = lv + NN;
  const double* D = lv + 2 * NN;
  if (blockIdx.x == 0 && both) {
    const double* DR = stack_level(w, 1, sp, nr - 1) + 2 * NN;
    for (int k = threadIdx.x; k < N; k += 256) {
      z.dlmaxi[k] = 1.0 / fmax(D[k], 1.0);
      z.dlmin[k] = fmin(D[k], 1.0);
      z.drmaxi[k] = 1.0 / fmax(DR[k], 1.0);
      z.drmin[k] = fmin(DR[k], 1.0);
    }
  }
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < NN; e += (long long)gridDim.x * 256) {
    const int r = (int)(e % N), c = (int)(e / N);
    const double dr = D[r];
    const double y = U[(long long)r * N + c] / fmax(dr, 1.0);  // (Dmax^-1 U^T)(r, c)
    z.Y[e] = y;
    if (!both) z.X[e] = y + fmin(dr, 1.0) * F[e];
  }
}

// back substitution of the diagonal block p: R_pp X(j0:j0+pb, c) = Y(j0:j0+pb, c), thread per
// column; rhs 0: Y, 1: the dynamic half-sweep's second right-hand side (dynx)
__global__ void __launch_bounds__(128) ztrsm_diag_kernel(const WalkerDev* __restrict__ W, int mode, int j, int p,
                                                         int rhs) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || sp >= w.S || j >= w.nstack) return;
  if (rhs && !w.dynx) return;
  const int N = w.N, j0 = p * TB;
  if (j0 >= N) return;
  const int pb = min(TB, N - j0);
  const ZScr z = zscr(w, sp);
  __shared__ double R[TB][TB + 1];
  __shared__ double rinv[TB];
  for (int e = threadIdx.x; e < TB * TB; e += 128) {
    const int i = e % TB, k = e / TB;
    R[i][k] = (i < pb && k < pb && i <= k) ? z.X[(long long)(j0 + k) * N + j0 + i] : 0.0;
  }
  __syncthreads();
  if (threadIdx.x < TB) {  // rows past a partial panel: 0 (their x stays 0)
    const double d = R[threadIdx.x][threadIdx.x];
    rinv[threadIdx.x] = (d != 0.0) ? 1.0 / d : 0.0;
    if (d == 0.0 && threadIdx.x < pb && blockIdx.x == 0) atomicOr(w.status, ST_SINGULAR);
  }
  __syncthreads();
  const int c = blockIdx.x * 128 + threadIdx.x;
  if (c >= N) return;
  double* y = (rhs ? w.dynx + (long long)sp * N * N : z.Y) + (long long)c * N + j0;
  double x[TB];
#pragma unroll
  for (int i = 0; i < TB; ++i) x[i] = (i < pb) ? y[i] : 0.0;
#pragma unroll
  for (int i = TB - 1; i >= 0; --i) {
    double s = x[i];
#pragma unroll
    for (int k = i + 1; k < TB; ++k) s = fma(-R[i][k], x[k], s);
    x[i] = s * rinv[i];
  }
#pragma unroll
  for (int i = 0; i < TB; ++i)
    if (i < pb) y[i] = x[i];
}

// boundary steps: G = X (left stack present) or X^T (right only), wrap error, trace
__global__ void __launch_bounds__(256) zgreens_out_kernel(const WalkerDev* __restrict__ W, int mode, int j,
                                                          int trace_slot) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || sp >= w.S || j >= w.nstack) return;
  int nl, nr;
  zstack_tops(w, mode, j, nl, nr);
  if (nl > 0 && nr > 0) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  const ZScr z = zscr(w, sp);
  double* G = w.G + sp * NN;
  double* tr = (w.trace && trace_slot >= 0 && trace_slot < w.trace_cap) ? w.trace + ((long long)trace_slot * 2 + sp) * NN
                                                                       : nullptr;
  const bool transpose_out = (nl == 0);
  const bool check = !(mode == MODE_INIT || (mode == MODE_BWD && j == w.nstack - 1));
  double err = 0.0;
  bool finite = true;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < NN; e += (long long)gridDim.x * 256) {
    const int r = (int)(e % N), c = (int)(e / N);
    const double v = transpose_out ? z.Y[(long long)r * N + c] : z.Y[e];
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

// dynamic half-sweep, forward step j: the second right-hand side Y2 = min(D_L, 1) F_L of the
// left stack's top level, column-major into dynx
__global__ void __launch_bounds__(256) zdyn_prep_kernel(const WalkerDev* __restrict__ W, int j) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || !w.dynx || sp >= w.S || j >= w.nstack) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  const double* lv = stack_level(w, 0, sp, j);  // forward step j: left stack of j + 1 levels
  const double* F = lv + NN;
  const double* D = lv + 2 * NN;
  double* Y2 = w.dynx + sp * NN;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < NN; e += (long long)gridDim.x * 256) {
    const int r = (int)(e % N);
    Y2[e] = fmin(D[r], 1.0) * F[e];
  }
}

// dynamic half-sweep at t = beta (right stack empty): G(beta,0) = X2, G(0,beta) = -X, with
// their wrap errors against the propagated values
__global__ void __launch_bounds__(256) zdyn_boundary_kernel(const WalkerDev* __restrict__ W, int j) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (!w.ozstab || !w.gt0 || !w.dynx || sp >= w.S || j != w.nstack - 1) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  const ZScr z = zscr(w, sp);
  double* t0 = zdyn_slot(w.gt0, w, sp, w.Lt);
  double* ot = zdyn_slot(w.g0t, w, sp, w.Lt);
  const double* X2 = w.dynx + sp * NN;
  double err = 0.0;
  bool finite = true;
  for (long long e = blockIdx.x * 256LL + threadIdx.x; e < NN; e += (long long)gridDim.x * 256) {
    const double a = X2[e], b = -z.Y[e];
    err = fmax(err, fmax(fabs(a - t0[e]), fabs(b - ot[e])));
    if (!isfinite(a) || !isfinite(b)) finite = false;
    t0[e] = a;
    ot[e] = b;
  }
  if (!finite) atomicOr(w.status, ST_NONFINITE_G);
  for (int o = 16; o > 0; o >>= 1) err = fmax(err, __shfl_xor_sync(0xffffffffu, err, o));
  if ((threadIdx.x & 31) == 0) atomicMax(w.wrap_bits, (unsigned long long)__double_as_longlong(err));
}

// --------------------------------------------------------------------------
// host side
// --------------------------------------------------------------------------
// the two product configurations: 56 bits (K <= 256) and 54 bits (K <= 1024)
#define ZGEMM56 zgemm_tc_kernel<8, 7, 32, 2, 2>
#define ZGEMM54 zgemm_tc_kernel<9, 6, 32, 4, 1>
static size_t ztc_smem(int S, int NT, int NS) { return (size_t)NS * oztc::stage_bytes(S, 128, NT); }
static size_t zpanel_smem(int maxN) { return sizeof(double) * ((size_t)TB * maxN + TB * TB); }

cudaError_t configure_stab_oz_kernels(int maxN) {
  cudaError_t e;
  if ((e = cudaFuncSetAttribute(ZGEMM56, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ztc_smem(8, 32, 2))))
    return e;
  if ((e = cudaFuncSetAttribute(ZGEMM54, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ztc_smem(9, 32, 4))))
    return e;
  if ((e = cudaFuncSetAttribute(zqr_panel_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)zpanel_smem(maxN > 0 ? maxN : 1))))
    return e;
  return cudaSuccess;
}

static void zgemm(const WalkerDev* W, int nw, int maxN, int op, int mode, int j, int p, int rows_max, int cols_max,
                  int trace_slot, cudaStream_t st) {
  const dim3 gs((std::max(rows_max, cols_max) + 31) / 32, 2, 2 * nw);
  zslice_kernel<8, 7><<<gs, 256, 0, st>>>(W, op, mode, j, p);
  if (maxN > 256) zslice_kernel<9, 6><<<gs, 256, 0, st>>>(W, op, mode, j, p);
  const dim3 g((cols_max + 31) / 32, (rows_max + 127) / 128, 2 * nw);
  ZGEMM56<<<g, 256, ztc_smem(8, 32, 2), st>>>(W, op, mode, j, p, trace_slot);
  if (maxN > 256) ZGEMM54<<<g, 256, ztc_smem(9, 32, 4), st>>>(W, op, mode, j, p, trace_slot);
}

// Householder panel p: the FP64 column factorization, then its Gram matrix, T factor and
// Vt = V T (the block reflector in the form the trailing products apply)
static void zpanel(const WalkerDev* W, int nw, int maxN, int mode, int j, int p, int push, cudaStream_t st) {
  zqr_panel_kernel<<<2 * nw, 256, zpanel_smem(maxN), st>>>(W, mode, j, p, push);
  zgemm(W, nw, maxN, Z_GRAM, mode, j, p, TB, TB, -1, st);
  ztfac_kernel<<<2 * nw, 32, 0, st>>>(W, mode, j, p);
  zgemm(W, nw, maxN, Z_VT, mode, j, p, maxN, TB, -1, st);
}

void oz_push(int mode, const WalkerDev* W, int nw, int j, int maxN, cudaStream_t st) {
  const int np = (maxN + TB - 1) / TB;
  zpush_prep_kernel<<<2 * nw, 256, sizeof(long long) * maxN, st>>>(W, mode, j);
  for (int p = 0; p < np; ++p) {
    zpanel(W, nw, maxN, mode, j, p, 1, st);
    zgemm(W, nw, maxN, Z_QR_W, mode, j, p, TB, maxN, -1, st);
    zgemm(W, nw, maxN, Z_QR_UPD, mode, j, p, maxN, maxN, -1, st);
  }
  zpush_fin_kernel<<<dim3(64, 2 * nw), 256, 0, st>>>(W, mode, j);
  zgemm(W, nw, maxN, Z_F, mode, j, 0, maxN, maxN, -1, st);
  for (int p = np - 1; p >= 0; --p) {
    zvt_kernel<<<dim3((maxN + 31) / 32, 2 * nw), 256, 0, st>>>(W, mode, j, p);
    zgemm(W, nw, maxN, Z_Q_W, mode, j, p, TB, maxN, -1, st);
    zgemm(W, nw, maxN, Z_Q_UPD, mode, j, p, maxN, maxN, -1, st);
  }
}

// The Green's assembly; with dyn (forward steps of the dynamic half-sweep) the same
// factorization of M also solves the second right-hand side and G(t,0), G(0,t) follow.
void oz_greens(int mode, const WalkerDev* W, int nw, int j, int trace_slot, int maxN, cudaStream_t st, bool dyn) {
  const int np = (maxN + TB - 1) / TB;
  zgreens_prep_kernel<<<dim3(64, 2 * nw), 256, 0, st>>>(W, mode, j);
  if (dyn) zdyn_prep_kernel<<<dim3(64, 2 * nw), 256, 0, st>>>(W, j);
  zgemm(W, nw, maxN, Z_GA, mode, j, 0, maxN, maxN, -1, st);
  zgemm(W, nw, maxN, Z_GB, mode, j, 0, maxN, maxN, -1, st);
  for (int p = 0; p < np; ++p) {
    zpanel(W, nw, maxN, mode, j, p, 0, st);
    zgemm(W, nw, maxN, Z_QR_W, mode, j, p, TB, maxN, -1, st);
    zgemm(W, nw, maxN, Z_QR_UPD, mode, j, p, maxN, maxN, -1, st);
    zgemm(W, nw, maxN, Z_AQ_W, mode, j, p, TB, maxN, -1, st);
    zgemm(W, nw, maxN, Z_AQ_UPD, mode, j, p, maxN, maxN, -1, st);
    if (dyn) {
      zgemm(W, nw, maxN, Z_AQ2_W, mode, j, p, TB, maxN, -1, st);
      zgemm(W, nw, maxN, Z_AQ2_UPD, mode, j, p, maxN, maxN, -1, st);
    }
  }
  for (int p = np - 1; p >= 0; --p) {
    zgemm(W, nw, maxN, Z_TR_UPD, mode, j, p, TB, maxN, -1, st);
    ztrsm_diag_kernel<<<dim3((maxN + 127) / 128, 2 * nw), 128, 0, st>>>(W, mode, j, p, 0);
    if (dyn) {
      zgemm(W, nw, maxN, Z_TR2_UPD, mode, j, p, TB, maxN, -1, st);
      ztrsm_diag_kernel<<<dim3((maxN + 127) / 128, 2 * nw), 128, 0, st>>>(W, mode, j, p, 1);
    }
  }
  zgemm(W, nw, maxN, Z_GG, mode, j, 0, maxN, maxN, trace_slot, st);
  zgreens_out_kernel<<<dim3(64, 2 * nw), 256, 0, st>>>(W, mode, j, trace_slot);
  if (dyn) {
    zgemm(W, nw, maxN, Z_DT0_OUT, mode, j, 0, maxN, maxN, -1, st);
    zgemm(W, nw, maxN, Z_D0T_OUT, mode, j, 0, maxN, maxN, -1, st);
    zdyn_boundary_kernel<<<dim3(64, 2 * nw), 256, 0, st>>>(W, j);
  }
}

}  // namespace dqmc
