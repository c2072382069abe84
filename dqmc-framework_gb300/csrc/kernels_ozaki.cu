// kernels_ozaki.cu — the mixed-precision products of the sweep: FP64-accurate
// (49-bit) matrix products on the BF16 tensor cores (see ozaki.cuh).
//
// Slicing is integer work on the FP64 bit patterns; the product runs the
// S(S+1)/2 slice pairs on the BF16 tensor cores (tcgen05, TMEM accumulators;
// the stand-alone product of the test hook uses mma.sync) with FP32
// accumulation, exact by construction, one accumulator per weight group, and
// recombines the groups in the epilogue.  Used for the wraps and the B-chain (the reference's
// mult_B_from_left/right, mult_invB_*, mult_transB_from_left,
// src/model/repulsive_hubbard.cpp:158-243, src/model/model_base.cpp:7-35).
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "dqmc_device.cuh"
#include "ozaki.cuh"
#include "oz_tc.cuh"
#include "tcgen05.cuh"

namespace dqmc {

using ozaki::kMaxSlices;

// --------------------------------------------------------------------------
// Slicing.  role 0 (left operand, A): lines are rows r, k runs over columns.
// role 1 (right operand, B): lines are columns c, k runs over rows.  X is
// column-major N x N (ld N).  pre (may be null) scales element k of every line
// before slicing.  layout 0 writes out[s][line][k] (row-major, ld ldk); layout
// 1 writes the tensor-core image (ozaki::tc_index, slice stride
// ozaki::tc_slice_elems).  One CTA of 256 threads per 32 lines.
// --------------------------------------------------------------------------
struct SliceJob {
  const double* X;
  unsigned short* out;  // BF16 bits, S slices
  int* exps;            // [N]
  const double* pre;    // along k, or null
};

__device__ __forceinline__ double xelem(const double* X, int N, int role, int line, int k) {
  return role == 0 ? X[(long long)k * N + line] : X[(long long)line * N + k];
}

__device__ void slice_lines(const SliceJob& job, int N, int ldk, int role, int bits, int slices, int line0,
                            int layout) {
  __shared__ int s_e[8][32];
  __shared__ double s_t[32][33];
  const int tid = threadIdx.x;
  // pass 1: exponent per line (integer max of exponent bounds)
  {
    const int ll = (role == 0) ? (tid & 31) : (tid >> 3);   // line in block
    const int kg = (role == 0) ? (tid >> 5) : (tid & 7);    // k group of 8
    int e = -1100;
    const int line = line0 + ll;
    if (line < N)
      for (int k = kg; k < N; k += 8) {
        double x = xelem(job.X, N, role, line, k);
        if (job.pre) x *= job.pre[k];
        e = max(e, ozaki::exp_bound(x));
      }
    s_e[kg][ll] = e;
  }
  __syncthreads();
  if (tid < 32) {
    int e = s_e[0][tid];
    for (int g = 1; g < 8; ++g) e = max(e, s_e[g][tid]);
    s_e[0][tid] = e;
    if (line0 + tid < N) job.exps[line0 + tid] = e;
  }
  __syncthreads();
  // pass 2: 32 x 32 tiles, staged so the BF16 writes run along k
  for (int k0 = 0; k0 < ldk; k0 += 32) {
    for (int e2 = tid; e2 < 32 * 32; e2 += blockDim.x) {
      int ll, kk;
      if (role == 0) { ll = e2 & 31; kk = e2 >> 5; } else { kk = e2 & 31; ll = e2 >> 5; }
      const int line = line0 + ll, k = k0 + kk;
      double x = 0.0;
      if (line < N && k < N) {
        x = xelem(job.X, N, role, line, k);
        if (job.pre) x *= job.pre[k];
      }
      s_t[ll][kk] = x;
    }
    __syncthreads();
    const int Q = bits * slices;
    if (layout == 0) {
      for (int e2 = tid; e2 < 32 * 32; e2 += blockDim.x) {
        const int kk = e2 & 31, ll = e2 >> 5;
        const int line = line0 + ll, k = k0 + kk;
        if (line < N && k < ldk) {
          bool neg;
          const unsigned long long q = ozaki::fixedq(s_t[ll][kk], s_e[0][ll], Q, neg);
          for (int s = 0; s < slices; ++s)
            job.out[((long long)s * N + line) * ldk + k] = ozaki::slice_bf16q(q, s, bits, Q, neg);
        }
      }
    } else {
      // one line and 4 consecutive k per thread: one 8-byte store per slice
      const int kq = tid & 7, ll = tid >> 3;
      const int line = line0 + ll, k = k0 + kq * 4;
      if (line < N && k < ldk) {
        unsigned long long q[4];
        bool ng[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) q[u] = ozaki::fixedq(s_t[ll][kq * 4 + u], s_e[0][ll], Q, ng[u]);
        const long long sstride = (long long)ozaki::tc_slice_elems(N, ldk);
        unsigned short* o = job.out + ozaki::tc_index(line, k, ozaki::tc_lines(N) / 8);
        for (int s = 0; s < slices; ++s) {
          ushort4 v;
          v.x = ozaki::slice_bf16q(q[0], s, bits, Q, ng[0]);
          v.y = ozaki::slice_bf16q(q[1], s, bits, Q, ng[1]);
          v.z = ozaki::slice_bf16q(q[2], s, bits, Q, ng[2]);
          v.w = ozaki::slice_bf16q(q[3], s, bits, Q, ng[3]);
          *reinterpret_cast<ushort4*>(o + s * sstride) = v;
        }
      }
    }
    __syncthreads();
  }
}

// --------------------------------------------------------------------------
// Product kernel: C(r,c) = sum_k A(r,k) B(k,c) from slices, 64x64 tile per
// CTA, 8 warps (2 x 4), warp tile 32 x 16, K staged 16 at a time (cp.async,
// double buffered).  The epilogue functor receives (r, c, value).
// --------------------------------------------------------------------------
struct ProdJob {
  const unsigned short* A;  // S slices: [S][N][ldk] (test hook) or tensor-core images (sweep)
  const unsigned short* B;
  const int* ea;
  const int* eb;
};

constexpr int kOzRow = 24;  // padded SMEM row (bf16): 48 bytes, conflict-free fragment loads

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::); }

__device__ __forceinline__ void mma_bf16(float (&c)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

template <int S, class Epi>
__device__ void ozaki_product_tile(const ProdJob& job, int N, int ldk, int bits, int r0, int c0, unsigned short* sm,
                                   Epi epi) {
  // sm: [2 stages][2 operands][S][64][kOzRow]
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  const int wm = wid >> 2, wn = wid & 3;  // warp tile origin (wm*32, wn*16)
  const int g = lane >> 2, t4 = lane & 3;
  float acc[S][2][2][4];  // weight groups m = i + j <= S - 1
#pragma unroll
  for (int m = 0; m < S; ++m)
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
      for (int b = 0; b < 2; ++b)
#pragma unroll
        for (int v = 0; v < 4; ++v) acc[m][a][b][v] = 0.f;

  const int stage_elems = 2 * S * 64 * kOzRow;
  auto load_stage = [&](int st, int k0) {
    unsigned short* base = sm + st * stage_elems;
    // 2 operands x S slices x 64 lines x 2 chunks of 16 bytes
    for (int e = tid; e < 2 * S * 64 * 2; e += blockDim.x) {
      const int ch = e & 1, line = (e >> 1) & 63, s = (e >> 7) % S, op = (e >> 7) / S;
      const int gl = (op == 0 ? r0 : c0) + line;
      const unsigned short* src = (op == 0 ? job.A : job.B) + ((long long)s * N + min(gl, N - 1)) * ldk + k0 + ch * 8;
      unsigned short* dst = base + ((op * S + s) * 64 + line) * kOzRow + ch * 8;
      cp_async16(dst, src, gl < N);
    }
    cp_async_commit();
  };

  const int nk = ldk / 16;
  load_stage(0, 0);
  for (int kb = 0; kb < nk; ++kb) {
    cp_async_wait_all();
    __syncthreads();
    if (kb + 1 < nk) load_stage((kb + 1) & 1, (kb + 1) * 16);
    const unsigned short* As = sm + (kb & 1) * stage_elems;
    const unsigned short* Bs = As + S * 64 * kOzRow;
#pragma unroll
    for (int i = 0; i < S; ++i) {
      unsigned a[2][4];
#pragma unroll
      for (int mt = 0; mt < 2; ++mt) {
        const unsigned short* p = As + (i * 64 + wm * 32 + mt * 16 + g) * kOzRow + 2 * t4;
        a[mt][0] = *(const unsigned*)(p);
        a[mt][1] = *(const unsigned*)(p + 8 * kOzRow);
        a[mt][2] = *(const unsigned*)(p + 8);
        a[mt][3] = *(const unsigned*)(p + 8 * kOzRow + 8);
      }
#pragma unroll
      for (int jj = 0; jj < S - i; ++jj) {
        unsigned b[2][2];
#pragma unroll
        for (int nt = 0; nt < 2; ++nt) {
          const unsigned short* p = Bs + (jj * 64 + wn * 16 + nt * 8 + g) * kOzRow + 2 * t4;
          b[nt][0] = *(const unsigned*)(p);
          b[nt][1] = *(const unsigned*)(p + 8);
        }
#pragma unroll
        for (int mt = 0; mt < 2; ++mt)
#pragma unroll
          for (int nt = 0; nt < 2; ++nt)
            mma_bf16(acc[i + jj][mt][nt], a[mt][0], a[mt][1], a[mt][2], a[mt][3], b[nt][0], b[nt][1]);
      }
    }
    __syncthreads();
  }
  // epilogue: C = 2^{ea_r + eb_c} sum_m 2^{-bits (m+2)} S_m
#pragma unroll
  for (int mt = 0; mt < 2; ++mt)
#pragma unroll
    for (int nt = 0; nt < 2; ++nt)
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        const int r = r0 + wm * 32 + mt * 16 + g + ((v >> 1) << 3);
        const int c = c0 + wn * 16 + nt * 8 + 2 * t4 + (v & 1);
        if (r >= N || c >= N) continue;
        // integer Horner in two halves (groups 0-3 and 4..S-1), each exact in 64 bits
        long long hi = 0, lo = 0;
#pragma unroll
        for (int m = 0; m < 4; ++m) hi = (hi << bits) + (long long)__float2int_rn(acc[m][mt][nt][v]);
#pragma unroll
        for (int m = 4; m < S; ++m) lo = (lo << bits) + (long long)__float2int_rn(acc[m][mt][nt][v]);
        const int e = job.ea[r] + job.eb[c];
        epi(r, c, ozaki::ldexp_i64(hi, e - 5 * bits) + ozaki::ldexp_i64(lo, e - bits * (S + 1)));
      }
}

}  // namespace dqmc

namespace dqmc {

namespace {
__device__ __forceinline__ bool oz_slice_of(const WalkerDev& w, int mode, int j, int q, int& t) {
  if (j >= w.nstack) return false;
  const int k = (mode == MODE_FWD) ? j : (w.nstack - 1 - j);
  const int t_lo = k * w.pace + 1, t_hi = min((k + 1) * w.pace, w.Lt);
  if (q >= t_hi - t_lo + 1) return false;
  t = (mode == MODE_FWD) ? t_lo + q : t_hi - q;
  return true;
}
__device__ __forceinline__ double oz_bscale(const WalkerDev& w, int t, int spin, int sgn, int i) {
  const int sf = (w.model == 0 && spin == 1) ? -1 : 1;
  const int s = w.fields[(long long)(t - 1) * w.N + i];
  return (sgn * sf * s > 0) ? w.e_pa : w.e_ma;
}
__device__ __forceinline__ double* oz_chain(const WalkerDev& w, int spin, int which) {
  return w.chain + ((long long)which * w.S + spin) * w.N * w.N;
}
}  // namespace

// Operations of one slice (same meaning as gemm_op_kernel's):
//   OZ_WL_FWD  work   = diag(e+) expK G          (A: expK const, B: G)
//   OZ_WR_FWD  G      = work expK^-1 diag(e-)    (A: work,       B: invK const)
//   OZ_CH_FWD  chain' = diag(e+) expK chain      (A: expK const, B: chain)
//   OZ_CH_BWD  chain' = expK^T diag(e+) chain    (A: expK^T = expK as B-slices, B: diag(e+) chain)
//   OZ_WR_BWD  work   = G diag(e+) expK          (A: G diag(e+), B: expK const)
//   OZ_WL_BWD  G      = expK^-1 diag(e-) work    (A: invK const, B: diag(e-) work)
// and the time-displaced steps of the dynamic half-sweep (the reference's
// mult_B_from_left and mult_invB_from_right, src/dqmc_walker.cpp:455-466), on the
// ping-pong slots [parity][S][N*N] of G(t,0) and G(0,t):
//   OZ_DT0     G(t,0) = diag(e+) expK G(t-1,0)   (A: expK const, B: G(t-1,0))
//   OZ_D0T     G(0,t) = G(0,t-1) expK^-1 diag(e-) (A: G(0,t-1),   B: invK const)
enum OzOp { OZ_WL_FWD = 0, OZ_WR_FWD = 1, OZ_CH_FWD = 2, OZ_CH_BWD = 3, OZ_WR_BWD = 4, OZ_WL_BWD = 5,
            OZ_DT0 = 6, OZ_D0T = 7 };

__device__ __forceinline__ double* oz_dyn(double* base, const WalkerDev& w, int spin, int t) {
  return base + ((long long)(t & 1) * w.S + spin) * w.N * w.N;
}

// slice the per-walker operand of op OP: grid (ceil(N/32), 2*nw), 256 threads
template <int OP>
__global__ void __launch_bounds__(256) oz_slice_kernel(const WalkerDev* __restrict__ W, int mode, int j, int q) {
  const int wi = blockIdx.y >> 1, sp = blockIdx.y & 1;
  const WalkerDev& w = W[wi];
  if (w.path != 2 || w.cb || sp >= w.S) return;
  int t;
  if (!oz_slice_of(w, mode, j, q, t)) return;
  const int N = w.N;
  const long long NN = (long long)N * N;
  __shared__ double s_pre[1024];
  int role = 1, sgn = 0;
  const double* X = nullptr;
  switch (OP) {
    case OZ_WL_FWD: X = w.G + sp * NN; role = 1; break;
    case OZ_WR_FWD: X = w.work + sp * NN; role = 0; break;
    case OZ_CH_FWD: X = oz_chain(w, sp, q & 1); role = 1; break;
    case OZ_CH_BWD: X = oz_chain(w, sp, q & 1); role = 1; sgn = +1; break;
    case OZ_WR_BWD: X = w.G + sp * NN; role = 0; sgn = +1; break;
    case OZ_WL_BWD: X = w.work + sp * NN; role = 1; sgn = -1; break;
    case OZ_DT0: X = w.gt0 ? oz_dyn(w.gt0, w, sp, t - 1) : nullptr; role = 1; break;
    case OZ_D0T: X = w.g0t ? oz_dyn(w.g0t, w, sp, t - 1) : nullptr; role = 0; break;
  }
  if (!X) return;
  if (sgn)
    for (int k = threadIdx.x; k < N; k += blockDim.x) s_pre[k] = oz_bscale(w, t, sp, sgn, k);
  __syncthreads();
  SliceJob job{X, w.sl + (long long)sp * w.slices * ozaki::tc_slice_elems(N, w.ldk), w.sle + (long long)sp * N,
               sgn ? s_pre : nullptr};
  slice_lines(job, N, w.ldk, role, w.slice_bits, w.slices, blockIdx.x * 32, 1);
}

// Product of op OP on the 5th-generation tensor cores: a 128 x NT output
// tile per CTA with the S weight groups accumulated in TMEM (S x NT columns),
// the operands streamed by oztc::mainloop (bulk copies through a ring of NS
// stages of 16-deep k chunks).  Two tile shapes per slice configuration, picked
// per batch by the autotuner (dqmc_init_greens): 128 x 32 tiles, two CTAs per SM
// (at most 256 TMEM columns, 105 KB (7 slices, 3 stages) or 80 KB (8 slices, 2
// stages) of shared memory and 128 registers each), or 128 x 64 tiles, one CTA
// per SM (512 TMEM columns, 3 or 4 stages).  Shape SH = 0 is 128 x 32 for the
// 49-bit configuration (7 slices, K <= 256) and 128 x 64 for the 48-bit one (8
// slices); SH = 1 swaps them.
__host__ __device__ constexpr int oz_tc_nt(int S, int SH) { return ((S <= 7) == (SH == 0)) ? 32 : 64; }
__host__ __device__ constexpr int oz_tc_stages(int S, int SH) {
  return oz_tc_nt(S, SH) == 32 ? (S <= 7 ? 3 : 2) : (S <= 7 ? 3 : 4);
}
__host__ __device__ constexpr int oz_tc_minb(int S, int SH) { return oz_tc_nt(S, SH) == 32 ? 2 : 1; }
__host__ __device__ constexpr int oz_tc_stage_bytes(int S, int SH) {
  return oztc::stage_bytes(S, 128, oz_tc_nt(S, SH));
}

template <int OP, int S, int SH>
__global__ void __launch_bounds__(256, oz_tc_minb(S, SH)) oz_prod_tc_kernel(const WalkerDev* __restrict__ W, int mode,
                                                                            int j, int q) {
  constexpr int MT = 128, NT = oz_tc_nt(S, SH), NS = oz_tc_stages(S, SH);
  constexpr int CW = (oz_tc_minb(S, SH) > 1) ? 8 : 16;  // TMEM columns per load in the epilogue
  constexpr unsigned TCOLS = (S * NT <= 256) ? 256u : 512u;
  const int wi = blockIdx.z >> 1, sp = blockIdx.z & 1;
  const WalkerDev& w = W[wi];
  if (w.path != 2 || w.cb || sp >= w.S || w.slices != S) return;
  int t;
  if (!oz_slice_of(w, mode, j, q, t)) return;
  const int N = w.N, ldk = w.ldk;
  const int r0 = blockIdx.y * MT, c0 = blockIdx.x * NT;
  if (r0 >= N || c0 >= N) return;
  const long long NN = (long long)N * N;
  const long long sstride = (long long)ozaki::tc_slice_elems(N, ldk);
  const unsigned short* ws = w.sl + (long long)sp * w.slices * sstride;
  const int* we = w.sle + (long long)sp * N;
  ProdJob job{};
  double* out = nullptr;
  switch (OP) {
    case OZ_WL_FWD: job = ProdJob{w.kA, ws, w.kAe, we}; out = w.work + sp * NN; break;
    case OZ_WR_FWD: job = ProdJob{ws, w.iB, we, w.iBe}; out = w.G + sp * NN; break;
    case OZ_CH_FWD: job = ProdJob{w.kA, ws, w.kAe, we}; out = oz_chain(w, sp, (q + 1) & 1); break;
    case OZ_CH_BWD: job = ProdJob{w.kB, ws, w.kBe, we}; out = oz_chain(w, sp, (q + 1) & 1); break;
    case OZ_WR_BWD: job = ProdJob{ws, w.kB, we, w.kBe}; out = w.work + sp * NN; break;
    case OZ_WL_BWD: job = ProdJob{w.iA, ws, w.iAe, we}; out = w.G + sp * NN; break;
    case OZ_DT0: job = ProdJob{w.kA, ws, w.kAe, we}; out = w.gt0 ? oz_dyn(w.gt0, w, sp, t) : nullptr; break;
    case OZ_D0T: job = ProdJob{ws, w.iB, we, w.iBe}; out = w.g0t ? oz_dyn(w.g0t, w, sp, t) : nullptr; break;
  }
  if (!out) return;
  extern __shared__ __align__(1024) unsigned char tsm[];
  __shared__ int eA[MT], eB[NT];
  __shared__ double s_scale[MT];  // exp(+-alpha s) of the output rows (or columns)
  __shared__ __align__(8) unsigned long long full[NS], done[NS];
  __shared__ unsigned tbase;
  __shared__ int s_fail, s_last;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  if (tid < MT) eA[tid] = (r0 + tid < N) ? job.ea[r0 + tid] : -1100;
  if (tid < NT) eB[tid] = (c0 + tid < N) ? job.eb[c0 + tid] : -1100;
  if (OP == OZ_WL_FWD || OP == OZ_CH_FWD || OP == OZ_DT0) {
    if (tid < MT) s_scale[tid] = (r0 + tid < N) ? oz_bscale(w, t, sp, +1, r0 + tid) : 0.0;
  } else if (OP == OZ_WR_FWD || OP == OZ_D0T) {
    if (tid < NT) s_scale[tid] = (c0 + tid < N) ? oz_bscale(w, t, sp, -1, c0 + tid) : 0.0;
  }
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
    // chunk c of the tile: (c * nlb + line0 / 8) 8-line blocks of 128 elements into each slice
    const long long cstep = (long long)(ozaki::tc_lines(N) / 8) * 128;
    bool ok;
    s_last = oztc::mainloop<S, MT, NT, NS>(tsm, full, done, taddr, job.A + (long long)(r0 / 8) * 128,
                                            job.B + (long long)(c0 / 8) * 128, sstride, cstep, ldk / 16, ok,
                                            w.wait_limit);
    s_fail = ok ? 0 : 1;
  }
  __syncthreads();
  const int last = s_last;
  const bool mma_done = last >= 0 && tc::mbar_wait(&done[last % NS], (last / NS) & 1);
  const int failed = __syncthreads_or(!mma_done || s_fail);
  tc::fence_after();
  constexpr int SB = (S <= 7) ? 7 : 6;  // bits per slice of the configuration (ozaki::cfg_for_k)
  const int q4 = warp & 3, half = warp >> 2;
  const int rl = q4 * 32 + lane, r = r0 + rl;
  if (!failed) {
    for (int cc = half * (NT / 2); cc < (half + 1) * (NT / 2); cc += CW) {
      uint32_t v[S][CW];
#pragma unroll
      for (int m = 0; m < S; ++m) tc::ldw<CW>(v[m], taddr + ((unsigned)(q4 * 32) << 16) + (unsigned)(m * NT + cc));
      tc::wait_ld();
      if (r < N) {
#pragma unroll
        for (int u = 0; u < CW; ++u) {
          const int cl = cc + u, col = c0 + cl;
          if (col >= N) continue;
          long long hi = 0, lo = 0;
#pragma unroll
          for (int m = 0; m < 4; ++m) hi = (hi << SB) + (long long)__float2int_rn(__uint_as_float(v[m][u]));
#pragma unroll
          for (int m = 4; m < S; ++m) lo = (lo << SB) + (long long)__float2int_rn(__uint_as_float(v[m][u]));
          const int e = eA[rl] + eB[cl];
          double val = ozaki::combine_hilo<S, (S <= 7 ? 7 : 6)>(hi, lo, e);
          if (OP == OZ_WL_FWD || OP == OZ_CH_FWD || OP == OZ_DT0) val *= s_scale[rl];
          if (OP == OZ_WR_FWD || OP == OZ_D0T) val *= s_scale[cl];
          out[(long long)col * N + r] = val;
        }
      }
    }
  } else if (tid == 0) {
    atomicOr(w.status, ST_TIMEOUT);
  }
  tc::fence_before();
  __syncthreads();
  if (warp == 0) tc::dealloc(taddr, TCOLS);
}

// constant operands (exp(-dtau K), exp(+dtau K)), sliced once per batch
__global__ void __launch_bounds__(256) oz_const_slice_kernel(const double* X, unsigned short* out, int* exps, int N,
                                                             int ldk, int role, int bits, int slices, int layout) {
  SliceJob job{X, out, exps, nullptr};
  slice_lines(job, N, ldk, role, bits, slices, blockIdx.x * 32, layout);
}

// stand-alone product C = A B (test hook): A, B column-major N x N on the device
__global__ void __launch_bounds__(256) oz_selftest_prod_kernel(const unsigned short* As, const int* ea,
                                                               const unsigned short* Bs, const int* eb, double* C,
                                                               int N, int ldk, int bits, int S) {
  extern __shared__ unsigned short ozsm[];
  ProdJob job{As, Bs, ea, eb};
  const int r0 = blockIdx.y * 64, c0 = blockIdx.x * 64;
  auto epi = [&](int r, int c, double v) { C[(long long)c * N + r] = v; };
  if (S == 7) ozaki_product_tile<7>(job, N, ldk, bits, r0, c0, ozsm, epi);
  else ozaki_product_tile<8>(job, N, ldk, bits, r0, c0, ozsm, epi);
}

static size_t oz_tc_smem(int S, int SH) { return (size_t)oz_tc_stages(S, SH) * oz_tc_stage_bytes(S, SH); }
size_t oz_prod_smem(int S) { return sizeof(unsigned short) * 2 * 2 * S * 64 * kOzRow; }

cudaError_t configure_ozaki_kernels() {
  cudaError_t e;
#define OZCFG(OP)                                                                                         \
  if ((e = cudaFuncSetAttribute(oz_prod_tc_kernel<OP, 7, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                (int)oz_tc_smem(7, 0))) ||                                                 \
      (e = cudaFuncSetAttribute(oz_prod_tc_kernel<OP, 8, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                (int)oz_tc_smem(8, 0))) ||                                                 \
      (e = cudaFuncSetAttribute(oz_prod_tc_kernel<OP, 7, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                (int)oz_tc_smem(7, 1))) ||                                                 \
      (e = cudaFuncSetAttribute(oz_prod_tc_kernel<OP, 8, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,  \
                                (int)oz_tc_smem(8, 1))))                                                   \
  return e
  OZCFG(OZ_WL_FWD); OZCFG(OZ_WR_FWD); OZCFG(OZ_CH_FWD); OZCFG(OZ_CH_BWD);
  OZCFG(OZ_WR_BWD); OZCFG(OZ_WL_BWD); OZCFG(OZ_DT0); OZCFG(OZ_D0T);
#undef OZCFG
  if ((e = cudaFuncSetAttribute(oz_selftest_prod_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)oz_prod_smem(8))))
    return e;
  return cudaSuccess;
}

// tile shape of the products issued by this host thread (the issuing batch's tuned shape)
static thread_local int g_oz_shape = 0;
void oz_set_shape(int shape) { g_oz_shape = shape ? 1 : 0; }

template <int OP, int SH>
static void oz_op_shape(const WalkerDev* W, int nw, int maxN, int mode, int j, int q, cudaStream_t st) {
  const dim3 g7((maxN + oz_tc_nt(7, SH) - 1) / oz_tc_nt(7, SH), (maxN + 127) / 128, 2 * nw);
  oz_prod_tc_kernel<OP, 7, SH><<<g7, 256, oz_tc_smem(7, SH), st>>>(W, mode, j, q);
  if (maxN > 256) {
    const dim3 g8((maxN + oz_tc_nt(8, SH) - 1) / oz_tc_nt(8, SH), (maxN + 127) / 128, 2 * nw);
    oz_prod_tc_kernel<OP, 8, SH><<<g8, 256, oz_tc_smem(8, SH), st>>>(W, mode, j, q);
  }
}

template <int OP>
static void oz_op(const WalkerDev* W, int nw, int maxN, int mode, int j, int q, cudaStream_t st) {
  oz_slice_kernel<OP><<<dim3((maxN + 31) / 32, 2 * nw), 256, 0, st>>>(W, mode, j, q);
  if (g_oz_shape) oz_op_shape<OP, 1>(W, nw, maxN, mode, j, q, st);
  else oz_op_shape<OP, 0>(W, nw, maxN, mode, j, q, st);
}

// the slice work of mixed walkers (wraps and chain through the tensor cores)
void mixed_wrap_fwd(const WalkerDev* W, int nw, int maxN, int j, int q, cudaStream_t st) {
  oz_op<OZ_WL_FWD>(W, nw, maxN, MODE_FWD, j, q, st);
  oz_op<OZ_WR_FWD>(W, nw, maxN, MODE_FWD, j, q, st);
}
void mixed_chain(const WalkerDev* W, int nw, int maxN, int mode, int j, int q, cudaStream_t st) {
  if (mode == MODE_FWD) oz_op<OZ_CH_FWD>(W, nw, maxN, mode, j, q, st);
  else oz_op<OZ_CH_BWD>(W, nw, maxN, mode, j, q, st);
}
// the time-displaced steps of the dynamic half-sweep for mixed walkers
void mixed_dynamic_prop(const WalkerDev* W, int nw, int maxN, int j, int q, cudaStream_t st) {
  oz_op<OZ_DT0>(W, nw, maxN, MODE_FWD, j, q, st);
  oz_op<OZ_D0T>(W, nw, maxN, MODE_FWD, j, q, st);
}
void mixed_wrap_bwd(const WalkerDev* W, int nw, int maxN, int j, int q, cudaStream_t st) {
  oz_op<OZ_WR_BWD>(W, nw, maxN, MODE_BWD, j, q, st);
  oz_op<OZ_WL_BWD>(W, nw, maxN, MODE_BWD, j, q, st);
}

void oz_slice_const(const double* X, unsigned short* out, int* exps, int N, int ldk, int role, int bits, int slices,
                    int layout, cudaStream_t st) {
  oz_const_slice_kernel<<<(N + 31) / 32, 256, 0, st>>>(X, out, exps, N, ldk, role, bits, slices, layout);
}

void oz_selftest(const double* A, const double* B, double* C, unsigned short* sa, int* ea, unsigned short* sb, int* eb,
                 int N, cudaStream_t st) {
  const ozaki::SliceCfg cfg = ozaki::cfg_for_k(N);
  const int ldk = (N + 15) / 16 * 16;
  oz_slice_const(A, sa, ea, N, ldk, 0, cfg.bits, cfg.slices, 0, st);
  oz_slice_const(B, sb, eb, N, ldk, 1, cfg.bits, cfg.slices, 0, st);
  const int t = (N + 63) / 64;
  oz_selftest_prod_kernel<<<dim3(t, t), 256, oz_prod_smem(cfg.slices), st>>>(sa, ea, sb, eb, C, N, ldk, cfg.bits,
                                                                             cfg.slices);
}

}  // namespace dqmc
