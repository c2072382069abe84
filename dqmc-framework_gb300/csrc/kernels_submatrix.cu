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
// on the 5th-generation tensor cores through exact 42-bit integer slices
// (ozaki.cuh; K <= 32 per flush): T = Gamma R_A (m x N), then
// G -= G0(:,I_A) T (N x N, K = m).  Both run as a pipelined tile loop: one
// thread stages the slices (bulk copies into shared memory, B tiles two
// ahead) and issues the MMAs of tile t+1 into one of two TMEM accumulators
// while all warps run the epilogue of tile t from the other.  The epilogue of
// T slices T directly (per-column exponents by warp reductions), so T never
// exists in FP64 outside registers.
//
// The decisions use the reference's ratio formula, evaluated with the same
// rounded operations, and the same uniform per site; G reaches them through
// a different but equivalent sequence of updates, so they agree with the
// reference's unless a ratio lies within rounding of its uniform.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "dqmc_device.cuh"
#include "ozaki.cuh"
#include "tcgen05.cuh"

namespace dqmc {

namespace {

constexpr int kSubThreads = 256;             // worker threads: decisions, slicing, epilogues
constexpr int kSubCTA = kSubThreads + 32;     // + one producer warp (bulk copies and MMAs)
constexpr int KB = 32;           // sites per block
constexpr int KK = KB * KB;
constexpr int OZS = 6, OZB = 7;  // 6 slices of 7 bits; group sums < 2^22 for K <= 32
// tensor-core tiles: 128 rows x 32 columns, K = 32 in two chunks of 16
constexpr int TM = 128, TN = 32;
constexpr int A_BYTES = OZS * 2 * TM * 32;  // A operand: [slice][chunk][128 lines x 16 k]
constexpr int B_BYTES = OZS * 2 * TN * 32;  // one B tile: [slice][chunk][32 lines x 16 k]
constexpr int NBB = 3;                      // B tiles in flight (loads run two tiles ahead)
constexpr int ACC_COLS = OZS * TN;          // TMEM columns of one accumulator (6 weight groups)
constexpr unsigned TMEM_COLS = 512;         // two accumulators

__host__ __device__ inline size_t al256(size_t x) { return (x + 255) & ~(size_t)255; }

// barrier of the eight worker warps alone (named barrier 1); __syncthreads joins the producer
__device__ __forceinline__ void wsync() { asm volatile("bar.sync 1, %0;" ::"n"(kSubThreads) : "memory"); }

// per-spin scratch in HBM (WalkerDev::msub): the operands' slices as tensor-core
// images (ozaki::tc_index, k stride 32) and the line exponents
struct SubOff {
  size_t sGm, sG, sR, sT, eGm, eG, eR, eT, mc, total;
};
__host__ __device__ inline size_t sub_sst(int N) { return (size_t)ozaki::tc_lines(N) * KB; }
__host__ __device__ inline SubOff sub_offsets(int N) {
  SubOff o;
  const size_t img = al256(OZS * sub_sst(N) * sizeof(unsigned short));
  o.sGm = 0;                                             // Gamma, lines = rows x (128-line image)
  o.sG = al256(OZS * sub_sst(1) * sizeof(unsigned short));  // G0(:, I_A), lines = rows
  o.sR = o.sG + img;                                     // R_A, lines = columns c
  o.sT = o.sR + img;                                     // T, lines = columns c
  o.eGm = o.sT + img;
  o.eG = o.eGm + al256(KB * sizeof(int));
  o.eR = o.eG + al256((size_t)N * sizeof(int));
  o.eT = o.eR + al256((size_t)N * sizeof(int));
  o.mc = o.eT + al256((size_t)N * sizeof(int));  // accepts of the current block (split kernels, spin 0's)
  o.total = o.mc + 256;
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

// Slices nlines lines x K (<= KB) of NOP operands (1 or 2) into their tensor-core images
// dst[o] (slice stride sst, nlb 8-line blocks per k chunk; k past K written as zeros) with one
// exponent per line (ex[o][line]); get(o, line, k) is the FP64 element.  The worker threads
// take part; 4 threads per line, 8 k each, both operands' loads in flight together.
// etmp: [2][256] scratch.
template <int NOP, class Get>
__device__ void slice_lines(Get get, int nlines, int K, unsigned short* const* dst, long long sst, int nlb,
                            int* const* ex, int* etmp) {
  const int tid = threadIdx.x, ll = tid & 63, part = tid >> 6;
  for (int l0 = 0; l0 < nlines; l0 += 64) {
    const int line = l0 + ll;
    double v[NOP][8];
    int e[NOP];
#pragma unroll
    for (int o = 0; o < NOP; ++o) {
      e[o] = -1100;
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const int k = part * 8 + u;
        v[o][u] = (line < nlines && k < K) ? get(o, line, k) : 0.0;
      }
    }
#pragma unroll
    for (int o = 0; o < NOP; ++o) {
#pragma unroll
      for (int u = 0; u < 8; ++u) e[o] = max(e[o], ozaki::exp_bound(v[o][u]));
      etmp[o * 256 + part * 64 + ll] = e[o];
    }
    wsync();
#pragma unroll
    for (int o = 0; o < NOP; ++o) {
      const int* et = etmp + o * 256;
      e[o] = max(max(et[ll], et[64 + ll]), max(et[128 + ll], et[192 + ll]));
    }
    if (line < nlines) {
#pragma unroll
      for (int o = 0; o < NOP; ++o) {
        if (part == 0) ex[o][line] = e[o];
        unsigned pk[OZS][4];
#pragma unroll
        for (int u = 0; u < 8; u += 2) {
          bool n0, n1;
          const unsigned long long q0 = ozaki::fixed42(v[o][u], e[o], n0), q1 = ozaki::fixed42(v[o][u + 1], e[o], n1);
#pragma unroll
          for (int s = 0; s < OZS; ++s)
            pk[s][u >> 1] = (unsigned)ozaki::slice_bf16(q0, s, OZB, n0) |
                            ((unsigned)ozaki::slice_bf16(q1, s, OZB, n1) << 16);
        }
        unsigned short* out = dst[o] + ozaki::tc_index(line, part * 8, nlb);
#pragma unroll
        for (int s = 0; s < OZS; ++s)
          *reinterpret_cast<uint4*>(out + s * sst) = make_uint4(pk[s][0], pk[s][1], pk[s][2], pk[s][3]);
      }
    }
    wsync();
  }
}

// The integer value sum_m S_m 2^(7 (5 - m)) of this thread's element of column u
// from the six weight-group sums S_m (exact FP32 integers, |S_m| < 2^22): the
// groups are read as integers through the 1.5 2^23 bias, combined in pairs
// P = 128 S_a + S_b (|P| < 2^30) in 32 bits, and the three pairs in 64.
__device__ __forceinline__ long long group_sum(const uint32_t (&v)[OZS][8], int u) {
  static_assert(OZS == 6 && OZB == 7, "pairing assumes six 7-bit groups");
  constexpr unsigned kBias = 0x4B400000u;  // bits of 1.5 2^23
  unsigned b[OZS];
#pragma unroll
  for (int m = 0; m < OZS; ++m) b[m] = __float_as_uint(__uint_as_float(v[m][u]) + 12582912.0f);
  const int p01 = (int)(b[0] * 128u + b[1] - 129u * kBias);
  const int p23 = (int)(b[2] * 128u + b[3] - 129u * kBias);
  const int p45 = (int)(b[4] * 128u + b[5] - 129u * kBias);
  return ((long long)p01 << 28) + ((long long)p23 << 14) + (long long)p45;
}

// The tile loop of one product, C = A B with A: nrb row blocks of 128 lines, B:
// the column tiles cb0, cb0 + cbs, ... < nct of 32 lines, K = 16 nk, both as
// tensor-core images in global memory (slice stride a_sst / b_sst, a_nlb / b_nlb
// line blocks per k chunk).  Called by all kSubCTA threads.  Tile u (global count
// across products) uses B buffer u % NBB and TMEM accumulator u & 1.  The
// producer (the first thread of the last warp) copies A at each row block and the
// B tiles two ahead, waits until the epilogue of tile u - 2 has read its
// accumulator, issues the MMAs of tile u and commits them to mmab[u & 1] and to the
// B buffer's bfree.  The eight worker warps run pre(row block, column tile, t + 1)
// (copies the next tile's epilogue needs that do not depend on the product), wait
// for the MMAs of tile t, run epi(row block, column tile, TMEM address, ok, t,
// t + 1 < tiles) and arrive on accfree[u & 1]; pre(.., 0) runs before the loop.
// The workers and the producer meet only through the mbarriers, and at the end.
struct SubTC {
  unsigned char* A;            // A_BYTES
  unsigned char* B;            // NBB x B_BYTES
  unsigned long long* ldA;     // [1]
  unsigned long long* ldB;     // [NBB]
  unsigned long long* mmab;    // [2] MMAs of the tile in accumulator a done
  unsigned long long* bfree;   // [NBB] MMAs reading B buffer b done
  unsigned long long* accfree; // [2] epilogue of the tile in accumulator a done (8 arrivals)
  unsigned tmem;
  volatile int* fail;          // shared flag: a bounded wait ran out
};

// the mbarriers of a SubTC, initialised by one thread
__device__ __forceinline__ void sub_tc_init(unsigned long long* ldA, unsigned long long* ldB, unsigned long long* mmab,
                                            unsigned long long* bfree, unsigned long long* accfree) {
  tc::mbar_init(ldA);
  for (int i = 0; i < NBB; ++i) {
    tc::mbar_init(&ldB[i]);
    tc::mbar_init(&bfree[i]);
  }
  for (int i = 0; i < 2; ++i) {
    tc::mbar_init(&mmab[i]);
    tc::mbar_init_n(&accfree[i], kSubThreads / 32);
  }
  tc::mbar_fence_init();
}

template <class Pre, class Epi>
__device__ void sub_gemm(const SubTC& tc, unsigned& gt, unsigned& nA, const unsigned short* aG, long long a_sst,
                         int a_nlb, int nrb, const unsigned short* bG, long long b_sst, int b_nlb, int nct, int nk,
                         Pre pre, Epi epi, int cb0 = 0, int cbs = 1) {
  const int tid = threadIdx.x;
  const int ncl = (nct > cb0) ? (nct - cb0 + cbs - 1) / cbs : 0;  // column tiles of this CTA
  const int ntiles = nrb * ncl;
  if (ntiles == 0) return;
  auto cb_of = [&](int t) { return cb0 + (t % ncl) * cbs; };
  if (tid >= kSubThreads) {
    // ---- producer (one thread; its warp reconverges before the final barrier)
    if (tid == kSubThreads) {
      constexpr uint32_t idesc = tc::idesc_bf16(TM, TN);
      auto load_b = [&](int t) {
        const unsigned u = gt + t;
        const int cb = cb_of(t), bb = (int)(u % NBB);
        // the buffer's previous tile (u - NBB) has finished its MMAs
        if (u >= NBB && !tc::mbar_wait(&tc.bfree[bb], ((u / NBB) - 1) & 1)) { *tc.fail = 1; return; }
        unsigned char* dst = tc.B + bb * B_BYTES;
        tc::mbar_expect_tx(&tc.ldB[bb], OZS * nk * TN * 32);
        for (int s2 = 0; s2 < OZS; ++s2)
          for (int kk = 0; kk < nk; ++kk)
            tc::bulk_g2s(dst + (s2 * 2 + kk) * TN * 32,
                         bG + s2 * b_sst + ((long long)kk * b_nlb + cb * (TN / 8)) * 128, TN * 32, &tc.ldB[bb]);
      };
      auto issue = [&](int t) {  // A if a new row block, then the MMAs of tile t
        const unsigned u = gt + t;
        const int rb = t / ncl, bb = (int)(u % NBB), acc = (int)(u & 1);
        if (t % ncl == 0) {
          // the A buffer is free once the MMAs of the previous tile (all earlier ones) completed
          if (u > 0 && !tc::mbar_wait(&tc.mmab[(u - 1) & 1], ((u - 1) >> 1) & 1)) { *tc.fail = 1; return; }
          tc::mbar_expect_tx(tc.ldA, OZS * nk * TM * 32);
          for (int s2 = 0; s2 < OZS; ++s2)
            for (int kk = 0; kk < nk; ++kk)
              tc::bulk_g2s(tc.A + (s2 * 2 + kk) * TM * 32,
                           aG + s2 * a_sst + ((long long)kk * a_nlb + rb * (TM / 8)) * 128, TM * 32, tc.ldA);
          if (!tc::mbar_wait(tc.ldA, nA & 1)) { *tc.fail = 1; return; }
          ++nA;
        }
        if (!tc::mbar_wait(&tc.ldB[bb], (u / NBB) & 1)) { *tc.fail = 1; return; }
        // the epilogue of tile u - 2 has read this accumulator
        if (u >= 2 && !tc::mbar_wait(&tc.accfree[acc], ((u >> 1) - 1) & 1)) { *tc.fail = 1; return; }
        tc::fence_after();
        const unsigned sa = tc::su32(tc.A), sb = tc::su32(tc.B + bb * B_BYTES);
        for (int kk = 0; kk < nk; ++kk)
  #pragma unroll
          for (int i = 0; i < OZS; ++i) {
            const uint64_t ad = tc::desc(sa + (i * 2 + kk) * TM * 32, 128, 256);
  #pragma unroll
            for (int jj = 0; jj < OZS - i; ++jj)
              tc::mma(tc.tmem + (unsigned)(acc * ACC_COLS + (i + jj) * TN), ad,
                      tc::desc(sb + (jj * 2 + kk) * TN * 32, 128, 256), idesc, kk > 0 || i > 0);
          }
        tc::commit(&tc.mmab[acc]);
        tc::commit(&tc.bfree[bb]);
      };
      if (!*tc.fail) load_b(0);
      if (ntiles > 1 && !*tc.fail) load_b(1);
      for (int t = 0; t < ntiles && !*tc.fail; ++t) {
        issue(t);
        if (t + 2 < ntiles && !*tc.fail) load_b(t + 2);  // its buffer held tile t - 1
      }
    }
    __syncwarp();
  } else {
    // ---- workers
    pre(0, cb_of(0), 0);
    for (int t = 0; t < ntiles; ++t) {
      const unsigned u = gt + t;
      const bool more = t + 1 < ntiles;
      if (more) pre((t + 1) / ncl, cb_of(t + 1), t + 1);
      if (!*tc.fail && !tc::mbar_wait(&tc.mmab[u & 1], (u >> 1) & 1)) *tc.fail = 1;
      tc::fence_after();
      const bool ok = __all_sync(0xffffffffu, !*tc.fail);  // warp-uniform: the epilogue's TMEM loads are .aligned
      epi(t / ncl, cb_of(t), tc.tmem + (unsigned)((u & 1) * ACC_COLS), ok, t, more);
      tc::fence_before();
      __syncwarp();
      if ((tid & 31) == 0) tc::mbar_arrive(&tc.accfree[u & 1]);
    }
  }
  __syncthreads();
  gt += ntiles;
}

constexpr int kEOff = -OZB * (OZS + 1);

// 8-byte asynchronous global -> shared copies (cp.async), one group per tile
__device__ __forceinline__ void cp_async8(void* sdst, const void* gsrc) {
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(tc::su32(sdst)), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait(bool one_pending) {
  if (one_pending)
    asm volatile("cp.async.wait_group 1;" ::: "memory");
  else
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// The flush's G staging: two tiles of 16 elements per thread, [tile & 1][u][thread]
constexpr int kStageBytes = 2 * 16 * kSubThreads * 8;

// FP64 state of one block's decisions in shared memory, each [S][KK]: the diagonal block
// G(I, I) ((r, c) at c * KB + r), the coefficients a_q, b_q ([q][x] at compact index x), u~_q,
// w~_q ([q][l] at block position l) and Gamma ((x, y) at y * KB + x)
struct SubState {
  double *Gb, *Ac, *Bc, *Ut, *Wt, *Gam;
};
// bytes of Gb .. Wt (the part the fused kernel's flush overlays with its G staging)
__host__ __device__ inline size_t sub_state_bytes(int S) {
  const size_t b = 5ull * S * KK * sizeof(double);
  return b > (size_t)kStageBytes ? b : (size_t)kStageBytes;
}

// Gb = G(I, I) of the block at sites i0 .. i0 + kb - 1, zero past kb (worker threads)
__device__ __forceinline__ void sub_load_block(const SubState& st, const double* const* G, int S, int N, int i0, int kb) {
  for (int e = threadIdx.x; e < S * KK; e += kSubThreads) {
    const int sp = e / KK, c = (e % KK) / KB, r = e % KB;
    st.Gb[e] = (r < kb && c < kb) ? G[sp][(long long)(i0 + c) * N + i0 + r] : 0.0;
  }
}

// The decisions of one block, flip by flip, and Gamma = sum_q a_q b_q^T; returns m, the
// accepts, with their block positions in s_pos.  uni and fld are the block's uniforms and
// fields (position l).  The sites are visited in order: warp 0 evaluates the ratios of all
// sites still to visit at once, on the diagonal as it stands, and the lowest accepted one is
// the next accept of the sequential visit, since every site before it saw the same diagonal.
// Each accept then takes two phases: (1) the coefficients u~, w~, a, b of the accept; (2)
// its rank-1 update of the block, warp 0 updating the diagonal of the sites still to visit
// before it scans them for the next accept, while warps 1-7 update the rest of the block and
// add a b^T to Gamma (the fma sequence of the closed sum over accepts, so Gamma is the same
// to the bit).  sign and acc_count are thread 0's.  Worker threads only.
__device__ __forceinline__ int sub_decide(const WalkerDev& w, int S, int kb, const double* uni, int8_t* fld,
                                          const SubState& st, int* s_pos, int* s_next, double* s_f, double& sign,
                                          long long& acc_count) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int e = tid; e < S * KK; e += kSubThreads) st.Gam[e] = 0.0;
  int m = 0, cur = 0;
  while (true) {
    if (warp == 0) {
      const int l = cur + lane;
      FlipRatio q{};
      double fq[2] = {0.0, 0.0};
      int s = 0;
      bool acc = false;
      if (l < kb) {
        if (m > 0)  // the previous accept's update of this site's diagonal element
          for (int sp = 0; sp < S; ++sp) {
            double* gb = st.Gb + sp * KK;
            gb[l * KB + l] = fma(-st.Ut[sp * KK + (m - 1) * KB + l], st.Wt[sp * KK + (m - 1) * KB + l], gb[l * KB + l]);
          }
        s = fld[l];
        const int si = s > 0 ? 0 : 1;
        const double gu = st.Gb[l * KB + l];
        const double gd = (S == 2) ? st.Gb[KK + l * KB + l] : gu;
        q = flip_ratio(w, si, gu, gd);  // reference operation order
        acc = uni[l] < fmin(1.0, fabs(q.r));
        flip_factors(w, q, fq);         // every lane: off the accepted lane's critical path
      }
      const unsigned amask = __ballot_sync(0xffffffffu, acc);
      const int first = amask ? __ffs(amask) - 1 : 32;
      if (l < kb && lane <= first && !isfinite(q.r)) atomicOr(w.status, ST_NONFINITE_RATIO);
      if (lane == first) {
        s_f[0] = fq[0];
        s_f[1] = fq[1];
        fld[l] = (int8_t)(-s);
      }
      const double rf = __shfl_sync(0xffffffffu, q.r, first & 31);
      if (lane == 0) {
        if (amask) {
          sign = (rf >= 0) ? sign : -sign;
          ++acc_count;
        }
        *s_next = amask ? cur + first : kb;
      }
    } else if (m > 0) {
      // the previous accept (position cur - 1): rank-1 update off the diagonal, Gamma term
      const int lp = cur - 1, q1 = m - 1;
      for (int e = tid - 32; e < S * KK; e += kSubThreads - 32) {
        const int sp = e / KK, c = (e % KK) / KB, r = e % KB;
        if (r > lp && c > lp && r < kb && c < kb && r != c)
          st.Gb[e] = fma(-st.Ut[sp * KK + q1 * KB + r], st.Wt[sp * KK + q1 * KB + c], st.Gb[e]);
        const int y = c, x = r;
        if (x <= q1 && y <= q1)
          st.Gam[e] = fma(st.Ac[sp * KK + q1 * KB + x], st.Bc[sp * KK + q1 * KB + y], st.Gam[e]);
      }
    }
    wsync();
    const int l = *s_next;
    if (l >= kb) break;
    // u~, w~ of accept m on the block, and its coefficients a_m, b_m
    for (int e = tid; e < S * 4 * KB; e += kSubThreads) {
      const int sp = e / (4 * KB), role = (e / KB) & 3, x = e % KB;
      const double f = s_f[sp];
      const double* gb = st.Gb + sp * KK;
      double* ut = st.Ut + sp * KK;
      double* wt = st.Wt + sp * KK;
      double* ac = st.Ac + sp * KK;
      double* bc = st.Bc + sp * KK;
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
    wsync();
    ++m;
    cur = l + 1;
  }
  return m;
}

// Spin sp of a block with m accepts at sites i0 + s_pos[q]: the slices of Gamma, G0(:, I_A) and
// R_A = E_A^T - G0(I_A, :) (taken before G changes), then T^T = R_A^T Gamma^T on the tensor
// cores: warp w and w + 4 share TMEM lanes 32 (w & 3).. (columns c) and take x in [0, 16) and
// [16, 32); the column exponent max over x goes through etmp, and the epilogue slices T straight
// into the B image of the flush (line c, k = x).  Line exponents: eGm [KB] of Gamma, eG [N] of
// G0(:, I_A), eR [N] of R_A, eT [N] of T (shared or global memory); etmp: [2][256] scratch.
// Called by all kSubCTA threads; the workers slice.
__device__ __forceinline__ void sub_prepare(const SubTC& tcs, unsigned& gt, unsigned& nA, const WalkerDev& w, int sp, int N, int m,
                            int i0, const int* s_pos, const double* gam, const double* Gs, int* eGm, int* eG, int* eR,
                            int* eT, int* etmp) {
  const SubOff so = sub_offsets(N);
  unsigned char* ms = w.msub + (size_t)sp * so.total;
  unsigned short* sGm = reinterpret_cast<unsigned short*>(ms + so.sGm);
  unsigned short* sG = reinterpret_cast<unsigned short*>(ms + so.sG);
  unsigned short* sR = reinterpret_cast<unsigned short*>(ms + so.sR);
  unsigned short* sT = reinterpret_cast<unsigned short*>(ms + so.sT);
  const int tid = threadIdx.x;
  const int nlbN = ozaki::tc_lines(N) / 8, nk = (m + 15) / 16;
  const long long sstN = (long long)sub_sst(N), sstG = (long long)sub_sst(1);
  if (tid < kSubThreads) {
    unsigned short* dGm[1] = {sGm};
    int* xGm[1] = {eGm};
    slice_lines<1>([&](int, int line, int k) { return gam[k * KB + line]; }, m, m, dGm, sstG, TM / 8, xGm, etmp);
    // G0(:, I_A) (lines = rows) and R_A (lines = columns) in one pass
    unsigned short* dGR[2] = {sG, sR};
    int* xGR[2] = {eG, eR};
    slice_lines<2>(
        [&](int o, int line, int k) {
          const int i = i0 + s_pos[k];
          return o == 0 ? Gs[(long long)i * N + line] : ((line == i) ? 1.0 : 0.0) - Gs[(long long)line * N + i];
        },
        N, m, dGR, sstN, nlbN, xGR, etmp);
    asm volatile("fence.proxy.async.global;" ::: "memory");  // generic writes -> bulk-copy reads
  }
  __syncthreads();
  sub_gemm(tcs, gt, nA, sR, sstN, nlbN, (N + TM - 1) / TM, sGm, sstG, TM / 8, 1, nk, [&](int, int, int) {},
           [&](int rb, int, unsigned tacc, bool ok, int tl, bool) {
             const int wq = (tid >> 5) & 3, xh = tid >> 7;
             const int c = rb * TM + wq * 32 + (tid & 31);
             const int ec = (c < N) ? eR[c] : 0;
             double tv[16];
             int e = -1100;
             if (ok) {
               uint32_t v[2][OZS][8];  // both halves' loads in flight before one wait
#pragma unroll
               for (int h = 0; h < 2; ++h)
#pragma unroll
                 for (int g = 0; g < OZS; ++g)
                   tc::ld8(v[h][g], tacc + ((unsigned)(wq * 32) << 16) + (unsigned)(g * TN + xh * 16 + h * 8));
               tc::wait_ld();
#pragma unroll
               for (int h = 0; h < 2; ++h)
#pragma unroll
                 for (int u = 0; u < 8; ++u) {
                   const int x = xh * 16 + h * 8 + u;
                   tv[h * 8 + u] =
                       (x < m && c < N) ? ozaki::ldexp_i64(group_sum(v[h], u), ec + eGm[x] + kEOff) : 0.0;
                   e = max(e, ozaki::exp_bound(tv[h * 8 + u]));
                 }
             }
             int* ex = etmp + (tl & 1) * kSubThreads;  // two tiles in flight between the halves
             ex[tid] = e;
             wsync();
             e = max(e, ex[tid ^ 128]);
             if (ok && c < N) {
               if (xh == 0) eT[c] = e;
               unsigned pk[OZS][8];
#pragma unroll
               for (int u = 0; u < 16; u += 2) {
                 bool n0, n1;
                 const unsigned long long q0 = ozaki::fixed42(tv[u], e, n0), q1 = ozaki::fixed42(tv[u + 1], e, n1);
#pragma unroll
                 for (int s2 = 0; s2 < OZS; ++s2)
                   pk[s2][u >> 1] = (unsigned)ozaki::slice_bf16(q0, s2, OZB, n0) |
                                    ((unsigned)ozaki::slice_bf16(q1, s2, OZB, n1) << 16);
               }
               unsigned short* o = sT + ozaki::tc_index(c, xh * 16, nlbN);
#pragma unroll
               for (int s2 = 0; s2 < OZS; ++s2) {
                 *reinterpret_cast<uint4*>(o + s2 * sstN) = make_uint4(pk[s2][0], pk[s2][1], pk[s2][2], pk[s2][3]);
                 *reinterpret_cast<uint4*>(o + s2 * sstN + 64) =
                     make_uint4(pk[s2][4], pk[s2][5], pk[s2][6], pk[s2][7]);
               }
             }
             asm volatile("fence.proxy.async.global;" ::: "memory");  // T's slices -> the flush's bulk copies
           });
}

// G -= G0(:, I_A) T for spin sp over the column tiles cb0, cb0 + cbs, ... of G (all kSubCTA
// threads; the workers run the epilogue): worker warp w reads
// TMEM lanes 32 (w & 3) .. (rows), columns 16 (w >> 2) ..  Each thread's 16 elements of G of
// the next tile are copied into stage (kStageBytes of shared memory) while the epilogue of the
// current tile runs, so the epilogue reads G from shared memory; eG, eT: line exponents.
__device__ __forceinline__ void sub_flush(const SubTC& tcs, unsigned& gt, unsigned& nA, const WalkerDev& w, int sp, int N, int m,
                          double* Gs, const int* eG, const int* eT, double* stage, int cb0, int cbs) {
  const SubOff so = sub_offsets(N);
  const unsigned char* ms = w.msub + (size_t)sp * so.total;
  const unsigned short* sG = reinterpret_cast<const unsigned short*>(ms + so.sG);
  const unsigned short* sT = reinterpret_cast<const unsigned short*>(ms + so.sT);
  const int tid = threadIdx.x, wq = (tid >> 5) & 3, half = tid >> 7;
  const int nlbN = ozaki::tc_lines(N) / 8, nk = (m + 15) / 16, nct = (N + TN - 1) / TN;
  const long long sstN = (long long)sub_sst(N);
  sub_gemm(tcs, gt, nA, sG, sstN, nlbN, (N + TM - 1) / TM, sT, sstN, nlbN, nct, nk,
           [&](int rb, int cb, int tl) {
             const int r = rb * TM + wq * 32 + (tid & 31), c0 = cb * TN + half * 16;
             double* dst = stage + (tl & 1) * 16 * kSubThreads + tid;
             if (r < N) {
#pragma unroll
               for (int u = 0; u < 16; ++u)
                 if (c0 + u < N) cp_async8(dst + u * kSubThreads, Gs + (long long)(c0 + u) * N + r);
             }
             cp_async_commit();
           },
           [&](int rb, int cb, unsigned tacc, bool ok, int tl, bool more) {
             cp_async_wait(more);  // this tile's copies (the next tile's may be in flight)
             if (!ok) return;
             const int r = rb * TM + wq * 32 + (tid & 31), c0 = cb * TN + half * 16;
             const double* gsv = stage + (tl & 1) * 16 * kSubThreads + tid;
             const int er = (r < N) ? eG[r] : 0;
             const unsigned ta = tacc + ((unsigned)(wq * 32) << 16);
             uint32_t v[2][OZS][8];  // both halves' loads in flight before one wait
#pragma unroll
             for (int h = 0; h < 2; ++h)
#pragma unroll
               for (int g = 0; g < OZS; ++g) tc::ld8(v[h][g], ta + (unsigned)(g * TN + half * 16 + h * 8));
             tc::wait_ld();
#pragma unroll
             for (int h = 0; h < 2; ++h)
#pragma unroll
               for (int u = 0; u < 8; ++u) {
                 const int c = c0 + h * 8 + u;
                 const long long sv = group_sum(v[h], u);
                 if (sv != 0 && r < N && c < N)
                   Gs[(long long)c * N + r] =
                       gsv[(h * 8 + u) * kSubThreads] - ozaki::ldexp_i64(sv, er + eT[c] + kEOff);
               }
           },
           cb0, cbs);
}

}  // namespace

size_t submatrix_scratch_bytes(int N) { return sub_offsets(N).total; }

// dynamic shared memory of the fused kernel: tensor-core operand buffers first (1024-byte
// aligned base), then the slice's uniforms [N], Gamma [S][KK], the block state (overlaid by the
// flush's G staging), the line exponents eG, eT, eR [N] and eGm [KB], the exponent scratch
// [2][256] and the fields [N]
size_t submatrix_smem_bytes(int N, int S) {
  const size_t Nu = (size_t)((N + 1) & ~1);
  return (size_t)A_BYTES + (size_t)NBB * B_BYTES + sizeof(double) * (Nu + (size_t)S * KK) + sub_state_bytes(S) +
         sizeof(int) * (3 * Nu + KB + 2 * kSubThreads) + (size_t)N;
}

// One slice for one walker per CTA: kSubCTA threads, the eight worker warps and the producer.
__global__ void __launch_bounds__(kSubCTA, 1) metropolis_sub_kernel(const WalkerDev* __restrict__ W, int mode, int j,
                                                                    int q) {
  const WalkerDev& w = W[blockIdx.x];
  if (w.path != 2) return;
  int t;
  if (!sub_slice_of(w, mode, j, q, t)) return;
  const int N = w.N, S = w.S, Lt = w.Lt, tid = threadIdx.x;
  const bool worker = tid < kSubThreads;
  const int Nu = (N + 1) & ~1;
  const long long NN = (long long)N * N;
  extern __shared__ __align__(1024) unsigned char smem[];
  double* uni = reinterpret_cast<double*>(smem + A_BYTES + NBB * B_BYTES);  // [N] uniforms of the slice
  SubState st;
  st.Gam = uni + Nu;
  st.Gb = st.Gam + S * KK;
  st.Ac = st.Gb + S * KK;
  st.Bc = st.Ac + S * KK;
  st.Ut = st.Bc + S * KK;
  st.Wt = st.Ut + S * KK;
  double* stage = st.Gb;  // the flush's G tiles over the dead block state
  int* s_eG = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(st.Gb) + sub_state_bytes(S));
  int* s_eT = s_eG + Nu;
  int* s_eR = s_eT + Nu;
  int* s_eGm = s_eR + Nu;
  int* etmp = s_eGm + KB;                                               // [2][256]
  int8_t* s_field = reinterpret_cast<int8_t*>(etmp + 2 * kSubThreads);  // [N]
  __shared__ int s_next, s_pos[KB], s_m;
  __shared__ double s_f[2];
  __shared__ __align__(8) unsigned long long bar_ldA, bar_ldB[NBB], bar_mma[2], bar_bfree[NBB], bar_accfree[2];
  __shared__ unsigned s_tmem;
  __shared__ int s_tcfail;

  double* G[2] = {w.G, (S == 2) ? w.G + NN : w.G};
  const int eff = t - 1;
  const unsigned long long sweep = (w.rng == 1) ? *w.sweep_ctr : 0ULL;
  if (worker)
    for (int i = tid; i < N; i += kSubThreads) {
      s_field[i] = w.fields[(long long)eff * N + i];
      const int attempt = (mode == MODE_FWD) ? (eff * N + i) : ((Lt - t) * N + i);
      uni[i] = (w.rng == 0) ? w.uni[attempt] : philox_uniform(w.seed, (unsigned)w.widx, sweep, (unsigned)(eff * N + i));
    }
  double sign = 0.0;
  long long acc_count = 0;
  if (tid == 0) {
    sign = *w.sign;
    s_tcfail = 0;
    sub_tc_init(&bar_ldA, bar_ldB, bar_mma, bar_bfree, bar_accfree);
  }
  if (tid < 32) tc::alloc(&s_tmem, TMEM_COLS);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const SubTC tcs{smem, smem + A_BYTES, &bar_ldA, bar_ldB, bar_mma, bar_bfree, bar_accfree, s_tmem, &s_tcfail};
  unsigned gt = 0, nA = 0;  // tiles and A loads so far (mbarrier phases)

  for (int i0 = 0; i0 < N; i0 += KB) {
    const int kb = min(KB, N - i0);
    if (worker) {
      sub_load_block(st, G, S, N, i0, kb);
      wsync();
      const int mm = sub_decide(w, S, kb, uni + i0, s_field + i0, st, s_pos, &s_next, s_f, sign, acc_count);
      if (tid == 0) s_m = mm;
    }
    __syncthreads();
    const int m = s_m;
    if (m == 0) continue;
    for (int sp = 0; sp < S; ++sp) {
      sub_prepare(tcs, gt, nA, w, sp, N, m, i0, s_pos, st.Gam + sp * KK, G[sp], s_eGm, s_eG, s_eR, s_eT, etmp);
      sub_flush(tcs, gt, nA, w, sp, N, m, G[sp], s_eG, s_eT, stage, 0, 1);
    }
  }

  int8_t* frw = w.fields + (long long)eff * N;
  if (worker)
    for (int i = tid; i < N; i += kSubThreads) frw[i] = s_field[i];
  // TMEM back: every committed MMA has completed (each tile's commit was waited on)
  tc::fence_before();
  __syncthreads();
  if (tid < 32) tc::dealloc(s_tmem, TMEM_COLS);
  if (tid == 0) {
    if (s_tcfail) atomicOr(w.status, ST_TIMEOUT);
    *w.sign = sign;
    *w.accepts += acc_count;
    if (mode == MODE_BWD && t == Lt) *w.sign_Lt = sign;
  }
}

// ---- the same updates split per 32-site block into two kernels ----------------
// For walkers too few to fill the GPU (one CTA per walker leaves most SMs idle at
// 32 walkers of N = 576), each block runs as a decision kernel (one CTA per walker:
// the decisions, Gamma, the slices of Gamma, G0(:, I_A) and R_A, T^T on the tensor
// cores) followed by a flush kernel whose CTAs share the walker's column tiles of G.
// The arithmetic is the fused kernel's (the same device functions).  The autotuner
// times both.

// dynamic shared memory of the decision kernel: the operand buffers, the block's uniforms,
// the FP64 block state, the exponent scratch [2][256] and the block's fields; of the flush
// kernel: the operand buffers, the G staging and the line exponents eG, eT [N]
size_t submatrix_block_smem_bytes(int S) {
  return (size_t)A_BYTES + (size_t)NBB * B_BYTES + sizeof(double) * (KB + 6ull * S * KK) +
         2 * kSubThreads * sizeof(int) + KB;
}
size_t submatrix_flush_smem_bytes(int N) {
  return (size_t)A_BYTES + (size_t)NBB * B_BYTES + kStageBytes + 2 * sizeof(int) * (size_t)((N + 1) & ~1);
}

__global__ void __launch_bounds__(kSubCTA) metropolis_sub_block_kernel(const WalkerDev* __restrict__ W, int mode,
                                                                       int j, int q, int blk) {
  const WalkerDev& w = W[blockIdx.x];
  if (w.path != 2) return;
  int t;
  if (!sub_slice_of(w, mode, j, q, t)) return;
  const int N = w.N, S = w.S, Lt = w.Lt, tid = threadIdx.x;
  const bool worker = tid < kSubThreads;
  const int i0 = blk * KB;
  if (i0 >= N) return;
  const int kb = min(KB, N - i0);
  const long long NN = (long long)N * N;
  extern __shared__ __align__(1024) unsigned char smem[];
  double* uni = reinterpret_cast<double*>(smem + A_BYTES + NBB * B_BYTES);  // [KB] uniforms of the block
  SubState st;
  st.Gam = uni + KB;
  st.Gb = st.Gam + S * KK;
  st.Ac = st.Gb + S * KK;
  st.Bc = st.Ac + S * KK;
  st.Ut = st.Bc + S * KK;
  st.Wt = st.Ut + S * KK;
  int* etmp = reinterpret_cast<int*>(st.Wt + S * KK);                   // [2][256]
  int8_t* s_field = reinterpret_cast<int8_t*>(etmp + 2 * kSubThreads);  // [KB]
  __shared__ int s_next, s_pos[KB], s_m;
  __shared__ double s_f[2];
  __shared__ __align__(8) unsigned long long bar_ldA, bar_ldB[NBB], bar_mma[2], bar_bfree[NBB], bar_accfree[2];
  __shared__ unsigned s_tmem;
  __shared__ int s_tcfail;

  const SubOff so = sub_offsets(N);
  const double* G[2] = {w.G, (S == 2) ? w.G + NN : w.G};
  const int eff = t - 1;
  const unsigned long long sweep = (w.rng == 1) ? *w.sweep_ctr : 0ULL;
  if (worker) {
    for (int l = tid; l < kb; l += kSubThreads) {
      const int i = i0 + l;
      s_field[l] = w.fields[(long long)eff * N + i];
      const int attempt = (mode == MODE_FWD) ? (eff * N + i) : ((Lt - t) * N + i);
      uni[l] = (w.rng == 0) ? w.uni[attempt] : philox_uniform(w.seed, (unsigned)w.widx, sweep, (unsigned)(eff * N + i));
    }
    sub_load_block(st, G, S, N, i0, kb);
    double sign = (tid == 0) ? *w.sign : 0.0;
    long long acc_count = 0;
    wsync();
    const int m = sub_decide(w, S, kb, uni, s_field, st, s_pos, &s_next, s_f, sign, acc_count);
    int8_t* frw = w.fields + (long long)eff * N + i0;
    for (int l = tid; l < kb; l += kSubThreads) frw[l] = s_field[l];
    if (tid == 0) {
      *w.sign = sign;
      *w.accepts += acc_count;
      if (mode == MODE_BWD && t == Lt && i0 + KB >= N) *w.sign_Lt = sign;
      *reinterpret_cast<int*>(w.msub + so.mc) = m;
      s_m = m;
      s_tcfail = 0;
      if (m > 0) sub_tc_init(&bar_ldA, bar_ldB, bar_mma, bar_bfree, bar_accfree);
    }
  }
  __syncthreads();
  const int m = s_m;
  if (m == 0) return;

  if (tid < 32) tc::alloc(&s_tmem, TMEM_COLS);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const SubTC tcs{smem, smem + A_BYTES, &bar_ldA, bar_ldB, bar_mma, bar_bfree, bar_accfree, s_tmem, &s_tcfail};
  unsigned gt = 0, nA = 0;
  for (int sp = 0; sp < S; ++sp) {
    unsigned char* ms = w.msub + (size_t)sp * so.total;
    sub_prepare(tcs, gt, nA, w, sp, N, m, i0, s_pos, st.Gam + sp * KK, G[sp], reinterpret_cast<int*>(ms + so.eGm),
                reinterpret_cast<int*>(ms + so.eG), reinterpret_cast<int*>(ms + so.eR),
                reinterpret_cast<int*>(ms + so.eT), etmp);
  }
  tc::fence_before();
  __syncthreads();
  if (tid < 32) tc::dealloc(s_tmem, TMEM_COLS);
  if (tid == 0 && s_tcfail) {
    atomicOr(w.status, ST_TIMEOUT);
    *reinterpret_cast<int*>(w.msub + so.mc) = 0;  // no flush from a product that gave up
  }
}

// The flush of block blk: G -= G0(:, I_A) T for both spins, the column tiles of G spread over
// the gridDim.x CTAs of a walker (CTA p takes tiles p, p + gridDim.x, ...).
__global__ void __launch_bounds__(kSubCTA) metropolis_sub_flush_kernel(const WalkerDev* __restrict__ W, int mode,
                                                                       int j, int q, int blk) {
  const WalkerDev& w = W[blockIdx.y];
  if (w.path != 2) return;
  int t;
  if (!sub_slice_of(w, mode, j, q, t)) return;
  const int N = w.N, S = w.S, tid = threadIdx.x;
  if (blk * KB >= N) return;
  const int nct = (N + TN - 1) / TN;
  if ((int)blockIdx.x >= nct) return;
  const SubOff so = sub_offsets(N);
  const int m = *reinterpret_cast<const int*>(w.msub + so.mc);
  if (m == 0) return;
  const int Nu = (N + 1) & ~1;
  const long long NN = (long long)N * N;
  extern __shared__ __align__(1024) unsigned char smem[];
  double* stage = reinterpret_cast<double*>(smem + A_BYTES + NBB * B_BYTES);
  int* s_eG = reinterpret_cast<int*>(reinterpret_cast<unsigned char*>(stage) + kStageBytes);
  int* s_eT = s_eG + Nu;
  __shared__ __align__(8) unsigned long long bar_ldA, bar_ldB[NBB], bar_mma[2], bar_bfree[NBB], bar_accfree[2];
  __shared__ unsigned s_tmem;
  __shared__ int s_tcfail;
  if (tid == 0) {
    s_tcfail = 0;
    sub_tc_init(&bar_ldA, bar_ldB, bar_mma, bar_bfree, bar_accfree);
  }
  if (tid < 32) tc::alloc(&s_tmem, TMEM_COLS);
  tc::fence_before();
  __syncthreads();
  tc::fence_after();
  const SubTC tcs{smem, smem + A_BYTES, &bar_ldA, bar_ldB, bar_mma, bar_bfree, bar_accfree, s_tmem, &s_tcfail};
  unsigned gt = 0, nA = 0;
  for (int sp = 0; sp < S; ++sp) {
    const unsigned char* ms = w.msub + (size_t)sp * so.total;
    const int* eG = reinterpret_cast<const int*>(ms + so.eG);
    const int* eT = reinterpret_cast<const int*>(ms + so.eT);
    if (tid < kSubThreads)
      for (int i = tid; i < N; i += kSubThreads) {
        s_eG[i] = eG[i];
        s_eT[i] = eT[i];
      }
    __syncthreads();
    sub_flush(tcs, gt, nA, w, sp, N, m, w.G + sp * NN, s_eG, s_eT, stage, (int)blockIdx.x, (int)gridDim.x);
  }
  tc::fence_before();
  __syncthreads();
  if (tid < 32) tc::dealloc(s_tmem, TMEM_COLS);
  if (tid == 0 && s_tcfail) atomicOr(w.status, ST_TIMEOUT);
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
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(metropolis_sub_block_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)submatrix_block_smem_bytes(2));
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(metropolis_sub_flush_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)submatrix_flush_smem_bytes(kMaxN));
  return e;
}

void launch_metropolis_sub(const WalkerDev* W, int nw, int mode, int j, int q, int maxN, int S_max, cudaStream_t st) {
  metropolis_sub_kernel<<<nw, kSubCTA, submatrix_smem_bytes(maxN, S_max), st>>>(W, mode, j, q);
}

// CTAs per walker of the split flush: two column tiles of 32 each (at least one CTA)
int submatrix_flush_ctas(int maxN) { return std::max(1, ((maxN + TN - 1) / TN + 1) / 2); }

// One slice of Metropolis by the split kernels: for each 32-site block the decisions (one CTA
// per walker) then the flush (submatrix_flush_ctas CTAs per walker); walkers whose N ends
// earlier skip the blocks past it.
void launch_metropolis_sub_split(const WalkerDev* W, int nw, int mode, int j, int q, int maxN, int S_max,
                                 cudaStream_t st) {
  const int nb = (maxN + KB - 1) / KB, P = submatrix_flush_ctas(maxN);
  const size_t sm1 = submatrix_block_smem_bytes(S_max), sm2 = submatrix_flush_smem_bytes(maxN);
  for (int blk = 0; blk < nb; ++blk) {
    metropolis_sub_block_kernel<<<nw, kSubCTA, sm1, st>>>(W, mode, j, q, blk);
    metropolis_sub_flush_kernel<<<dim3(P, nw), kSubCTA, sm2, st>>>(W, mode, j, q, blk);
  }
}

}  // namespace dqmc
