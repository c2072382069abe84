// ozaki.cuh — FP64-accurate matrix products on the BF16 tensor cores.
//
// An FP64 operand is cut into S slices of B-bit signed integers that share one
// power-of-two exponent per row (left operand) or per column (right operand):
//     x(r,k) = 2^{e_r} * sum_i a_i(r,k) 2^{-B(i+1)} + (remainder < 2^{e_r - B S}),
// computed from the IEEE bit pattern with integer operations only (no FP64 pipe).
// Integers |a_i| < 2^B are exact in BF16, and a slice-pair product summed over
// K terms stays below 2^24 when (2^B - 1)^2 K < 2^22, so the tensor core's FP32
// accumulation of a group m = i + j (at most 4 pairs for m <= 3) is exact; the
// groups m >= 4 carry weights 2^{-4B} and below, where FP32 rounding is far
// under the kept precision.  The product is
//     C(r,c) = 2^{e_r + f_c} sum_m 2^{-B(m+2)} S_m(r,c),   S_m = sum_{i+j=m} A_i B_j.
// The sweep's wraps and B-chain use B = 7, S = 7 (49 bits, 28 slice products)
// for K <= 256 and B = 6, S = 8 (48 bits, 36 products) for K <= 1024: at
// beta = 10 the chain of a stabilization interval amplifies the truncation of
// 42-bit products into |dG| of a few 1e-6, 49 bits keep it near 1e-8.  The
// rank-k Metropolis flushes (K <= 32) use B = 7, S = 6.  This is the splitting
// scheme of Ozaki, Ogita, Oishi and Rump (Numer. Algorithms 2012) restated for
// BF16 inputs.
#pragma once
#include <cstdint>

namespace dqmc {
namespace ozaki {

constexpr int kMaxSlices = 8;

struct SliceCfg {
  int bits, slices;
};
__host__ __device__ constexpr SliceCfg cfg_for_k(int K) { return K <= 256 ? SliceCfg{7, 7} : SliceCfg{6, 8}; }

// The tensor-core image of a slice (the sweep's operands): k in chunks of 16,
// 8-line blocks of 256 bytes in core-matrix order ((k / 8) * 128 + (line % 8) * 16
// + (k % 8) * 2 bytes), the blocks of one chunk side by side, lines padded to a
// multiple of 128.  A tile's chunk (128 or 64 consecutive lines) is then one
// contiguous range, the layout the tensor core reads from shared memory.
__host__ __device__ inline int tc_lines(int N) { return (N + 127) / 128 * 128; }
__host__ __device__ inline size_t tc_slice_elems(int N, int ldk) { return (size_t)ldk * tc_lines(N); }
__host__ __device__ inline long long tc_index(int line, int k, int nlb) {
  return ((long long)(k >> 4) * nlb + (line >> 3)) * 128 + ((k >> 3) & 1) * 64 + (line & 7) * 8 + (k & 7);
}

// exponent e with |x| < 2^e (0 for x == 0); integer only
__device__ __forceinline__ int exp_bound(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int ex = (int)((b >> 52) & 0x7ff);
  return ex == 0 ? -1100 : ex - 1022;  // normal: |x| in [2^(ex-1023), 2^(ex-1022))
}

// Q-bit truncated fixed-point magnitude of |x| / 2^e (e >= exp_bound(x), Q <= 62), and sign
__device__ __forceinline__ unsigned long long fixedq(double x, int e, int Q, bool& neg) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex == 0) return 0ULL;
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFULL) | 0x10000000000000ULL;
  const int s = ex - 1075 - e + Q;  // |x| 2^{Q-e} = m 2^s, s <= Q - 53
  if (s >= 0) return m << s;
  if (s <= -64) return 0ULL;
  return m >> (-s);
}
// slice i of a Q-bit magnitude with B bits per slice, as a signed BF16 bit pattern
__device__ __forceinline__ unsigned short slice_bf16q(unsigned long long q, int i, int bits, int Q, bool neg) {
  const unsigned v = (unsigned)((q >> (Q - bits * (i + 1))) & ((1u << bits) - 1));
  const float f = neg ? -(float)v : (float)v;  // exact: v < 2^8
  return (unsigned short)(__float_as_uint(f) >> 16);
}

// 42-bit truncated fixed-point magnitude of |x| / 2^e (e >= exp_bound(x)), and sign
__device__ __forceinline__ unsigned long long fixed42(double x, int e, bool& neg) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  neg = (b >> 63) != 0;
  const int ex = (int)((b >> 52) & 0x7ff);
  if (ex == 0) return 0ULL;  // zero (subnormals flushed: far below any kept bit here)
  const unsigned long long m = (b & 0xFFFFFFFFFFFFFULL) | 0x10000000000000ULL;  // 53 bits
  // |x| / 2^e = m * 2^{ex - 1075 - e};  want floor(that * 2^42) = m >> (1033 + e - ex)
  const int sh = 1033 + e - ex;
  if (sh >= 64) return 0ULL;
  if (sh <= 0) return m << (-sh);  // cannot happen for e >= exp_bound(x)
  return m >> sh;
}

// slice i of a 42-bit magnitude with B bits per slice, as a signed BF16 bit pattern
__device__ __forceinline__ unsigned short slice_bf16(unsigned long long q, int i, int bits, bool neg) {
  const int sh = 42 - bits * (i + 1);
  const unsigned v = (unsigned)((sh >= 0 ? (q >> sh) : (q << (-sh))) & ((1u << bits) - 1));
  const float f = neg ? -(float)v : (float)v;  // exact: v < 2^8
  return (unsigned short)(__float_as_uint(f) >> 16);  // exact truncation: low 16 bits are zero
}

// x * 2^e by exponent arithmetic (two steps keep each factor a normal double)
__device__ __forceinline__ double scale2(double x, int e) {
  if (e > 1000) { x *= 0x1p1000; e -= 1000; }
  if (e < -1000) { x *= 0x1p-1000; e += 1000; }
  e = max(-1022, min(1023, e));
  return x * __longlong_as_double((long long)(e + 1023) << 52);
}

// ---- epilogue: recombining the S weight groups with integer operations -----
// GB300 issues FP64 at 1/64 of its FP32 rate, so the epilogue avoids FP64
// arithmetic: each group sum is an integer-valued FP32 number, the groups are
// added as one 64-bit integer v = sum_m S_m 2^{B(S-1-m)} (|v| < 2^61 for the
// configurations above), and v 2^e is assembled as IEEE-754 bits (truncated
// to 53 bits, below the kept precision).

// exact value of an integer-valued float with |x| < 2^22 (FP32 add + integer subtract)
__device__ __forceinline__ int f2i_small(float x) { return __float_as_int(x + 12582912.0f) - 0x4B400000; }

// v * 2^e as a double, built from the bits (0 below the normal range)
__device__ __forceinline__ double ldexp_i64(long long v, int e) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = (unsigned long long)v & 0x8000000000000000ULL;
  unsigned long long a = sgn ? (0ULL - (unsigned long long)v) : (unsigned long long)v;
  const int p = 63 - __clzll((long long)a);  // index of the leading one
  a = (p >= 52) ? (a >> (p - 52)) : (a << (52 - p));
  const int ex = p + e + 1023;
  if (ex <= 0) return 0.0;
  if (ex >= 2047) return __longlong_as_double((long long)(sgn | 0x7FF0000000000000ULL));
  return __longlong_as_double((long long)(sgn | ((unsigned long long)ex << 52) | (a & 0xFFFFFFFFFFFFFULL)));
}

// The S weight-group sums of an element, read as hi = groups 0..3 (|hi| < 2^44 for
// the configurations used: B = 7 with K <= 256, B = 6 with K <= 1024) and lo =
// groups 4..S-1, as one FP64 value 2^e sum_m S_m 2^(-B (m + 2)): hi and the
// rounded top of lo form one 63-bit integer hi 2^(B (S - 4) - D) + round(lo / 2^D)
// with D = B (S - 4) - 19, so a single conversion replaces two and an FP64 add.
// The 2^D units of lo dropped lie below the slices' own truncation (at most
// 2^(e - 2B - 37) against K 2^(e - B S) for the products that use it).
template <int S, int B>
__device__ __forceinline__ double combine_hilo(long long hi, long long lo, int e) {
  constexpr int D = B * (S - 4) - 19;
  static_assert(D >= 1 && D < 32, "hi/lo split");
  const long long v = (hi << (B * (S - 4) - D)) + ((lo + (1LL << (D - 1))) >> D);
  return ldexp_i64(v, e - B * (S + 1) + D);
}

// one BF16 tensor-core MMA m16n8k16, FP32 accumulate in place
__device__ __forceinline__ void mma16816(float (&c)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                         unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

}  // namespace ozaki
}  // namespace dqmc
