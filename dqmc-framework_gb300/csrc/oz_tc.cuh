// oz_tc.cuh — the main loop shared by the slice-pair products on the
// 5th-generation tensor cores (wraps, B-chain and stabilization products).
//
// Operands are pre-sliced into S integer slices stored as the tensor core's
// shared-memory image (ozaki::tc_index): k in chunks of 16, 8-line blocks of
// 256 bytes, so that the 16-deep chunk of one slice over a tile's MT (or NT)
// consecutive lines is one contiguous range of MT * 32 bytes.  One thread
// streams the chunks with bulk asynchronous copies into a ring of NS stages
// (each completing on its own mbarrier's byte count), issues the S (S+1) / 2
// MMAs of a chunk (slice pair (i, j) accumulates into weight group i + j, S
// groups of NT FP32 columns in TMEM) and refills a stage once the MMAs that read
// it have completed (their commit mbarrier): NS - 1 chunks are in flight while
// the tensor core works.  Every wait is bounded; on a timeout the loop stops,
// waits (bounded) for the copies it issued and reports the failure.
#pragma once
#include <cstdint>

#include "tcgen05.cuh"

namespace dqmc {
namespace oztc {

// bytes of one stage: S slices of an MT x 16 A chunk and an NT x 16 B chunk
__host__ __device__ constexpr int stage_bytes(int S, int MT, int NT) { return S * (MT + NT) * 16 * 2; }

// Thread-only main loop.  a0 / b0: slice 0 of the tile's first line block at
// chunk 0; consecutive slices sstride elements apart, consecutive chunks cstep.
// Returns the last chunk whose MMAs were committed (-1: none); ok = false on a
// timeout.  The MMAs of chunk `ret` completing (done[ret % NS], parity
// (ret / NS) & 1) means all of them have.  land_limit bounds the waits for a
// chunk's operands to land; the waits that drain copies in flight after a
// timeout keep the full limit, so no copy is outstanding when the loop returns.
template <int S, int MT, int NT, int NS>
__device__ int mainloop(unsigned char* tsm, unsigned long long* full, unsigned long long* done, unsigned taddr,
                        const unsigned short* a0, const unsigned short* b0, long long sstride, long long cstep,
                        int nch, bool& ok, int land_limit = 1 << 24) {
  constexpr int A_SL = MT * 32, B_SL = NT * 32, STAGE = stage_bytes(S, MT, NT);
  constexpr uint32_t idesc = tc::idesc_bf16(MT, NT);
  auto produce = [&](int c, int st) {
    unsigned char* sA = tsm + st * STAGE;
    unsigned char* sB = sA + S * A_SL;
    tc::mbar_expect_tx(&full[st], STAGE);
#pragma unroll
    for (int s2 = 0; s2 < S; ++s2) {
      tc::bulk_g2s(sA + s2 * A_SL, a0 + s2 * sstride + c * cstep, A_SL, &full[st]);
      tc::bulk_g2s(sB + s2 * B_SL, b0 + s2 * sstride + c * cstep, B_SL, &full[st]);
    }
  };
  int produced = 0, landed = 0, last = -1;
  ok = true;
  for (; produced < min(NS, nch); ++produced) produce(produced, produced);
  for (int c = 0; c < nch; ++c) {
    const int st = c % NS;
    if (!tc::mbar_wait(&full[st], (c / NS) & 1, land_limit)) { ok = false; break; }
    landed = c + 1;
    tc::fence_after();
    const unsigned sa = tc::su32(tsm + st * STAGE), sb = sa + S * A_SL;
#pragma unroll
    for (int i = 0; i < S; ++i) {
      // K-major core matrices: 128 bytes apart along k, 8-line groups 256 bytes apart
      const uint64_t ad = tc::desc(sa + i * A_SL, 128, 256);
#pragma unroll
      for (int jj = 0; jj < S - i; ++jj)
        tc::mma(taddr + (unsigned)((i + jj) * NT), ad, tc::desc(sb + jj * B_SL, 128, 256), idesc, c > 0 || i > 0);
    }
    tc::commit(&done[st]);
    last = c;
    if (c >= 1 && c - 1 + NS < nch) {  // the stage of chunk c - 1 is free once its MMAs completed
      const int pc = c - 1;
      if (!tc::mbar_wait(&done[pc % NS], (pc / NS) & 1)) { ok = false; break; }
      produce(pc + NS, pc % NS);
      ++produced;
    }
  }
  if (!ok)
    for (int c = landed; c < produced; ++c) tc::mbar_wait(&full[c % NS], (c / NS) & 1);  // copies in flight
  return last;
}

}  // namespace oztc
}  // namespace dqmc
