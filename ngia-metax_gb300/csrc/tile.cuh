// tile.cuh — the register-tile update of the banded bit-parallel LCS shared
// by the alignment kernels (align.cu) and the serving kernels (serve.cu):
// band-row rings, one tile of rep blocks over the columns of a query block,
// and the build-time tuning of the tiled kernel.
#pragma once
#include <stdint.h>

#include "common.cuh"
#include "dp_asm.cuh"

// Build-time tuning of the tiled kernel: NGIA_TILED_MAIN_DNA and
// NGIA_TILED_BLOCKS_DNA set the DNA main tile width and the resident CTAs per
// SM requested from the register allocator.  On GB300 (1M DNA, s=0.85) 16
// slots at 4 CTAs ran fastest: 24 slots (3 or 2 CTAs) and 32 slots (2 CTAs)
// were 15-45% slower.
#ifndef NGIA_TILED_MAIN_DNA
#define NGIA_TILED_MAIN_DNA 16
#endif
#ifndef NGIA_TILED_BLOCKS_DNA
#define NGIA_TILED_BLOCKS_DNA 4
#endif

namespace ngia {

constexpr int kAlignThreads = 128;  // threads per CTA of every alignment kernel

// Band rows of one lane's pair, indexed by absolute rep block j.  Windows of
// up to RING blocks keep them in shared memory (row j of thread t at
// (j mod RING) * threads + t: the 32 lanes of a warp hit 32 banks); wider
// windows keep them in global scratch with the same layout over all lanes
// of the grid (a warp's accesses to one row are one 128-byte line).
template <int RING>
struct SmemRing {
  uint32_t *base;  // ring + threadIdx.x
  __device__ __forceinline__ uint32_t &operator[](int j) const { return base[(j & (RING - 1)) * kAlignThreads]; }
};
struct GlobalRing {
  uint32_t *base;  // scratch + global lane index
  uint32_t mask;   // ring size - 1 (a power of two >= the widest window)
  int64_t stride;  // lanes of the grid
  __device__ __forceinline__ uint32_t &operator[](int j) const { return base[(int64_t)(j & mask) * stride]; }
};
template <int RING>
struct RingOf {
  using T = SmemRing<RING>;
};
template <>
struct RingOf<0> {
  using T = GlobalRing;
};

// One tile: band rows base .. base+TW-1 (rows above je are padding) through
// the `cols` columns of the current query block, whose P plane words are
// cur[]; s_pl points at the representative's planes (shared or global
// memory).  cw holds the column carries into the tile (column k at bit
// 31-k after the shift below), ncw collects the carries out.  Returns the
// change of the zero count over the tile's rows.
template <int P, int TW, class Ring>
__device__ __forceinline__ int tiled_tile(const Ring &ring, const uint32_t *s_pl, int base, int je, int cols,
                                          const uint32_t (&cur)[P], uint32_t &cw, uint32_t &ncw) {
  uint32_t row[TW], pl[P][TW];
  int zold = 0;
#pragma unroll
  for (int m = 0; m < TW; m++) {
    const int j = base + m;
    const bool in = j <= je;
    row[m] = in ? ring[j] : 0u;
    zold += in ? __popc(~row[m]) : 0;
#pragma unroll
    for (int p = 0; p < P; p++) pl[p][m] = in ? s_pl[j * P + p] : 0u;
  }
  uint32_t rv[P];
#pragma unroll
  for (int p = 0; p < P; p++) rv[p] = __brev(cur[p]);
#pragma unroll 2
  for (int k = 0; k < cols; k++) {
    uint32_t mk[P];
#pragma unroll
    for (int p = 0; p < P; p++) {
      mk[p] = (uint32_t)((int)rv[p] >> 31);
      rv[p] <<= 1;
    }
    dp_tile<P, TW, true, true>(row, pl, mk, cw, ncw);
  }
  int znew = 0;
#pragma unroll
  for (int m = 0; m < TW; m++) {
    const int j = base + m;
    if (j <= je) {
      ring[j] = row[m];
      znew += __popc(~row[m]);
    }
  }
  return znew - zold;
}

// The last tile of a block row, exactly `rem` (1..MT-1, warp-uniform) slots wide.
template <int P, class Ring, int MT>
__device__ __forceinline__ int tiled_rem(int rem, const Ring &ring, const uint32_t *s_pl, int base, int je, int cols,
                                         const uint32_t (&cur)[P], uint32_t &cw, uint32_t &ncw) {
  switch (rem) {
#define NGIA_REM(W) \
  case W:           \
    if (W < MT) return tiled_tile<P, (W < MT ? W : 1), Ring>(ring, s_pl, base, je, cols, cur, cw, ncw); \
    return 0;
    NGIA_REM(1) NGIA_REM(2) NGIA_REM(3) NGIA_REM(4) NGIA_REM(5) NGIA_REM(6) NGIA_REM(7) NGIA_REM(8)
    NGIA_REM(9) NGIA_REM(10) NGIA_REM(11) NGIA_REM(12) NGIA_REM(13) NGIA_REM(14) NGIA_REM(15) NGIA_REM(16)
    NGIA_REM(17) NGIA_REM(18) NGIA_REM(19) NGIA_REM(20) NGIA_REM(21) NGIA_REM(22) NGIA_REM(23) NGIA_REM(24)
    NGIA_REM(25) NGIA_REM(26) NGIA_REM(27) NGIA_REM(28) NGIA_REM(29) NGIA_REM(30) NGIA_REM(31)
#undef NGIA_REM
    default:
      return 0;
  }
}

// Main tile width of the tiled kernel (16 slots; NGIA_TILED_MAIN_DNA for DNA).
__host__ __device__ constexpr int tiled_main(int P) { return P == 2 ? NGIA_TILED_MAIN_DNA : 16; }
__host__ __device__ constexpr int tiled_min_blocks(int P) { return P == 2 ? NGIA_TILED_BLOCKS_DNA : 2; }

}  // namespace ngia
