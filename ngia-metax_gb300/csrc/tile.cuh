// tile.cuh — the register-tile update of the banded bit-parallel LCS shared
// by the alignment kernels (align.cu) and the serving kernels (serve.cu):
// band-row rings, one tile of rep blocks over the columns of a query block,
// and the build-time tuning of the tiled kernel.
#pragma once
#include <stdint.h>

#include "common.cuh"
#include "dp_asm.cuh"

// Build-time tuning of the DNA alignment kernels (swept on GB300, 1M DNA):
//  NGIA_TILED_MAIN_DNA / NGIA_TILED_BLOCKS_DNA  main tile width and resident
//    CTAs per SM of the tiled kernel: 16 slots at 4 CTAs.  24 and 32 slots,
//    and 5 CTAs, were slower (the kernel is sensitive to its instruction
//    footprint: wider tiles mean larger unrolled bodies).  With the FMA-pipe
//    bookkeeping: 4 CTAs 0.723 of the INT32 bound, 5 CTAs (95 registers)
//    0.685, the main tiles without prefetch 0.691, both 0.669.
//  NGIA_ALIGN_EQ / NGIA_WIN_EQ  match words from the representative's match
//    table (1) instead of from plane registers (0): 16% (tiled, s=0.85) and
//    12-26% (window kernels, s=0.9-0.95) more candidate seqs/s.
//  NGIA_EQ_UNROLL  columns per loop trip of the match-table tile: 1.  Two,
//    four and eight ran at 0.92x, 0.64x and 0.41x: the larger bodies miss in
//    the instruction cache.
//  NGIA_EQ_PF_MAIN / NGIA_EQ_PF_WIN  load the next column's match words
//    during the current column (eq_columns) in the main tiled tile / the
//    window kernels: main on (+2% at s=0.85 and 0.9, -5% at 0.95), windows
//    off (+30% for the 32-block window class alone at s=0.85-0.9, but slower
//    at 0.95 and no faster overall).
//  (Running the last main tile and the remainder as one tile of 17-31 slots,
//  to save a tile's per-column overhead, ran at 0.45x.)
//  NGIA_EQ_REM_ROUND  remainder tiles rounded up to a multiple of this
//    width (fewer tile variants, more padding slots): 1 (2 and 4 no faster).
#ifndef NGIA_TILED_MAIN_DNA
#define NGIA_TILED_MAIN_DNA 16
#endif
#ifndef NGIA_TILED_BLOCKS_DNA
#define NGIA_TILED_BLOCKS_DNA 4
#endif
#ifndef NGIA_ALIGN_EQ
#define NGIA_ALIGN_EQ 1
#endif
#ifndef NGIA_WIN_EQ
#define NGIA_WIN_EQ 1
#endif
#ifndef NGIA_SERVE_EQ
#define NGIA_SERVE_EQ 1
#endif
// NGIA_SERVE_PF: next-column prefetch in the serving / round kernel's main
// tiles; off (with the FMA-pipe bookkeeping: 60.2k against 64.3k queries/s).
#ifndef NGIA_SERVE_PF
#define NGIA_SERVE_PF 0
#endif
#ifndef NGIA_EQ_UNROLL
#define NGIA_EQ_UNROLL 1
#endif
#ifndef NGIA_EQ_PF_MAIN
#define NGIA_EQ_PF_MAIN 1
#endif
#ifndef NGIA_EQ_PF_WIN
#define NGIA_EQ_PF_WIN 0
#endif
#ifndef NGIA_EQ_REM_ROUND
#define NGIA_EQ_REM_ROUND 1
#endif
//  NGIA_EQ_FMA  1: the tiled DNA kernel takes each column's code, the match
//    words' address and the tile's carry pop/push as multiply-adds by
//    run-time constants (IMAD on the FMA pipe, which the ALU-bound kernel
//    leaves idle) instead of logic/shift/add instructions on the ALU pipe:
//    +2.9% candidate seqs/s (k_align_tiled<2,64>: 7.43 -> 7.26 ms/launch).
//  NGIA_EQ_NOZOLD  1 (with NGIA_EQ_FMA): a tile returns the zero count of
//    its rows after the block (their sum is the window's count) instead of
//    the change, so the rows' zero count before the block is not taken:
//    +1.5% more (7.06 ms/launch; frac 0.688 -> 0.724 of the 3-instruction
//    bound together).
//  NGIA_EQ_MADC  with NGIA_EQ_FMA: every k-th slot's add-with-carry as a
//    multiply-add with carry (IMAD.X) by a run-time 1; 0 = none (k = 2, 3
//    ran at 0.97x, 0.98x: the core chain stays on the ALU pipe).
#ifndef NGIA_EQ_FMA
#define NGIA_EQ_FMA 1
#endif
#ifndef NGIA_EQ_MADC
#define NGIA_EQ_MADC 0
#endif
#ifndef NGIA_EQ_NOZOLD
#define NGIA_EQ_NOZOLD 1
#endif
//  NGIA_EQ_ZCARRY  1 (with NGIA_EQ_FMA): the tiles count no zeros at all.
//    Over one column a window's zero count grows by exactly the carry out of
//    its top row (with carry 0 into its bottom; checked exhaustively on
//    small widths), so when every busy lane of the warp fills the warp's
//    tiles exactly (no padding slot above its window) the block's growth is
//    the popcount of the last tile's carry-out word; otherwise the window is
//    recounted from the ring.  Off: on GB300 (1M DNA, s=0.85) it ran at
//    0.99x (7.11 vs 7.07 ms per launch); the warp vote and the recounts of
//    windows that do not fill their tiles cost more than the popcounts saved.
//  NGIA_TILED_MERGE1  1 (with NGIA_EQ_FMA): when a warp's windows leave a
//    one-slot remainder (the dominant 49-block window of 1M DNA s=0.85 is
//    16+16+16+1), the last main tile and that slot run as one tile of MT+1
//    slots, saving a tile's per-column overhead.  Off: 0.99x on GB300
//    (7.15 vs 7.07 ms per launch, 1M DNA s=0.85; with straight tiles 6.85
//    against 6.83 ms).
//  NGIA_WIN_FMA  1: the register-window kernels take each column's code and
//    the match words' address as multiply-adds on the FMA pipe, as the tiled
//    kernel does.  Off: no difference on GB300 (the 32-block class of 1M DNA
//    0.444 ms per iteration either way, the 20,000-sequence job's graph
//    form 2.93-3.00 s): these classes' launches are bound by latency.
#ifndef NGIA_WIN_FMA
#define NGIA_WIN_FMA 0
#endif
#ifndef NGIA_TILED_MERGE1
#define NGIA_TILED_MERGE1 0
#endif
#ifndef NGIA_EQ_ZCARRY
#define NGIA_EQ_ZCARRY 0
#endif
//  NGIA_TILE_STRAIGHT  1: a main tile whose rows lie inside the lane's
//    window and do not wrap around the shared-memory ring loads and stores
//    them at one base address with immediate offsets, without the per-row
//    window test, and counts their zeros from one sum of population counts;
//    NGIA_TILE_STRAIGHT_REM the same for the remainder tiles.  1M DNA
//    s=0.85: 7.07 -> 6.84 ms per launch (main tiles), 6.82 (both): 0.723 ->
//    0.749 of the 3-instruction bound.
//  NGIA_SERVE_STRAIGHT  the same for the tiles with the match table in
//    global memory (representative per pair).  Off: no difference on the
//    service (64.1k against 64.7k queries/s capacity on 200 DNA query
//    batches against 14,077 resident representatives).
#ifndef NGIA_TILE_STRAIGHT
#define NGIA_TILE_STRAIGHT 1
#endif
#ifndef NGIA_TILE_STRAIGHT_REM
#define NGIA_TILE_STRAIGHT_REM 1
#endif
//  NGIA_ZC_SKIP  1: a warp counts its rows' zeros after a query block only
//    when one of its lanes could fail the rejection test there.  Zeros
//    never decrease and the residues left fall by at most 32 per block, so
//    after a count with slack S = zeros + residues left - cutoff >= 0 the
//    next floor(S / 32) blocks cannot reject; the pair is rejected at the
//    same block as with a count after every block.  Off: slower on GB300
//    (1M DNA s=0.85: 6.88 against 6.83 ms per launch; the warp vote and the
//    branch cost more than the population counts they skip).
#ifndef NGIA_ZC_SKIP
#define NGIA_ZC_SKIP 0
#endif
//  NGIA_EQ_PF_REM  1: the remainder tiles also load the next column's match
//    words during the current one.  Off: the tiled launch alone 6.75 against
//    6.83 ms (plain-driver replay), but the graph-driven iterations, where
//    the length buckets' launches overlap, no faster (136.15M against
//    136.17M candidate seqs/s).
#ifndef NGIA_EQ_PF_REM
#define NGIA_EQ_PF_REM 0
#endif
#ifndef NGIA_SERVE_STRAIGHT
#define NGIA_SERVE_STRAIGHT 0
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
  static constexpr int kSize = RING;
  uint32_t *base;  // ring + threadIdx.x
  __device__ __forceinline__ uint32_t &operator[](int j) const { return base[(j & (RING - 1)) * kAlignThreads]; }
  __device__ __forceinline__ uint32_t *at(int j) const { return base + (j & (RING - 1)) * kAlignThreads; }
};
struct GlobalRing {
  static constexpr int kSize = 0;  // no straight-tile path
  __device__ __forceinline__ uint32_t *at(int) const { return nullptr; }
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

// DNA match table: for every rep block j its four match words, word 4j + c =
// the rows of block j whose residue is c (c = plane-0 bit | plane-1 bit << 1),
// i.e. ~(p0 ^ m0) & ~(p1 ^ m1) for the masks of residue c — the same words
// the plane form builds per column.  kEqPad zero blocks follow the last rep
// block, so a tile's padding slots (rows above je, whose row words are 0 and
// mask whatever they read) stay inside the table.
constexpr int kEqPad = 32;
constexpr int kEqUnroll = NGIA_EQ_UNROLL;  // columns per loop trip of tiled_tile_eq
__host__ __device__ constexpr int eq_words(int max_nb) { return 4 * (max_nb + kEqPad); }
// Word offset of the match table in the tiled kernel's dynamic shared memory:
// after the planes, the k-mer bitset and the row ring (ring = 0: global ring).
__host__ __device__ constexpr int tiled_eq_off(int P, int max_nb, int ring) {
  return ((max_nb * P + 3) & ~3) + kListWords + ring * kAlignThreads;
}

// Builds the match table of the representative whose planes are staged at
// s_pl (nb1 blocks) with all threads of the CTA; the caller synchronises.
__device__ __forceinline__ void build_eq(const uint32_t *s_pl, int nb1, uint32_t *s_eq) {
  for (int j = threadIdx.x; j < nb1 + kEqPad; j += blockDim.x) {
    const bool real = j < nb1;
    const uint32_t p0 = real ? s_pl[2 * j] : 0u, p1 = real ? s_pl[2 * j + 1] : 0u;
    uint4 e;
    e.x = real ? ~p0 & ~p1 : 0u;
    e.y = p0 & ~p1;
    e.z = ~p0 & p1;
    e.w = p0 & p1;
    *reinterpret_cast<uint4 *>(s_eq + 4 * j) = e;
  }
}

// Column codes of one 32-residue query block as byte offsets into a block's
// four match words: column k's offset 4c sits in bits 4(k%8)..4(k%8)+3 of
// q[k/8].
__device__ __forceinline__ void eq_codes(const uint32_t (&cur)[2], uint32_t (&q)[4]) {
#pragma unroll
  for (int s = 0; s < 4; s++) {
    uint32_t a = (cur[0] >> (8 * s)) & 0xFFu, b = (cur[1] >> (8 * s)) & 0xFFu;
    a = (a | (a << 12)) & 0x000F000Fu;
    a = (a | (a << 6)) & 0x03030303u;
    a = (a | (a << 3)) & 0x11111111u;
    b = (b | (b << 12)) & 0x000F000Fu;
    b = (b | (b << 6)) & 0x03030303u;
    b = (b | (b << 3)) & 0x11111111u;
    q[s] = (a << 2) | (b << 3);
  }
}

// Match words of the TW slots at eb (block-major table, byte offset `off`
// selects the residue's word of each block).
template <int TW>
__device__ __forceinline__ void eq_load(uint32_t (&e)[TW], const char *eb, uint32_t off) {
  const uint32_t *p = reinterpret_cast<const uint32_t *>(eb + off);
#pragma unroll
  for (int m = 0; m < TW; m++) e[m] = p[4 * m];
}

// All `cols` columns of one query block through a register tile of TW
// slots whose match words start at eb; CC: the tile takes column carries in
// cw and hands them out in ncw.  PF: the next column's match words are loaded
// while the current column updates (two columns per loop trip), hiding the
// shared-memory latency behind the carry chain; loads past the last column
// read offset 0 (in bounds, unused).
template <int TW, bool CC, bool PF>
__device__ __forceinline__ void eq_columns(uint32_t (&row)[TW], const char *eb, const uint32_t (&q)[4], int cols,
                                           uint32_t &cw, uint32_t &ncw) {
  uint32_t w0 = q[0], w1 = q[1], w2 = q[2], w3 = q[3];
  for (int k0 = 0; k0 < cols; k0 += 8) {
    uint32_t w = w0;
    w0 = w1;
    w1 = w2;
    w2 = w3;
    const int n = min(8, cols - k0);
    if constexpr (PF) {
      uint32_t ea[TW], eo[TW];
      eq_load<TW>(ea, eb, w & 12u);
      w >>= 4;
      int k = 0;
#pragma unroll 1
      for (; k + 2 <= n; k += 2) {
        eq_load<TW>(eo, eb, w & 12u);
        w >>= 4;
        dp_tile_eq<TW, CC, CC>(row, ea, cw, ncw);
        eq_load<TW>(ea, eb, w & 12u);
        w >>= 4;
        dp_tile_eq<TW, CC, CC>(row, eo, cw, ncw);
      }
      if (k < n) dp_tile_eq<TW, CC, CC>(row, ea, cw, ncw);
    } else {
#pragma unroll kEqUnroll
      for (int k = 0; k < n; k++) {
        uint32_t ev[TW];
        eq_load<TW>(ev, eb, w & 12u);
        w >>= 4;
        dp_tile_eq<TW, CC, CC>(row, ev, cw, ncw);
      }
    }
  }
}

// tiled_tile for DNA with the match table: per column one shared-memory load
// per slot and three integer instructions per 32 cells (AND, add with carry,
// LOP3) instead of four.  s_eq points at the table; q holds the column codes.
template <int TW, bool PF, class Ring>
__device__ __forceinline__ int tiled_tile_eq(const Ring &ring, const uint32_t *s_eq, int base, int je, int nb1,
                                             int cols, const uint32_t (&q)[4], uint32_t &cw, uint32_t &ncw) {
  uint32_t row[TW];
  int zold = 0;
#pragma unroll
  for (int m = 0; m < TW; m++) {
    const int j = base + m;
    const bool in = j <= je;
    row[m] = in ? ring[j] : 0u;
    zold += in ? __popc(~row[m]) : 0;
  }
  // A tile past the rep's last block (a lane with a narrower window than its
  // warp's widest) is all padding: it reads the zero blocks after nb1.
  const char *eb = reinterpret_cast<const char *>(s_eq + 4 * min(base, nb1));
  eq_columns<TW, true, PF>(row, eb, q, cols, cw, ncw);
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

// ---- match-table tiles with the per-column bookkeeping on the FMA pipe -------
// Run-time constants 1 and 4: ptxas cannot fold a multiply by them into a
// shift or an add, so the multiply-adds below stay IMADs (FMA pipe).
struct FmaK {
  uint32_t one, four;
};

// Bit i of x (i < 16) to bit 2i.
__device__ __forceinline__ uint32_t spread16(uint32_t x) {
  x &= 0xFFFFu;
  x = (x | (x << 8)) & 0x00FF00FFu;
  x = (x | (x << 4)) & 0x0F0F0F0Fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

// Column codes of one 32-residue query block, first column on top: w[h]
// holds columns 16h..16h+15, two bits each (plane-1 bit above plane-0 bit),
// column 16h in bits 31..30.
__device__ __forceinline__ void eq_codes_top(const uint32_t (&cur)[2], uint32_t (&w)[2]) {
  const uint32_t r0 = __brev(cur[0]), r1 = __brev(cur[1]);
  w[0] = spread16(r0 >> 16) | (spread16(r1 >> 16) << 1);
  w[1] = spread16(r0) | (spread16(r1) << 1);
}

// Shared-memory address of the next column's match words: code = w >> 30,
// w <<= 2, address = eb + 4 code — three multiply-adds.
__device__ __forceinline__ uint32_t eq_next_addr(uint32_t &w, uint32_t eb, const FmaK &k) {
  uint32_t c, a;
  asm("mul.hi.u32 %0, %1, %2;" : "=r"(c) : "r"(w), "r"(k.four));
  asm("mul.lo.u32 %0, %0, %1;" : "+r"(w) : "r"(k.four));
  asm("mad.lo.u32 %0, %1, %2, %3;" : "=r"(a) : "r"(c), "r"(k.four), "r"(eb));
  return a;
}

// Match words of TW slots at shared address a (slot m at a + 16 m; the
// offsets are immediates of the loads).
template <int M, int TW>
struct EqLoad {
  static __device__ __forceinline__ void run(uint32_t (&e)[TW], uint32_t a) {
    EqLoad<M - 1, TW>::run(e, a);
    asm volatile("ld.shared.u32 %0, [%1+%2];" : "=r"(e[M - 1]) : "r"(a), "n"(16 * (M - 1)));
  }
};
template <int TW>
struct EqLoad<0, TW> {
  static __device__ __forceinline__ void run(uint32_t (&)[TW], uint32_t) {}
};
template <int TW>
__device__ __forceinline__ void eq_load_s(uint32_t (&e)[TW], uint32_t a) {
  EqLoad<TW, TW>::run(e, a);
}

// eq_columns with the codes on top of w[] and the FMA-pipe bookkeeping.
template <int TW, bool CC, bool PF>
__device__ __forceinline__ void eq_columns_f(uint32_t (&row)[TW], uint32_t eb, const uint32_t (&wc)[2], int cols,
                                             uint32_t &cw, uint32_t &ncw, const FmaK &k) {
#pragma unroll 1
  for (int h = 0; h < 2; h++) {
    const int n = min(16, cols - 16 * h);
    if (n <= 0) break;
    uint32_t w = wc[h];
    if constexpr (PF) {
      uint32_t ea[TW], eo[TW];
      eq_load_s<TW>(ea, eq_next_addr(w, eb, k));
      int c = 0;
#pragma unroll 1
      for (; c + 2 <= n; c += 2) {
        eq_load_s<TW>(eo, eq_next_addr(w, eb, k));
        dp_tile_eqf<TW, CC, CC, NGIA_EQ_MADC>(row, ea, cw, ncw, k.one);
        eq_load_s<TW>(ea, eq_next_addr(w, eb, k));  // past the last column: code 0, in bounds
        dp_tile_eqf<TW, CC, CC, NGIA_EQ_MADC>(row, eo, cw, ncw, k.one);
      }
      if (c < n) dp_tile_eqf<TW, CC, CC, NGIA_EQ_MADC>(row, ea, cw, ncw, k.one);
    } else {
#pragma unroll 1
      for (int c = 0; c < n; c++) {
        uint32_t ev[TW];
        eq_load_s<TW>(ev, eq_next_addr(w, eb, k));
        dp_tile_eqf<TW, CC, CC, NGIA_EQ_MADC>(row, ev, cw, ncw, k.one);
      }
    }
  }
}

// tiled_tile_eq with the FMA-pipe bookkeeping; s_eq_s is the table's
// shared-memory address.  NGIA_EQ_NOZOLD: returns the zero count of the
// tile's rows after the block instead of its change.
// Straight tile: rows base .. base+TW-1 all inside the lane's window
// (<= je) and contiguous in the shared-memory ring (no wrap).  Its rows are
// then at rp + m * threads, immediate offsets from one address.
template <int TW, class Ring>
__device__ __forceinline__ bool tile_straight(const Ring &ring, int base, int je, uint32_t *&rp) {
  if constexpr (Ring::kSize >= TW) {
    rp = ring.at(base);
    return base + TW - 1 <= je && (base & (Ring::kSize - 1)) + TW <= Ring::kSize;
  } else {
    rp = nullptr;
    return false;
  }
}
template <int TW>
__device__ __forceinline__ void tile_load_straight(uint32_t (&row)[TW], const uint32_t *rp) {
#pragma unroll
  for (int m = 0; m < TW; m++) row[m] = rp[m * kAlignThreads];
}
// Stores a straight tile's rows; returns their zero count (ZC) or 0.
template <int TW, bool ZC>
__device__ __forceinline__ int tile_store_straight(const uint32_t (&row)[TW], uint32_t *rp, bool cnt = true) {
#pragma unroll
  for (int m = 0; m < TW; m++) rp[m * kAlignThreads] = row[m];
  if (!ZC || !cnt) return 0;
  int ones = 0;
#pragma unroll
  for (int m = 0; m < TW; m++) ones += __popc(row[m]);
  return 32 * TW - ones;
}

template <int TW, bool PF, class Ring, bool ZC = true, bool ST = NGIA_TILE_STRAIGHT>
__device__ __forceinline__ int tiled_tile_eqf(const Ring &ring, uint32_t s_eq_s, int base, int je, int nb1, int cols,
                                              const uint32_t (&wc)[2], uint32_t &cw, uint32_t &ncw, const FmaK &k,
                                              bool cnt = true) {
  uint32_t row[TW];
  int zold = 0;
  uint32_t *rp = nullptr;
  bool straight = false;
  if constexpr (ST && NGIA_EQ_NOZOLD) straight = tile_straight<TW>(ring, base, je, rp);
  if (straight) {
    tile_load_straight<TW>(row, rp);
  } else {
#pragma unroll
    for (int m = 0; m < TW; m++) {
      const int j = base + m;
      const bool in = j <= je;
      row[m] = in ? ring[j] : 0u;
      if (ZC && !NGIA_EQ_NOZOLD) zold += in ? __popc(~row[m]) : 0;
    }
  }
  eq_columns_f<TW, true, PF>(row, s_eq_s + 16u * (uint32_t)min(base, nb1), wc, cols, cw, ncw, k);
  if (straight) return tile_store_straight<TW, ZC>(row, rp, cnt);
  int znew = 0;
#pragma unroll
  for (int m = 0; m < TW; m++) {
    const int j = base + m;
    if (j <= je) {
      ring[j] = row[m];
      if (ZC && cnt) znew += __popc(~row[m]);
    }
  }
  return znew - zold;
}

template <class Ring, int MT, bool ZC = true>
__device__ __forceinline__ int tiled_rem_eqf(int rem, const Ring &ring, uint32_t s_eq_s, int base, int je, int nb1,
                                             int cols, const uint32_t (&wc)[2], uint32_t &cw, uint32_t &ncw,
                                             const FmaK &k, bool cnt = true) {
  switch (rem) {
#define NGIA_REM(W) \
  case W:           \
    if (W < MT) return tiled_tile_eqf<(W < MT ? W : 1), NGIA_EQ_PF_REM != 0, Ring, ZC, NGIA_TILE_STRAIGHT_REM>(ring, s_eq_s, base, je, nb1, cols, wc, cw, ncw, k, cnt); \
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

// ---- the same bookkeeping with the match table in global memory ------------
// (kernels that take the representative per pair read its table through L1)
__device__ __forceinline__ uint64_t eq_next_addr_g(uint32_t &w, uint64_t eb, const FmaK &k) {
  uint32_t c;
  uint64_t a;
  asm("mul.hi.u32 %0, %1, %2;" : "=r"(c) : "r"(w), "r"(k.four));
  asm("mul.lo.u32 %0, %0, %1;" : "+r"(w) : "r"(k.four));
  asm("mad.wide.u32 %0, %1, %2, %3;" : "=l"(a) : "r"(c), "r"(k.four), "l"(eb));
  return a;
}

template <int M, int TW>
struct EqLoadG {
  static __device__ __forceinline__ void run(uint32_t (&e)[TW], uint64_t a) {
    EqLoadG<M - 1, TW>::run(e, a);
    asm volatile("ld.global.nc.u32 %0, [%1+%2];" : "=r"(e[M - 1]) : "l"(a), "n"(16 * (M - 1)));
  }
};
template <int TW>
struct EqLoadG<0, TW> {
  static __device__ __forceinline__ void run(uint32_t (&)[TW], uint64_t) {}
};

template <int TW, bool CC, bool PF>
__device__ __forceinline__ void eq_columns_fg(uint32_t (&row)[TW], uint64_t eb, const uint32_t (&wc)[2], int cols,
                                              uint32_t &cw, uint32_t &ncw, const FmaK &k) {
#pragma unroll 1
  for (int h = 0; h < 2; h++) {
    const int n = min(16, cols - 16 * h);
    if (n <= 0) break;
    uint32_t w = wc[h];
    if constexpr (PF) {
      uint32_t ea[TW], eo[TW];
      EqLoadG<TW, TW>::run(ea, eq_next_addr_g(w, eb, k));
      int c = 0;
#pragma unroll 1
      for (; c + 2 <= n; c += 2) {
        EqLoadG<TW, TW>::run(eo, eq_next_addr_g(w, eb, k));
        dp_tile_eqf<TW, CC, CC, NGIA_EQ_MADC>(row, ea, cw, ncw, k.one);
        EqLoadG<TW, TW>::run(ea, eq_next_addr_g(w, eb, k));  // past the last column: code 0, in bounds
        dp_tile_eqf<TW, CC, CC, NGIA_EQ_MADC>(row, eo, cw, ncw, k.one);
      }
      if (c < n) dp_tile_eqf<TW, CC, CC, NGIA_EQ_MADC>(row, ea, cw, ncw, k.one);
    } else {
#pragma unroll 1
      for (int c = 0; c < n; c++) {
        uint32_t ev[TW];
        EqLoadG<TW, TW>::run(ev, eq_next_addr_g(w, eb, k));
        dp_tile_eqf<TW, CC, CC, NGIA_EQ_MADC>(row, ev, cw, ncw, k.one);
      }
    }
  }
}

// tiled_tile_eqf with the table at global address eqb; returns the zero
// count of the tile's rows after the block.
template <int TW, bool PF, class Ring>
__device__ __forceinline__ int tiled_tile_eqfg(const Ring &ring, uint64_t eqb, int base, int je, int nb1, int cols,
                                               const uint32_t (&wc)[2], uint32_t &cw, uint32_t &ncw, const FmaK &k) {
  uint32_t row[TW];
  uint32_t *rp = nullptr;
  bool straight = false;
  if constexpr (NGIA_SERVE_STRAIGHT != 0) straight = tile_straight<TW>(ring, base, je, rp);
  if (straight) {
    tile_load_straight<TW>(row, rp);
  } else {
#pragma unroll
    for (int m = 0; m < TW; m++) {
      const int j = base + m;
      row[m] = j <= je ? ring[j] : 0u;
    }
  }
  eq_columns_fg<TW, true, PF>(row, eqb + 16ull * (uint64_t)min(base, nb1), wc, cols, cw, ncw, k);
  if (straight) return tile_store_straight<TW, true>(row, rp);
  int znew = 0;
#pragma unroll
  for (int m = 0; m < TW; m++) {
    const int j = base + m;
    if (j <= je) {
      ring[j] = row[m];
      znew += __popc(~row[m]);
    }
  }
  return znew;
}

// The last tile of a block row: `rem` slots rounded up to a multiple of R
// (1..32; fewer tile bodies for kernels whose warps see many window widths).
template <class Ring, int R>
__device__ __forceinline__ int tiled_rem_eqfg(int rem, const Ring &ring, uint64_t eqb, int base, int je, int nb1,
                                              int cols, const uint32_t (&wc)[2], uint32_t &cw, uint32_t &ncw,
                                              const FmaK &k) {
  switch ((rem + R - 1) / R * R) {
#define NGIA_REMG(W) \
  case W:            \
    if (W % R == 0) return tiled_tile_eqfg<W % R == 0 ? W : 1, false, Ring>(ring, eqb, base, je, nb1, cols, wc, cw, ncw, k); \
    return 0;
    NGIA_REMG(1) NGIA_REMG(2) NGIA_REMG(3) NGIA_REMG(4) NGIA_REMG(5) NGIA_REMG(6) NGIA_REMG(7) NGIA_REMG(8)
    NGIA_REMG(9) NGIA_REMG(10) NGIA_REMG(11) NGIA_REMG(12) NGIA_REMG(13) NGIA_REMG(14) NGIA_REMG(15) NGIA_REMG(16)
#undef NGIA_REMG
    default:
      return 0;
  }
}

constexpr int kEqRemRound = NGIA_EQ_REM_ROUND;  // remainder tile widths: multiples of this

template <class Ring, int MT>
__device__ __forceinline__ int tiled_rem_eq(int rem, const Ring &ring, const uint32_t *s_eq, int base, int je,
                                            int nb1, int cols, const uint32_t (&q)[4], uint32_t &cw, uint32_t &ncw) {
  switch (rem) {
#define NGIA_REM(W) \
  case W:           \
    if (W < MT && W % kEqRemRound == 0)                                                                     \
      return tiled_tile_eq<(W < MT && W % kEqRemRound == 0 ? W : kEqRemRound), false, Ring>(ring, s_eq, base, je, nb1,  \
                                                                                     cols, q, cw, ncw);         \
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
