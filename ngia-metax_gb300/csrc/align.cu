// align.cu — banded bit-parallel LCS identity kernels (the reference's
// kernel_dynamicGen/Pro, CUDA/signalNode/src/func.cu:450-604).
//
// The reference computes, per (representative, query) pair, a block-banded
// form of the Allison–Dix / Hyyrö bit-vector LCS: the representative's net
// residues are the rows (32 per word, line[j]), the query's net residues the
// columns, processed in 32-column blocks i.  For query block i only rep
// blocks j in [max(i-B,0), min(i+B,nb1-1)] are updated, with
// B = (ceil(fma(-L2,s,L1)) + 31)/32; the carry into the lowest band block is
// 0 and the carry out of the highest is dropped; blocks outside the band keep
// their state.  The score is the number of zero bits of line[] over the net
// length, accepted when >= ceil(L2*s).
//
// Two kernels reproduce that exactly:
//
// k_align_win<P,WC>  one thread per pair.  The band window (at most WC rep
//   blocks) lives in registers: row[m] for slot m = rep block js+m.  For each
//   query residue the whole window is updated as one multi-word addition
//   whose carries ride the hardware carry flag (add.cc/addc.cc).  The match
//   word of a slot comes, for DNA, from the representative's match table in
//   shared memory (four words per rep block, one per residue code; tile.cuh),
//   so a 32-cell word costs one load and three integer instructions (AND,
//   IADD3.X, LOP3); protein builds it from the rep's planes held in registers
//   (one LOP3 per plane).  When the band slides, the departing block's zero
//   count is banked and the registers shift down one slot; an entering block
//   starts all-ones.  Lanes claim pairs from the class queue independently
//   (warp-aggregated atomics).
//
// k_align_tiled<P,RING>  wider windows: one thread per pair, the band rows
//   in a ring (shared memory for windows up to RING = 64 or 128 blocks,
//   global scratch for any width with RING = 0), updated tile by tile with
//   the same generated instruction sequences.
//
// Both stop a pair early once it provably cannot reach the cutoff: each query
// residue raises the counted zeros by at most one (the bit-vector update only
// moves a zero downwards within a run of ones, or adds one at the top of the
// updated segment), so zeros_now + residues_left < cutoff is a rejection.
// Accepted pairs are always computed to the end (their score is reported).
#include <algorithm>
#include <climits>
#include <cstdlib>
#include <mutex>

#include "ctx.h"
#include "tile.cuh"

namespace ngia {

constexpr int kRepPlanesOff = 32;  // planes offset inside rb.rep_rec (filter.cu)

// Resident CTAs per SM requested from the register allocator for the
// register-window kernel of P planes and WC slots.
__host__ __device__ constexpr int win_min_blocks(int P, int WC) {
  return P == 2 ? (WC <= 8 ? 6 : WC <= 16 ? 4 : WC <= 24 ? 3 : 2) : (WC <= 8 ? 4 : 2);
}

struct AlignHdr {
  int qn, L1, net1, nb1, word_after, rep;
};

// Reads the iteration header and stages the representative's planes (and,
// when the short-word test follows the alignment, its k-mer bitset) into
// shared memory with bulk copies.  Returns false when there is no work.
template <int P>
// warp_mode: 1 for the warp-per-pair kernel (works on classes with at most
// warp_pairs pairs), 0 for the thread-per-pair kernels (more than that); the
// other kernel of a class returns here, before any staging.
__device__ __forceinline__ bool align_setup(const DevDB &db, const RunBufs &rb, const RunParams &prm, int cls,
                                            int score_mode, int warp_pairs, int warp_mode, uint32_t *smem,
                                            uint64_t *bar, AlignHdr &h) {
  __shared__ int s_hdr[6];
  RunState *st = rb.st;
  if (threadIdx.x == 0) {
    const bool skip = !score_mode && (st->done || st->iter >= st->iter_limit || st->err);
    const int qn = skip ? 0 : (int)st->qcount[cls];
    const bool mine = warp_mode ? qn <= warp_pairs : qn > warp_pairs;
    // warp-per-pair: one pair per warp of this CTA
    const bool idle = warp_mode && (int)(blockIdx.x * (blockDim.x >> 5)) >= qn;
    s_hdr[0] = mine && !idle ? qn : 0;
    s_hdr[1] = st->rep_len;
    s_hdr[2] = st->rep_net;
    s_hdr[3] = st->rep_nb;
    s_hdr[4] = !score_mode && st->word_active && !st->word_first;
    s_hdr[5] = st->rep;
  }
  __syncthreads();
  h.qn = s_hdr[0];
  if (h.qn == 0) return false;
  h.L1 = s_hdr[1];
  h.net1 = s_hdr[2];
  h.nb1 = s_hdr[3];
  h.word_after = s_hdr[4];
  h.rep = s_hdr[5];
  const uint32_t plane_words = (uint32_t)((h.nb1 * P + 3) & ~3);
  const uint32_t list_words = h.word_after ? (uint32_t)max(4, (int)((1u << (prm.w * (P == 2 ? 2 : 5))) / 32u)) : 0u;
  if (threadIdx.x == 0) {
    mbar_init(bar, 1);
    const uint32_t bytes = 4u * (plane_words + list_words);
    if (bytes) {
      mbar_expect_tx(bar, bytes);
      if (plane_words) bulk_g2s(smem, rb.rep_rec + kRepPlanesOff, 4u * plane_words, bar);
      if (list_words) bulk_g2s(smem + plane_words, rb.rep_list, 4u * list_words, bar);
    } else {
      asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
    }
  }
  __syncthreads();
  bool ok = mbar_wait_bounded(bar, 0, prm.wait_polls);
  if (!ok) {
    set_error(st, NGIA_ERR_MBAR_TIMEOUT, 10 + cls);
    mbar_wait_bounded(bar, 0, kWaitPolls);  // let the copy in flight land
  }
  return __syncthreads_and(ok);
}

// Claims the next queue entry for every idle lane with one atomic per warp.
// state: -1 idle, -2 queue exhausted, >= 0 the claimed entry.
__device__ __forceinline__ void claim(RunState *st, int cls, int qn, int lane, int &state) {
  const bool need = state == -1;
  const unsigned nm = __ballot_sync(kFullMask, need);
  if (!nm) return;
  const int leader = __ffs(nm) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&st->qhead[cls], (uint32_t)__popc(nm));
  base = __shfl_sync(kFullMask, base, leader);
  if (need) {
    const uint32_t idx = base + (uint32_t)__popc(nm & ((1u << lane) - 1u));
    state = idx < (uint32_t)qn ? (int)idx : -2;
  }
}

// Outcome of one pair: membership (or the pair score in score mode).
template <int P>
__device__ __forceinline__ void finish_pair(const DevDB &db, const RunBufs &rb, const RunParams &prm,
                                            const AlignHdr &h, int score_mode, int entry, int cand, int sum,
                                            int cutoff, int L2, int net2, const uint32_t *qpl,
                                            const uint32_t *s_list, unsigned long long &members) {
  if (score_mode) {
    rb.score_out[4 * entry + 2] = sum;
    return;
  }
  bool pass = !(sum < cutoff);
  if (pass && h.word_after) {
    // short-word test of func.cu:376-396, evaluated only for aligned members
    int ws = 0;
    {
      constexpr int bits = P == 2 ? 2 : 5;
      const uint32_t mask = (1u << (prm.w * bits)) - 1u;
      uint32_t word = 0;
      for (int i = 0; i < net2; i += 32) {
        uint32_t pl[P];
#pragma unroll
        for (int p = 0; p < P; p++) pl[p] = qpl[(i >> 5) * P + p];
        const int lim = min(32, net2 - i);
        for (int j = 0; j < lim; j++) {
          uint32_t c = 0;
#pragma unroll
          for (int p = 0; p < P; p++) c |= ((pl[p] >> j) & 1u) << p;
          word = ((word << bits) | c) & mask;
          if (i + j >= prm.w - 1) ws += (s_list[word >> 5] >> (word & 31)) & 1u;
        }
      }
    }
    pass = !(ws < word_min(L2, prm.w, prm.s));
  }
  if (pass) {
    rb.cluster[cand] = h.rep;
    rb.ident[cand] = sum;
    atomicAnd(&rb.alive[cand >> 5], ~(1u << (cand & 31)));
    members++;
  }
}

__device__ __forceinline__ void flush_align_stats(RunState *st, int cls, unsigned long long pairs,
                                                  unsigned long long members, unsigned long long cells,
                                                  unsigned long long done, unsigned long long *s_qwords) {
  for (int o = 16; o; o >>= 1) {
    pairs += __shfl_down_sync(kFullMask, pairs, o);
    members += __shfl_down_sync(kFullMask, members, o);
    cells += __shfl_down_sync(kFullMask, cells, o);
    done += __shfl_down_sync(kFullMask, done, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (pairs) atomicAdd(&st->st_align_pairs, pairs);
    if (members) atomicAdd(&st->st_members, members);
    if (cells) atomicAdd(&st->st_band_cells, cells);
    if (done) {
      atomicAdd(&st->st_done_cells, done * 32ull);
      atomicAdd(&st->st_class_done[cls], done * 32ull);
    }
  }
  __syncthreads();
  if (threadIdx.x == 0 && *s_qwords) atomicAdd(&st->st_class_qwords[cls], *s_qwords);
}

template <int P, int WC>
__global__ void __launch_bounds__(kAlignThreads, win_min_blocks(P, WC))
    k_align_win(DevDB db, RunBufs rb, RunParams prm, int cls, int score_mode, int warp_pairs) {
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ uint64_t bar;
  AlignHdr h;
  __shared__ unsigned long long s_qw;  // query plane words of the pairs taken (algorithmic bytes / 4)
  if (threadIdx.x == 0) s_qw = 0;
  if (!align_setup<P>(db, rb, prm, cls, score_mode, warp_pairs, 0, smem, &bar, h)) return;
  const uint32_t *s_pl = smem;
  const uint32_t *s_list = smem + ((h.nb1 * P + 3) & ~3);
  constexpr bool kEq = P == 2 && NGIA_WIN_EQ;
  uint32_t *s_eq = smem + tiled_eq_off(P, db.max_nb, 0);
  if constexpr (kEq) {
    build_eq(s_pl, h.nb1, s_eq);  // the representative's match table (tile.cuh)
    __syncthreads();
  }
  RunState *st = rb.st;
  const int lane = threadIdx.x & 31;
  const float s = prm.s;
  const int nb1 = h.nb1;
  const uint32_t vlast = (h.net1 & 31) ? ((1u << (h.net1 & 31)) - 1u) : 0xFFFFFFFFu;
  // 1 and 4 as values ptxas cannot fold (nb1 is read from shared memory)
  const uint32_t one_rt = 1u + (uint32_t)(h.nb1 < 0);
  const FmaK fk{one_rt, one_rt << 2};
  (void)fk;

  uint32_t row[WC], pl[kEq ? 1 : P][WC], cur[P], nxt[P];
  int state = -1, entry = 0, cand = 0;
  int i = 0, nq = 0, B = 0, js = 0, je = -1, net2 = 0, L2 = 0, cutoff = 0, lastcols = 32, frozen = 0;
  const uint32_t *qpl = nullptr;
  unsigned long long n_pairs = 0, n_members = 0, n_cells = 0, n_done = 0;

  for (;;) {
    claim(st, cls, h.qn, lane, state);
    if (__all_sync(kFullMask, state == -2)) break;
    if (state < 0) continue;
    // ---- start of a newly claimed pair -----------------------------------
    if (qpl == nullptr) {
      entry = rb.queue[cls][state];  // candidate, or pair slot in score mode
      cand = score_mode ? rb.score_cands[entry] : entry;
      L2 = __ldg(db.len + cand);
      net2 = __ldg(db.net + cand);
      nq = (net2 + 31) >> 5;
      lastcols = (net2 & 31) ? (net2 & 31) : 32;
      B = band_blocks(h.L1, L2, s);
      cutoff = cutoff_of(L2, s);
      qpl = db.words + __ldg(db.off + cand) + db.hw;
      i = 0;
      js = 0;
      je = min(B, nb1 - 1);
      frozen = 0;
      if (!score_mode) {
        n_pairs++;
        n_cells += (unsigned long long)band_cells(B, nb1, net2);
        atomicAdd(&s_qw, (unsigned long long)(nq * P));
      }
      if (B < 0 || je < 0 || nq == 0) {
        finish_pair<P>(db, rb, prm, h, score_mode, entry, cand, 0, cutoff, L2, net2, qpl, s_list, n_members);
        qpl = nullptr;
        state = -1;
        continue;
      }
#pragma unroll
      for (int m = 0; m < WC; m++) {
        row[m] = 0xFFFFFFFFu;
        if constexpr (!kEq) {
#pragma unroll
          for (int p = 0; p < P; p++) pl[p][m] = (m <= je) ? s_pl[m * P + p] : 0u;
        }
      }
#pragma unroll
      for (int p = 0; p < P; p++) cur[p] = __ldg(qpl + p);
    }
    // ---- one 32-residue query block ---------------------------------------
    const int cols = (i == nq - 1) ? lastcols : 32;
    n_done += (unsigned long long)(je - js + 1) * cols;
    if (i + 1 < nq) {
#pragma unroll
      for (int p = 0; p < P; p++) nxt[p] = __ldg(qpl + (i + 1) * P + p);
    }
    uint32_t cw_unused = 0;
    if constexpr (kEq) {
      // match words of slot m for column k: s_eq[4 (js + m) + code_k]; slots
      // past je read blocks not in the band (or the table's zero blocks):
      // those rows are reset when they enter the band
      if constexpr (NGIA_WIN_FMA) {  // the per-column bookkeeping on the FMA pipe (tile.cuh)
        uint32_t wc[2];
        eq_codes_top(cur, wc);
        eq_columns_f<WC, false, NGIA_EQ_PF_WIN>(row, smem_u32(s_eq) + 16u * (uint32_t)js, wc, cols, cw_unused,
                                                 cw_unused, fk);
      } else {
        uint32_t q[4];
        eq_codes(cur, q);
        const char *eb = reinterpret_cast<const char *>(s_eq + 4 * js);
        eq_columns<WC, false, NGIA_EQ_PF_WIN>(row, eb, q, cols, cw_unused, cw_unused);
      }
    } else {
    uint32_t rv[P];
#pragma unroll
    for (int p = 0; p < P; p++) rv[p] = __brev(cur[p]);
    int k = 0;
    for (; k + 2 <= cols; k += 2) {
      uint32_t mk[P];
#pragma unroll
      for (int p = 0; p < P; p++) {
        mk[p] = (uint32_t)((int)rv[p] >> 31);
        rv[p] <<= 1;
      }
      dp_tile<P, WC, false, false>(row, pl, mk, cw_unused, cw_unused);
#pragma unroll
      for (int p = 0; p < P; p++) {
        mk[p] = (uint32_t)((int)rv[p] >> 31);
        rv[p] <<= 1;
      }
      dp_tile<P, WC, false, false>(row, pl, mk, cw_unused, cw_unused);
    }
    if (k < cols) {
      uint32_t mk[P];
#pragma unroll
      for (int p = 0; p < P; p++) mk[p] = (uint32_t)((int)rv[p] >> 31);
      dp_tile<P, WC, false, false>(row, pl, mk, cw_unused, cw_unused);
    }
    }
    // ---- slide the band to query block i+1 --------------------------------
    i++;
    bool finished = i >= nq;
    if (!finished) {
      if (i - B > 0) {  // js advances: block js leaves the band for good
        frozen += __popc(~row[0] & (js == nb1 - 1 ? vlast : 0xFFFFFFFFu));
#pragma unroll
        for (int m = 0; m < WC - 1; m++) {
          row[m] = row[m + 1];
          if constexpr (!kEq) {
#pragma unroll
            for (int p = 0; p < P; p++) pl[p][m] = pl[p][m + 1];
          }
        }
        js++;
      }
      if (i + B <= nb1 - 1) {  // je advances: block je enters all-ones
        je++;
        const int slot = je - js;
        uint32_t v[P];
#pragma unroll
        for (int p = 0; p < P; p++) v[p] = kEq ? 0u : s_pl[je * P + p];
#pragma unroll
        for (int m = 0; m < WC; m++)
          if (m == slot) {
            row[m] = 0xFFFFFFFFu;
            if constexpr (!kEq) {
#pragma unroll
              for (int p = 0; p < P; p++) pl[p][m] = v[p];
            }
          }
      }
      if (js > je) finished = true;  // band ran past the representative
    }
    const int n = je - js + 1;
    if (finished) {
      int sum = frozen;
#pragma unroll
      for (int m = 0; m < WC; m++)
        if (m < n) sum += __popc(~row[m] & (js + m == nb1 - 1 ? vlast : 0xFFFFFFFFu));
      finish_pair<P>(db, rb, prm, h, score_mode, entry, cand, sum, cutoff, L2, net2, qpl, s_list, n_members);
      qpl = nullptr;
      state = -1;
      continue;
    }
    if (!score_mode) {
      int z = frozen;
#pragma unroll
      for (int m = 0; m < WC; m++) z += (m < n) ? __popc(~row[m]) : 0;
      if (z + (net2 - 32 * i) < cutoff) {  // cannot reach the cutoff any more
        qpl = nullptr;
        state = -1;
        continue;
      }
    }
#pragma unroll
    for (int p = 0; p < P; p++) cur[p] = nxt[p];
  }
  flush_align_stats(st, cls, n_pairs, n_members, n_cells, n_done, &s_qw);
}


// One register tile of TW window slots starting at rep block `base` for all
// `cols` residues of the current query block: rows come from and return to
// the shared-memory ring, planes from the staged representative.  The 32
// column carries enter in `cw` (column 0 at bit 31; zero for the lowest
// tile) and leave in `ncw` (ignored after the highest tile).  Slots past `je`
// are padding: computed, never stored.  Returns the change of the tile's
// zero count (all bits).
// Tiled window: windows of up to RING rep blocks (any width for RING = 0).
// Each lane keeps its pair's band rows in a ring indexed by absolute rep
// block (SmemRing / GlobalRing above) and runs each query block tile by tile in
// ascending rep-block order, all residues of the block per tile — the
// reference's (i, j, k) loop order at tile granularity.  Full tiles are MT
// slots (tiled_main); the remainder runs as one tile of exactly its width;
// the column carries pass between tiles in one word (one instruction to pop a
// carry, one to push it).  A warp's lanes start their pairs together (see the
// refill below), so their windows are equally wide and padding is rare.
//
template <int P, int RING>
__global__ void __launch_bounds__(kAlignThreads, tiled_min_blocks(P))
    k_align_tiled(DevDB db, RunBufs rb, RunParams prm, int cls, int score_mode, int warp_pairs) {
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ uint64_t bar;
  AlignHdr h;
  __shared__ unsigned long long s_qw;  // query plane words of the pairs taken (algorithmic bytes / 4)
  if (threadIdx.x == 0) s_qw = 0;
  if (!align_setup<P>(db, rb, prm, cls, score_mode, warp_pairs, 0, smem, &bar, h)) return;
  const uint32_t *s_pl = smem;
  const uint32_t *s_list = smem + ((h.nb1 * P + 3) & ~3);
  RunState *st = rb.st;
  constexpr bool kEq = P == 2 && NGIA_ALIGN_EQ;
  uint32_t *s_eq = smem + tiled_eq_off(P, db.max_nb, RING);
  if constexpr (kEq) {
    build_eq(s_pl, h.nb1, s_eq);  // the representative's match table (tile.cuh)
    __syncthreads();
  }
  const uint32_t s_eq_s = smem_u32(s_eq);
  // 1 and 4 as values ptxas cannot fold (nb1 is read from shared memory)
  const uint32_t one_rt = 1u + (uint32_t)(h.nb1 < 0);
  const FmaK fk{one_rt, one_rt << 2};
  (void)s_eq_s;
  (void)fk;
  typename RingOf<RING>::T ring;
  if constexpr (RING > 0) {
    ring.base = smem + (((db.max_nb * P + 3) & ~3) + kListWords) + threadIdx.x;
  } else {
    const int64_t TL = (int64_t)gridDim.x * blockDim.x;
    if ((int64_t)(rb.ring_mask + 1) * TL > rb.scratch_words) {
      if (threadIdx.x == 0) set_error(st, NGIA_ERR_SCRATCH, 20);
      return;
    }
    ring.base = rb.scratch + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    ring.mask = rb.ring_mask;
    ring.stride = TL;
  }
  const int lane = threadIdx.x & 31;
  const float s = prm.s;
  const int nb1 = h.nb1;
  const uint32_t vlast = (h.net1 & 31) ? ((1u << (h.net1 & 31)) - 1u) : 0xFFFFFFFFu;

  int state = -1, entry = 0, cand = 0;
  int i = 0, nq = 0, B = 0, js = 0, je = -1, net2 = 0, L2 = 0, cutoff = 0, lastcols = 32, frozen = 0, zw = 0;
  int zskip = 0;  // query blocks this lane's pair cannot be rejected at (NGIA_ZC_SKIP)
  bool active = false;
  const uint32_t *qpl = nullptr;
  uint32_t cur[P], nxt[P];
  unsigned long long n_pairs = 0, n_members = 0, n_cells = 0, n_done = 0;
  for (;;) {
    // A warp refills once prm.refill of its lanes are idle (or none is busy).
    // Queue entries next to each other are candidates of similar length, so
    // lanes that start together keep equal band windows block after block.
    {
      const unsigned idle = __ballot_sync(kFullMask, state == -1);
      const bool any_busy = __any_sync(kFullMask, state >= 0);  // every lane votes
      if (__popc(idle) >= prm.refill || !any_busy) claim(st, cls, h.qn, lane, state);
    }
    if (__all_sync(kFullMask, state == -2)) break;
    // No lane leaves the loop body early: the warp-wide reductions below are
    // executed by all 32 lanes (lanes without a pair contribute neutral values).
    bool busy = state >= 0;
    if (busy && !active) {
      entry = rb.queue[cls][state];
      cand = score_mode ? rb.score_cands[entry] : entry;
      L2 = __ldg(db.len + cand);
      net2 = __ldg(db.net + cand);
      nq = (net2 + 31) >> 5;
      lastcols = (net2 & 31) ? (net2 & 31) : 32;
      B = band_blocks(h.L1, L2, s);
      cutoff = cutoff_of(L2, s);
      qpl = db.words + __ldg(db.off + cand) + db.hw;
      i = 0;
      js = 0;
      je = min(B, nb1 - 1);
      frozen = 0;
      zw = 0;
      zskip = score_mode ? INT_MAX : 0;
      if (!score_mode) {
        n_pairs++;
        n_cells += (unsigned long long)band_cells(B, nb1, net2);
        atomicAdd(&s_qw, (unsigned long long)(nq * P));
      }
      if (B < 0 || je < 0 || nq == 0) {
        finish_pair<P>(db, rb, prm, h, score_mode, entry, cand, 0, cutoff, L2, net2, qpl, s_list, n_members);
        state = -1;
        busy = false;
      } else {
        for (int j = 0; j <= je; j++) ring[j] = 0xFFFFFFFFu;
#pragma unroll
        for (int p = 0; p < P; p++) cur[p] = __ldg(qpl + p);
        active = true;
      }
    }
    // Warp-uniform tile sequence: the full MT-slot tiles every busy lane
    // needs, then tiles sized for the largest remainder in the warp.
    // Lanes with narrower windows compute padding slots instead of taking a
    // different branch.
    const int n = busy ? je - js + 1 : 0;
    constexpr int MT = tiled_main(P);
    const int full = (int)__reduce_min_sync(kFullMask, busy ? (unsigned)(n / MT) : 0xFFFFFFFFu);
    int rem = (int)__reduce_max_sync(kFullMask, busy ? (unsigned)(n - MT * full) : 0u);
    // every busy lane's window ends exactly at the warp's last tile slot
    // (all lanes vote, before the idle ones leave the body)
    bool exact_cover = false;
    if constexpr (kEq && NGIA_EQ_FMA && NGIA_EQ_ZCARRY) exact_cover = __all_sync(kFullMask, !busy || n - MT * full == rem);
    (void)exact_cover;
    // the warp counts zeros after this block when one of its lanes may be
    // rejected there
    const bool cnt = !(kEq && NGIA_EQ_FMA && NGIA_ZC_SKIP) || __any_sync(kFullMask, busy && zskip <= 0);
    if (!busy) continue;
    const int cols = (i == nq - 1) ? lastcols : 32;
    n_done += (unsigned long long)n * cols;
    if (i + 1 < nq) {
#pragma unroll
      for (int p = 0; p < P; p++) nxt[p] = __ldg(qpl + (i + 1) * P + p);
    }
    if constexpr (kEq && NGIA_EQ_FMA) {
      using Ring = typename RingOf<RING>::T;
      constexpr bool kZC = !NGIA_EQ_ZCARRY;  // tiles count zeros
      uint32_t wc[2];
      eq_codes_top(cur, wc);
      uint32_t cw = 0, ncw = 0, last = 0;
      int base = js;
      if (kZC && NGIA_EQ_NOZOLD) zw = 0;  // the tiles return their rows' zero counts
      // a one-slot remainder joins the last main tile (warp-uniform)
      const bool merge1 = NGIA_TILED_MERGE1 && rem == 1 && full > 0;
      for (int t = merge1 ? 1 : 0; t < full; t++, base += MT) {
        zw += tiled_tile_eqf<MT, NGIA_EQ_PF_MAIN, Ring, kZC>(ring, s_eq_s, base, je, nb1, cols, wc, cw, ncw, fk, cnt);
        last = ncw;
        cw = ncw << (32 - cols);  // column 0's carry at bit 31
        ncw = 0;
      }
      if (merge1) {
        zw += tiled_tile_eqf<MT + 1, NGIA_EQ_PF_MAIN, Ring, kZC>(ring, s_eq_s, base, je, nb1, cols, wc, cw, ncw, fk, cnt);
        last = ncw;
        rem = 0;
      }
      for (; rem >= MT; rem -= MT, base += MT) {
        zw += tiled_tile_eqf<MT, NGIA_EQ_PF_MAIN, Ring, kZC>(ring, s_eq_s, base, je, nb1, cols, wc, cw, ncw, fk, cnt);
        last = ncw;
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      if (rem > 0) {
        zw += tiled_rem_eqf<Ring, MT, kZC>(rem, ring, s_eq_s, base, je, nb1, cols, wc, cw, ncw, fk, cnt);
        last = ncw;
      }
      if constexpr (!kZC) {
        if (exact_cover) {
          zw += __popc(last);  // the carries out of the window's top row over the block's columns
        } else {
          int z = 0;
          for (int j = js; j <= je; j++) z += __popc(~ring[j]);
          zw = z;
        }
      }
    } else if constexpr (kEq) {
      rem = (rem + kEqRemRound - 1) / kEqRemRound * kEqRemRound;  // extra slots are padding
      uint32_t q[4];
      eq_codes(cur, q);
      uint32_t cw = 0, ncw = 0;
      int base = js;
      for (int t = 0; t < full; t++, base += MT) {
        zw += tiled_tile_eq<MT, NGIA_EQ_PF_MAIN, typename RingOf<RING>::T>(ring, s_eq, base, je, nb1, cols, q, cw, ncw);
        cw = ncw << (32 - cols);  // column 0's carry at bit 31
        ncw = 0;
      }
      for (; rem >= MT; rem -= MT, base += MT) {
        zw += tiled_tile_eq<MT, NGIA_EQ_PF_MAIN, typename RingOf<RING>::T>(ring, s_eq, base, je, nb1, cols, q, cw, ncw);
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      if (rem > 0)
        zw += tiled_rem_eq<typename RingOf<RING>::T, MT>(rem, ring, s_eq, base, je, nb1, cols, q, cw, ncw);
    } else {
      uint32_t cw = 0, ncw = 0;
      int base = js;
      for (int t = 0; t < full; t++, base += MT) {
        zw += tiled_tile<P, MT, typename RingOf<RING>::T>(ring, s_pl, base, je, cols, cur, cw, ncw);
        cw = ncw << (32 - cols);  // column 0's carry at bit 31
        ncw = 0;
      }
      for (; rem >= MT; rem -= MT, base += MT) {
        zw += tiled_tile<P, MT, typename RingOf<RING>::T>(ring, s_pl, base, je, cols, cur, cw, ncw);
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      if (rem > 0) zw += tiled_rem<P, typename RingOf<RING>::T, MT>(rem, ring, s_pl, base, je, cols, cur, cw, ncw);
    }
    i++;
    bool finished = i >= nq;
    if (!finished) {
      if (i - B > 0) {  // block js leaves the band
        const uint32_t r0 = ring[js];
        frozen += __popc(~r0 & (js == nb1 - 1 ? vlast : 0xFFFFFFFFu));
        zw -= __popc(~r0);
        js++;
      }
      if (i + B <= nb1 - 1) {  // block je enters all-ones
        je++;
        ring[je] = 0xFFFFFFFFu;
      }
      if (js > je) finished = true;
    }
    if (finished) {
      int sum = frozen;
      for (int j = js; j <= je; j++)
        sum += __popc(~ring[j] & (j == nb1 - 1 ? vlast : 0xFFFFFFFFu));
      finish_pair<P>(db, rb, prm, h, score_mode, entry, cand, sum, cutoff, L2, net2, qpl, s_list, n_members);
      active = false;
      state = -1;
      continue;
    }
    if (cnt) {
      const int slack = score_mode ? INT_MAX : frozen + zw + (net2 - 32 * i) - cutoff;
      if (slack < 0) {
        active = false;
        state = -1;
        continue;
      }
      zskip = slack >> 5;  // the next blocks whose test cannot fail
    } else {
      zskip--;
    }
#pragma unroll
    for (int p = 0; p < P; p++) cur[p] = nxt[p];
  }
  flush_align_stats(st, cls, n_pairs, n_members, n_cells, n_done, &s_qw);
}


// ---- one warp per pair ------------------------------------------------------------
// For iterations with few queued pairs of a class, the latency of one pair
// on one thread (every residue of the query against the whole band window,
// in order) bounds the iteration.  k_align_warp gives each pair a warp.  The
// band's rows are cut into strips of 32, one row word per lane, and all 32
// lanes apply the same query residue together: the strip is one 1,024-bit
// addition row + (row & match) + carry, whose word carries are resolved with
// carry lookahead over the lanes — lane l's word sum yields a generate bit
// (it overflowed) and a propagate bit (it is all ones); with G and Pm the
// ballots of those, the carry into every lane is a bit of
// ((G | Pm) + G + carry_in) ^ (G | Pm) ^ G, and that 32-bit addition's own
// carry is the strip's carry out.  Strips of a query block run bottom-up, the
// column carries of one strip (a 32-bit mask) feeding the next; the lowest
// band row takes carry 0 and the top row's carry is dropped (the reference's
// band semantics).  Band rows live in shared memory (all nb1 rows of the
// pair, all-ones until they enter the band), loaded at a strip's start and
// stored at its end; after every query block the zero count (kept as the
// sum of the lanes' row changes) gives the exact early rejection test.
// sum = a + b over W words (word 0 lowest); returns the carry out.
template <int W>
__device__ __forceinline__ uint32_t add_words(const uint32_t (&a)[W], const uint32_t (&b)[W], uint32_t (&sum)[W]) {
  uint32_t c;
  if constexpr (W == 1) {
    asm("add.cc.u32 %0, %2, %3;\n\taddc.u32 %1, 0, 0;" : "=r"(sum[0]), "=r"(c) : "r"(a[0]), "r"(b[0]));
  } else if constexpr (W == 2) {
    asm("add.cc.u32 %0, %3, %5;\n\taddc.cc.u32 %1, %4, %6;\n\taddc.u32 %2, 0, 0;"
        : "=r"(sum[0]), "=r"(sum[1]), "=r"(c)
        : "r"(a[0]), "r"(a[1]), "r"(b[0]), "r"(b[1]));
  } else {
    static_assert(W == 4, "W is 1, 2 or 4");
    asm("add.cc.u32 %0, %5, %9;\n\taddc.cc.u32 %1, %6, %10;\n\taddc.cc.u32 %2, %7, %11;\n\t"
        "addc.cc.u32 %3, %8, %12;\n\taddc.u32 %4, 0, 0;"
        : "=r"(sum[0]), "=r"(sum[1]), "=r"(sum[2]), "=r"(sum[3]), "=r"(c)
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
  }
  return c;
}

// sum += c (0 or 1) over W words; the carry out is dropped.
template <int W>
__device__ __forceinline__ void carry_in_words(uint32_t (&sum)[W], uint32_t c) {
  if constexpr (W == 1) {
    sum[0] += c;
  } else if constexpr (W == 2) {
    asm("add.cc.u32 %0, %0, %2;\n\taddc.u32 %1, %1, 0;" : "+r"(sum[0]), "+r"(sum[1]) : "r"(c));
  } else {
    asm("add.cc.u32 %0, %0, %4;\n\taddc.cc.u32 %1, %1, 0;\n\taddc.cc.u32 %2, %2, 0;\n\taddc.u32 %3, %3, 0;"
        : "+r"(sum[0]), "+r"(sum[1]), "+r"(sum[2]), "+r"(sum[3])
        : "r"(c));
  }
}

// Banded LCS of one pair by one warp, W row words per lane; returns the
// zero count, or -1 when may_reject and the pair cannot reach the cutoff.
template <int P, int W>
__device__ __forceinline__ int warp_pair(uint32_t *rows, const uint32_t *s_pl, int nb1, uint32_t vlast,
                                         const uint32_t *qpl, int nq, int lastcols, int B, int net2, int cutoff,
                                         bool may_reject, int lane, unsigned long long &n_done) {
  for (int j = lane; j < nb1; j += 32) rows[j] = 0xFFFFFFFFu;
  __syncwarp();
  int delta = 0;
  uint32_t nxt[P];
#pragma unroll
  for (int p = 0; p < P; p++) nxt[p] = __ldg(qpl + p);
  for (int i = 0; i < nq; i++) {
    uint32_t cur[P];
#pragma unroll
    for (int p = 0; p < P; p++) {
      cur[p] = nxt[p];
      if (i + 1 < nq) nxt[p] = __ldg(qpl + (i + 1) * P + p);
    }
    const int js = max(i - B, 0), je = min(i + B, nb1 - 1);
    const int strips = je >= js ? (je - js + 32 * W) / (32 * W) : 0;
    const int cols = (i == nq - 1) ? lastcols : 32;
    if (lane == 0) n_done += (unsigned long long)(je - js + 1) * cols;
    uint32_t cmask = 0;  // carry into the strip, bit k for column k
    for (int sidx = 0; sidx < strips; sidx++) {
      // lane l holds the W consecutive rows j0 .. j0+W-1 of the strip; rows
      // above the band hold 0: they neither generate nor propagate (and no
      // row above them could take their carry)
      const int j0 = js + 32 * W * sidx + W * lane;
      uint32_t row[W], row0[W], pl[W][P], rv[P];
#pragma unroll
      for (int w = 0; w < W; w++) {
        const bool have = j0 + w <= je;
        row[w] = have ? rows[j0 + w] : 0u;
        row0[w] = row[w];
#pragma unroll
        for (int p = 0; p < P; p++) pl[w][p] = have ? s_pl[(j0 + w) * P + p] : 0u;
      }
#pragma unroll
      for (int p = 0; p < P; p++) rv[p] = __brev(cur[p]);  // residue k's bit moves to the sign bit
      uint32_t cout = 0;
      for (int k = 0; k < cols; k++) {
        uint32_t m[P], x[W], sum[W];
#pragma unroll
        for (int p = 0; p < P; p++) {
          m[p] = (uint32_t)((int)rv[p] >> 31);
          rv[p] <<= 1;
        }
#pragma unroll
        for (int w = 0; w < W; w++) {
          x[w] = row[w];
#pragma unroll
          for (int p = 0; p < P; p++) x[w] &= ~(pl[w][p] ^ m[p]);
        }
        const uint32_t gen = add_words<W>(row, x, sum);
        uint32_t ones = sum[0];
#pragma unroll
        for (int w = 1; w < W; w++) ones &= sum[w];
        const uint32_t G = __ballot_sync(kFullMask, gen);
        const uint32_t Pm = __ballot_sync(kFullMask, ones == 0xFFFFFFFFu);
        const uint32_t X = G | Pm;
        const unsigned long long tot = (unsigned long long)X + G + ((cmask >> k) & 1u);
        cout |= (uint32_t)(tot >> 32) << k;
        carry_in_words<W>(sum, (((uint32_t)tot ^ X ^ G) >> lane) & 1u);
#pragma unroll
        for (int w = 0; w < W; w++) row[w] = sum[w] | (row[w] ^ x[w]);  // stored only for rows in the band
      }
#pragma unroll
      for (int w = 0; w < W; w++) {
        const int j = j0 + w;
        if (j > je) continue;
        rows[j] = row[w];
        const uint32_t mk = (j == nb1 - 1) ? vlast : 0xFFFFFFFFu;
        delta += __popc(~row[w] & mk) - __popc(~row0[w] & mk);
      }
      cmask = cout;
    }
    __syncwarp();  // this block's rows are stored before the next block loads them
    if (may_reject && i + 1 < nq) {
      int z = delta;
#pragma unroll
      for (int o = 16; o; o >>= 1) z += __shfl_xor_sync(kFullMask, z, o);
      if (z + (net2 - 32 * (i + 1)) < cutoff) {  // cannot reach the cutoff any more
        return -1;
      }
    }
  }
  int sum = delta;
#pragma unroll
  for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(kFullMask, sum, o);
  return sum;
}

template <int P>
__global__ void __launch_bounds__(kAlignThreads)
    k_align_warp(DevDB db, RunBufs rb, RunParams prm, int cls, int score_mode, int warp_pairs) {
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ uint64_t bar;
  AlignHdr h;
  __shared__ unsigned long long s_qw;  // query plane words of the pairs taken (algorithmic bytes / 4)
  if (threadIdx.x == 0) s_qw = 0;
  if (!align_setup<P>(db, rb, prm, cls, score_mode, warp_pairs, 1, smem, &bar, h)) return;
  const uint32_t *s_pl = smem;
  const uint32_t *s_list = smem + ((h.nb1 * P + 3) & ~3);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t *rows = smem + (((db.max_nb * P + 3) & ~3) + kListWords) + warp * db.max_nb;
  RunState *st = rb.st;
  const float s = prm.s;
  const int nb1 = h.nb1;
  const uint32_t vlast = (h.net1 & 31) ? ((1u << (h.net1 & 31)) - 1u) : 0xFFFFFFFFu;
  unsigned long long n_pairs = 0, n_members = 0, n_cells = 0, n_done = 0;
  const int nwarps = gridDim.x * (blockDim.x >> 5);
  for (int e = blockIdx.x * (blockDim.x >> 5) + warp; e < h.qn; e += nwarps) {
    const int entry = score_mode ? e : rb.queue[cls][e];
    const int cand = score_mode ? rb.score_cands[entry] : entry;
    const int L2 = __ldg(db.len + cand), net2 = __ldg(db.net + cand);
    const int nq = (net2 + 31) >> 5;
    const int lastcols = (net2 & 31) ? (net2 & 31) : 32;
    const int B = band_blocks(h.L1, L2, s);
    const int cutoff = cutoff_of(L2, s);
    const uint32_t *qpl = db.words + __ldg(db.off + cand) + db.hw;
    if (!score_mode && lane == 0) {
      n_pairs++;
      n_cells += (unsigned long long)band_cells(B, nb1, net2);
      atomicAdd(&s_qw, (unsigned long long)(nq * P));
    }
    if (B < 0 || nq == 0) {
      if (lane == 0) finish_pair<P>(db, rb, prm, h, score_mode, entry, cand, 0, cutoff, L2, net2, qpl, s_list, n_members);
      continue;
    }
    // row words per lane by this pair's band window: 32 rows per strip up to
    // windows of 32 blocks, then 64, then 128
    const int A = window_of(B, nb1);
    const int sum = A <= 32   ? warp_pair<P, 1>(rows, s_pl, nb1, vlast, qpl, nq, lastcols, B, net2, cutoff, !score_mode,
                                                lane, n_done)
                    : A <= 64 ? warp_pair<P, 2>(rows, s_pl, nb1, vlast, qpl, nq, lastcols, B, net2, cutoff, !score_mode,
                                                lane, n_done)
                              : warp_pair<P, 4>(rows, s_pl, nb1, vlast, qpl, nq, lastcols, B, net2, cutoff, !score_mode,
                                                lane, n_done);
    if (sum < 0) continue;  // rejected early
    if (lane == 0) finish_pair<P>(db, rb, prm, h, score_mode, entry, cand, sum, cutoff, L2, net2, qpl, s_list, n_members);
    __syncwarp();
  }
  flush_align_stats(st, cls, n_pairs, n_members, n_cells, n_done, &s_qw);
}

// ---- dispatch ---------------------------------------------------------------------
typedef void (*AlignFn)(DevDB, RunBufs, RunParams, int, int, int);

static AlignFn warp_fn(int type, int cls) {
  (void)cls;
  return type == 0 ? k_align_warp<2> : k_align_warp<5>;
}constexpr int kWarpKernel = kNumClasses;  // index of the warp kernel in the attribute table

// DNA buckets 2 and 3 (windows of 17-32 blocks) receive pairs only when
// NGIA_DNA_WIN_CLASSES (common.cuh) keeps them; by default those windows go
// to bucket 4, the 64-slot tiled kernel.
static AlignFn align_fn(int type, int cls) {
  if (type == 0) {
    switch (cls) {
      case 0: return k_align_win<2, 8>;
      case 1: return k_align_win<2, 16>;
      case 2: return k_align_win<2, 24>;
      case 3: return k_align_win<2, 32>;
      case 4: return k_align_tiled<2, 64>;
      case 5: return k_align_tiled<2, 128>;
      default: return k_align_tiled<2, 0>;
    }
  }
  switch (cls) {
    case 0: return k_align_win<5, 8>;
    case 1: return k_align_win<5, 16>;
    case 2: return k_align_tiled<5, 64>;
    case 3: return k_align_tiled<5, 128>;
    default: return k_align_tiled<5, 0>;
  }
}

// Dynamic shared memory: rep planes | k-mer bitset | (tiled class) row ring
// | (warp kernel, cls = kWarpKernel) every row of one pair per warp.
static size_t align_smem(int type, int max_nb, int cls) {
  const int P = type ? 5 : 2;
  size_t words = (size_t)(((max_nb * P + 3) & ~3) + kListWords);
  if (cls == kWarpKernel) return 4u * (words + (size_t)(kAlignThreads / 32) * max_nb);
  const bool tiled = is_tiled_class(type, cls) || cls == generic_class(type);  // k_align_tiled
  const int ring = tiled ? class_cap(type, cls) : 0;  // 64, 128, or 0 (global ring)
  words = (size_t)tiled_eq_off(P, max_nb, ring);
  if (P == 2 && (tiled ? NGIA_ALIGN_EQ : NGIA_WIN_EQ)) words += (size_t)eq_words(max_nb);
  return 4u * words;
}

// The dynamic shared memory limit is a property of the kernel on a device, not
// of a context: it only ever grows, so that a context opened on a database of
// shorter records cannot lower it beneath the launches of an open context on
// longer ones.
cudaError_t align_configure(int type, int max_nb) {
  static std::mutex mu;
  static int configured[64][2][kNumClasses + 1] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  for (int c = 0; c <= kNumClasses; c++) {
    if (c >= num_classes(type) && c != kWarpKernel) continue;
    const int want = (int)align_smem(type, max_nb, c);
    int &have = configured[dev][type ? 1 : 0][c];
    if (want <= have) continue;
    if (c == kWarpKernel) {
      for (int k = 0; k < num_classes(type); k++) {
        e = cudaFuncSetAttribute((const void *)warp_fn(type, k), cudaFuncAttributeMaxDynamicSharedMemorySize, want);
        if (e != cudaSuccess) return e;
      }
    } else {
      e = cudaFuncSetAttribute((const void *)align_fn(type, c), cudaFuncAttributeMaxDynamicSharedMemorySize, want);
      if (e != cudaSuccess) return e;
    }
    have = want;
  }
  return cudaSuccess;
}

// Resident CTAs per SM of class `cls` (persistent grid = that x SM count).
// (cls = kNumClasses: the warp kernel.)
int align_occupancy(int type, int cls, int max_nb) {
  int nb = 0;
  const void *fn = cls == kWarpKernel ? (const void *)warp_fn(type, num_classes(type) - 1) : (const void *)align_fn(type, cls);
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, kAlignThreads, align_smem(type, max_nb, cls)) !=
      cudaSuccess)
    return 1;
  return nb < 1 ? 1 : nb;
}

int align_threads() { return kAlignThreads; }

// Launches class `cls`: the thread-per-pair kernel, and (in clustering) the
// warp-per-pair kernel; which of the two works is decided on the device from
// the class's queued pair count against c->warp_pairs.
cudaError_t launch_align(ngia_ctx *c, int cls, cudaStream_t s, int score_mode) {
  AlignFn fn = align_fn(c->db.type, cls);
  DevDB db = c->db;
  RunBufs rb = c->rb;
  RunParams prm = c->prm;
  // per length bucket (class): its own warp-per-pair cut-off and CTA count
  // when the tuner chose them
  int wp = score_mode ? -1 : (c->cls_warp_pairs[cls] >= 0 ? c->cls_warp_pairs[cls] : c->warp_pairs);
  const int grid = std::max(1, c->grid_align[cls] / std::max(1, c->cls_grid_div[cls]));
  void *args[] = {&db, &rb, &prm, &cls, &score_mode, &wp};
  cudaError_t e = cudaLaunchKernel((const void *)fn, dim3(grid), dim3(kAlignThreads), args,
                                   align_smem(c->db.type, c->db.max_nb, cls), s);
  if (e != cudaSuccess || wp <= 0) return e;  // no class can go warp-per-pair
  return cudaLaunchKernel((const void *)warp_fn(c->db.type, cls), dim3(c->grid_warp), dim3(kAlignThreads), args,
                          align_smem(c->db.type, c->db.max_nb, kWarpKernel), s);
}


}  // namespace ngia
