// assign.cuh — per-pair-representative filter and banded LCS over a set of
// representatives (a RepStore) and a query database, shared by the serving
// loop (serve.cu: resident representatives, first accepting one per query)
// and the speculative greedy rounds (spec.cu: the next K unclustered
// sequences as representatives, every accepting one per query as a bit
// mask).  The per-pair tests are the reference's (composition,
// func.cu:323-354; short words, 357-447; banded LCS, 450-604).
#pragma once
#include <stdint.h>

#include <mutex>

#include "common.cuh"
#include "kmer.cuh"
#include "tile.cuh"

namespace ngia {
namespace {

constexpr int kServeClasses = 3;    // band windows <= 64 blocks, <= 128, wider
constexpr unsigned long long kNoRep = ~0ull;

// Device view of the resident representatives.
struct RepStore {
  const uint32_t *words;
  const int64_t *off;
  const int32_t *len, *net;
  const uint32_t *cnt;
  const uint32_t *lists;  // n x list_words k-mer bitsets (empty when net < 16)
  int32_t n, list_words;
  const int32_t *count;   // when set: the representatives in use (on the device, <= n)
  const uint32_t *eq;     // DNA: match table of representative r at r * eq_stride (tile.cuh layout)
  int64_t eq_stride;      // words per table: 4 x (largest plane blocks + kEqPad)
};

// DNA match tables (tile.cuh) of the representatives, one CTA each: four
// words per plane block, zero from the representative's last block to the
// end of its table.
__global__ void k_rep_eq(RepStore rs, uint32_t *eq) {
  const int r = blockIdx.x;
  if (rs.count && r >= *rs.count) return;
  const uint32_t *rec = rs.words + rs.off[r];
  const int nb1 = ((int)rec[1] + 31) / 32;
  const uint32_t *pl = rec + 6;  // DNA header words
  uint4 *t = reinterpret_cast<uint4 *>(eq + (int64_t)r * rs.eq_stride);
  const int blocks = (int)(rs.eq_stride / 4);
  for (int j = threadIdx.x; j < blocks; j += blockDim.x) {
    const bool real = j < nb1;
    const uint32_t p0 = real ? pl[2 * j] : 0u, p1 = real ? pl[2 * j + 1] : 0u;
    uint4 e;
    e.x = real ? ~p0 & ~p1 : 0u;
    e.y = p0 & ~p1;
    e.z = ~p0 & p1;
    e.w = p0 & p1;
    t[j] = e;
  }
}

// Buffers of the assignment rounds of one slot.
struct RoundBufs {
  int2 *queue[kServeClasses];  // (representative, query) pairs of a round
  uint32_t *ctl;               // [0..2] pairs queued per class, [3..5] claimed, [6] queries left
  unsigned long long *key;     // per query: rep << 32 | score of the best accepting rep
  uint32_t *todo;              // bitmap of the queries not assigned yet
  unsigned long long *stats;   // [0] pairs aligned, [1] in-band cells computed
  int64_t cap;                 // pairs per class queue
  // mask form (speculative rounds): every accepting representative is kept
  unsigned long long *mask;    // per query: bit r = representative r accepts it
  int32_t *score;              // score of (r, q) at r * score_stride + q, for accepted pairs
  int64_t score_stride;
};

__host__ __device__ inline int serve_class(int A) { return A <= 64 ? 0 : A <= 128 ? 1 : 2; }

// k-mer presence bitset of every representative (the list of k_prep).
template <int P>
__global__ void k_rep_lists(RepStore rs, int w, uint32_t *lists) {
  __shared__ uint32_t s_list[kListWords];
  const int r = blockIdx.x;
  if (rs.count && r >= *rs.count) return;
  const int lw = rs.list_words;
  for (int i = threadIdx.x; i < lw; i += blockDim.x) s_list[i] = 0;
  __syncthreads();
  const uint32_t *rec = rs.words + rs.off[r];
  const int net1 = (int)rec[1];
  if (net1 >= 16) {
    constexpr int bits = P == 2 ? 2 : 5;
    const uint32_t mask = (1u << (w * bits)) - 1u;
    const uint32_t *planes = rec + (P == 2 ? 6 : 30);
    for (int p = w - 1 + threadIdx.x; p < net1; p += blockDim.x) {
      uint32_t word = 0;
      for (int t = p - w + 1; t <= p; t++) word = (word << bits) | code_at<P>(planes, t);
      word &= mask;
      atomicOr(&s_list[word >> 5], 1u << (word & 31));
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < lw; i += blockDim.x) lists[(int64_t)r * lw + i] = s_list[i];
}

// One CTA per representative of the chunk: composition test (and the
// short-word test in word-first order) for every unassigned query; the
// survivors are queued per class with one global atomic per class and CTA
// (two passes over the queries: decide into shared memory, then write).
template <int P>
__global__ void __launch_bounds__(256) k_serve_filter(DevDB qdb, RepStore rs, RunParams prm, RoundBufs rb, int r0,
                                                      int word_first) {
  extern __shared__ uint8_t s_res[];  // per query: 0 = out, 1 + class
  __shared__ uint32_t s_rc[28], s_cnt[kServeClasses], s_base[kServeClasses], s_pos[kServeClasses];
  constexpr int A = P == 2 ? 4 : 28;
  const int r = r0 + blockIdx.x;
  const uint32_t *rec = rs.words + rs.off[r];
  if (threadIdx.x < A) s_rc[threadIdx.x] = rec[2 + threadIdx.x];
  if (threadIdx.x < kServeClasses) s_cnt[threadIdx.x] = s_pos[threadIdx.x] = 0;
  __syncthreads();
  const int L1 = (int)rec[0], net1 = (int)rec[1], nb1 = (net1 + 31) / 32;
  const float s = prm.s;
  const bool word_here = word_first && !prm.precise && net1 >= 16;
  const uint32_t *rlist = rs.lists + (int64_t)r * rs.list_words;
  const int n = qdb.n, nbw = (n + 31) / 32;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int wi = warp; wi < nbw; wi += blockDim.x >> 5) {
    const uint32_t bits = rb.todo[wi];
    const int q = wi * 32 + lane;
    int res = 0;
    if ((bits >> lane) & 1u) {
      // a smaller representative of this round may already hold q
      const bool open = (rb.key[q] >> 32) > (unsigned long long)r;
      const int L2 = __ldg(qdb.len + q);
      bool pass = open && !(base_sum<A>(qdb.cnt, q, s_rc) < cutoff_of(L2, s));
      if (pass && word_here) {
        const int net2 = __ldg(qdb.net + q);
        if (net2 >= 16) {
          const uint32_t *planes = qdb.words + __ldg(qdb.off + q) + qdb.hw;
          pass = !(word_count<P>(planes, net2, prm.w, rlist) < word_min(L2, prm.w, s));
        }
      }
      if (pass) res = 1 + serve_class(window_of(band_blocks(L1, L2, s), nb1));
    }
    if (q < n) s_res[q] = (uint8_t)res;
    const unsigned pm = __ballot_sync(kFullMask, res != 0);
    if (res) {
      const unsigned peers = __match_any_sync(pm, res);
      if (lane == __ffs(peers) - 1) atomicAdd(&s_cnt[res - 1], (uint32_t)__popc(peers));
    }
  }
  __syncthreads();
  if (threadIdx.x < kServeClasses)
    s_base[threadIdx.x] = s_cnt[threadIdx.x] ? atomicAdd(&rb.ctl[threadIdx.x], s_cnt[threadIdx.x]) : 0u;
  __syncthreads();
  for (int wi = warp; wi < nbw; wi += blockDim.x >> 5) {
    const int q = wi * 32 + lane;
    const int res = q < n ? s_res[q] : 0;
    const unsigned pm = __ballot_sync(kFullMask, res != 0);
    if (!res) continue;
    const unsigned peers = __match_any_sync(pm, res);
    const int leader = __ffs(peers) - 1;
    uint32_t b = 0;
    if (lane == leader) b = atomicAdd(&s_pos[res - 1], (uint32_t)__popc(peers));
    b = __shfl_sync(peers, b, leader);
    const int64_t slot = (int64_t)s_base[res - 1] + b + __popc(peers & ((1u << lane) - 1u));
    if (slot < rb.cap) rb.queue[res - 1][slot] = make_int2(r, q);
  }
}

// NGIA_SERVE_STAGE 1 (DNA): each warp copies the match table of the
// representative its pairs use into its own shared-memory region and runs
// the tiles with the FMA-pipe bookkeeping of the clustering kernel
// (tile.cuh); the claimed pairs start in groups that share a representative.
// 0 (default): every lane reads its pair's table from global memory (L1).
// Measured on GB300: serving 56.5k vs 59.2k queries/s (200 batches of
// 1-4,096 DNA queries against 14,077 representatives, 16 slots), speculative
// rounds of the 20,000-sequence job 0.685 vs 0.507 s.
// The kernel is bound by the ALU pipe (80% busy, loads 50%), so the shared
// tables save little, while groups leave lanes idle (27.7 of 32 active): a
// claim holds pairs of several representatives, above all in the
// speculative rounds, whose queue interleaves the candidates.
#ifndef NGIA_SERVE_STAGE
#define NGIA_SERVE_STAGE 0
#endif
// NGIA_SERVE_FMA (DNA, without staging): the per-column bookkeeping on the FMA
// pipe with the table in global memory (as k_align_tiled does with its
// shared-memory table).  Measured on GB300: serving 64.3k against 58.9k
// queries/s (serving 200 DNA query batches, p99 642 against 782 ms), the
// speculative rounds of the 20,000-sequence job 0.489 against 0.506 s.
// NGIA_SERVE_REM_ROUND: remainder tiles rounded up to a multiple of this width
// (fewer tile bodies); 2, 4 and 8 gave 63.5k, 62.2k and 59.1k queries/s.
#ifndef NGIA_SERVE_FMA
#define NGIA_SERVE_FMA 1
#endif
#ifndef NGIA_SERVE_REM_ROUND
#define NGIA_SERVE_REM_ROUND 1
#endif

// Banded LCS of the queued (representative, query) pairs of one class: the
// loop of k_align_tiled (align.cu) with the representative taken per pair.
// MASK = false: first match (rb.key keeps the smallest accepting rep per
// query, pairs of larger reps are skipped once a smaller one accepted);
// MASK = true: every pair runs and an accepted one sets bit r of rb.mask[q]
// and its score.
// A warp claims 32 queue entries once none of its lanes holds a pair.  With
// staging (DNA), the claimed pairs start in groups: each group is the lanes
// whose pair has the representative of the first waiting lane, that
// representative's table is copied into the warp's region unless it is
// there already, and the next group starts when the current one is done.
// The filters queue the pairs of one representative next to each other (one
// CTA per representative in serving, per-candidate pushes in the
// speculative rounds), so a claim holds one or two groups.
template <int P, int RING, bool MASK>
__global__ void __launch_bounds__(kAlignThreads, tiled_min_blocks(P))
    k_serve_align(DevDB qdb, RepStore rs, RunParams prm, RoundBufs rb, int cls, int word_after, uint32_t *scratch,
                  int64_t scratch_words, uint32_t ring_mask) {
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ uint32_t s_qn;
  constexpr bool kStage = P == 2 && NGIA_SERVE_EQ && NGIA_SERVE_STAGE;
  if (threadIdx.x == 0) s_qn = (int64_t)rb.ctl[cls] < rb.cap ? rb.ctl[cls] : (uint32_t)rb.cap;
  __syncthreads();
  const uint32_t qn = s_qn;
  if (qn == 0) return;
  typename RingOf<RING>::T ring;
  if constexpr (RING > 0) {
    ring.base = smem + threadIdx.x;
  } else {
    const int64_t TL = (int64_t)gridDim.x * blockDim.x;
    if ((int64_t)(ring_mask + 1) * TL > scratch_words) return;  // the host sizes the grid to the scratch
    ring.base = scratch + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    ring.mask = ring_mask;
    ring.stride = TL;
  }
  // this warp's match-table region (after the shared ring)
  uint32_t *w_eq = smem + (RING > 0 ? RING * kAlignThreads : 0) + (int64_t)(threadIdx.x >> 5) * rs.eq_stride;
  const uint32_t w_eq_s = smem_u32(w_eq);
  (void)w_eq_s;
  // 1 and 4 as values ptxas cannot fold (the FMA-pipe bookkeeping of tile.cuh)
  const uint32_t one_rt = 1u + (uint32_t)(qn == 0u);
  const FmaK fk{one_rt, one_rt << 2};
  (void)fk;
  int staged = -1;  // representative whose table is in the warp's region (warp-uniform)
  const int lane = threadIdx.x & 31;
  const float s = prm.s;
  const int hw = qdb.hw;
  int state = -1;  // -1 idle, -2 queue exhausted, >= 0 a claimed entry (waiting or running)
  int r = 0, q = 0, i = 0, nq = 0, B = 0, js = 0, je = -1, net1 = 0, nb1 = 0, net2 = 0, L2 = 0, cutoff = 0;
  int lastcols = 32, frozen = 0, zw = 0;
  uint32_t vlast = 0;
  bool active = false;
  const uint32_t *qpl = nullptr, *rpl = nullptr;
  uint32_t cur[P], nxt[P];
  unsigned long long n_pairs = 0, n_cells = 0;
  // every loop pass advances a running lane by one query block, claims, or
  // starts a group: bounded by the queued pairs' blocks (each at most
  // kMaxBlocks) and the groups per claim, per warp
  const long long guard_max = ((long long)qn + 64) * (kMaxBlocks + 36);
  long long guard = 0;
  for (;;) {
    if (++guard > guard_max) {
      if (lane == 0) atomicExch(&rb.ctl[7], 1u);
      break;
    }
    {  // refill once prm.refill lanes are idle or none holds a pair (as in
       // k_align_tiled; with staging only when none holds a pair); the warp
       // votes run on all 32 lanes before they are combined per lane
      const bool any_held = __any_sync(kFullMask, state >= 0);
      const unsigned idle = __ballot_sync(kFullMask, state == -1);
      const bool refill_now = !any_held || (!kStage && __popc(idle) >= prm.refill);
      const bool need = state == -1 && refill_now;
      const unsigned nm = __ballot_sync(kFullMask, need);
      if (nm) {
        const int leader = __ffs(nm) - 1;
        uint32_t base = 0;
        if (lane == leader) base = atomicAdd(&rb.ctl[3 + cls], (uint32_t)__popc(nm));
        base = __shfl_sync(kFullMask, base, leader);
        if (need) {
          const uint32_t idx = base + (uint32_t)__popc(nm & ((1u << lane) - 1u));
          state = idx < qn ? (int)idx : -2;
          if (state >= 0) {
            const int2 e = rb.queue[cls][state];
            r = e.x;
            q = e.y;
          }
        }
      }
    }
    if (__all_sync(kFullMask, state == -2)) break;
    // start claimed pairs: without staging at once; with staging in groups
    // sharing a representative, the next group once no pair runs
    bool start = state >= 0 && !active;
    if constexpr (kStage) {
      start = false;
      if (!__any_sync(kFullMask, active)) {
        const unsigned pm = __ballot_sync(kFullMask, state >= 0);
        if (pm) {
          const int rg = __shfl_sync(kFullMask, r, __ffs(pm) - 1);
          if (rg != staged) {
            const uint32_t *rrec = rs.words + rs.off[rg];
            const int words = 4 * (((int)rrec[1] + 31) / 32 + kEqPad);  // table blocks + zero blocks
            const uint4 *src = reinterpret_cast<const uint4 *>(rs.eq + (int64_t)rg * rs.eq_stride);
            __syncwarp();
            for (int t = lane; t < words / 4; t += 32) reinterpret_cast<uint4 *>(w_eq)[t] = __ldg(src + t);
            __syncwarp();
            staged = rg;
          }
          start = state >= 0 && r == rg;
        }
      }
    }
    if (start) {
      const uint32_t *rrec = rs.words + rs.off[r];
      const int L1 = (int)rrec[0];
      net1 = (int)rrec[1];
      nb1 = (net1 + 31) >> 5;
      rpl = rrec + hw;
      vlast = (net1 & 31) ? ((1u << (net1 & 31)) - 1u) : 0xFFFFFFFFu;
      L2 = __ldg(qdb.len + q);
      net2 = __ldg(qdb.net + q);
      nq = (net2 + 31) >> 5;
      lastcols = (net2 & 31) ? (net2 & 31) : 32;
      B = band_blocks(L1, L2, s);
      cutoff = cutoff_of(L2, s);
      qpl = qdb.words + __ldg(qdb.off + q) + hw;
      i = 0;
      js = 0;
      je = min(B, nb1 - 1);
      frozen = 0;
      zw = 0;
      if (!MASK && (rb.key[q] >> 32) < (unsigned long long)r) {
        state = -1;  // a smaller representative already holds q
      } else if (B < 0 || je < 0 || nq == 0) {
        if (!(0 < cutoff)) {
          if (MASK) {
            rb.score[(int64_t)r * rb.score_stride + q] = 0;
            atomicOr(&rb.mask[q], 1ull << r);
          } else {
            atomicMin(&rb.key[q], (unsigned long long)r << 32);
          }
        }
        state = -1;
      } else {
        for (int j = 0; j <= je; j++) ring[j] = 0xFFFFFFFFu;
#pragma unroll
        for (int p = 0; p < P; p++) cur[p] = __ldg(qpl + p);
        active = true;
        n_pairs++;
      }
    }
    const bool busy = active;
    constexpr int MT = tiled_main(P);
    const int n = busy ? je - js + 1 : 0;
    const int full = (int)__reduce_min_sync(kFullMask, busy ? (unsigned)(n / MT) : 0xFFFFFFFFu);
    int rem = (int)__reduce_max_sync(kFullMask, busy ? (unsigned)(n - MT * full) : 0u);
    if (!busy) continue;
    const int cols = (i == nq - 1) ? lastcols : 32;
    n_cells += (unsigned long long)n * cols * 32;
    if (i + 1 < nq) {
#pragma unroll
      for (int p = 0; p < P; p++) nxt[p] = __ldg(qpl + (i + 1) * P + p);
    }
    using Ring = typename RingOf<RING>::T;
    if constexpr (kStage) {  // match words from the warp's staged table (shared memory)
      uint32_t wc[2];
      eq_codes_top(cur, wc);
      uint32_t cw = 0, ncw = 0;
      int base = js;
      if (NGIA_EQ_NOZOLD) zw = 0;  // the tiles return their rows' zero counts
      for (int t = 0; t < full; t++, base += MT) {
        zw += tiled_tile_eqf<MT, NGIA_SERVE_PF, Ring>(ring, w_eq_s, base, je, nb1, cols, wc, cw, ncw, fk);
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      for (; rem >= MT; rem -= MT, base += MT) {
        zw += tiled_tile_eqf<MT, NGIA_SERVE_PF, Ring>(ring, w_eq_s, base, je, nb1, cols, wc, cw, ncw, fk);
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      if (rem > 0) zw += tiled_rem_eqf<Ring, MT>(rem, ring, w_eq_s, base, je, nb1, cols, wc, cw, ncw, fk);
    } else if constexpr (P == 2 && NGIA_SERVE_EQ && NGIA_SERVE_FMA) {
      // match words from the pair's representative's table (global memory,
      // L1), the per-column bookkeeping on the FMA pipe as in k_align_tiled
      const uint64_t req = (uint64_t)(rs.eq + (int64_t)r * rs.eq_stride);
      uint32_t wc[2];
      eq_codes_top(cur, wc);
      uint32_t cw = 0, ncw = 0;
      int base = js;
      zw = 0;  // the tiles return their rows' zero counts
      for (int t = 0; t < full; t++, base += MT) {
        zw += tiled_tile_eqfg<MT, NGIA_SERVE_PF, Ring>(ring, req, base, je, nb1, cols, wc, cw, ncw, fk);
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      for (; rem >= MT; rem -= MT, base += MT) {
        zw += tiled_tile_eqfg<MT, NGIA_SERVE_PF, Ring>(ring, req, base, je, nb1, cols, wc, cw, ncw, fk);
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      if (rem > 0) zw += tiled_rem_eqfg<Ring, NGIA_SERVE_REM_ROUND>(rem, ring, req, base, je, nb1, cols, wc, cw, ncw, fk);
    } else if constexpr (P == 2 && NGIA_SERVE_EQ) {  // match words from the pair's representative's table
      const uint32_t *req = rs.eq + (int64_t)r * rs.eq_stride;
      uint32_t q4[4];
      eq_codes(cur, q4);
      uint32_t cw = 0, ncw = 0;
      int base = js;
      for (int t = 0; t < full; t++, base += MT) {
        zw += tiled_tile_eq<MT, NGIA_SERVE_PF, Ring>(ring, req, base, je, nb1, cols, q4, cw, ncw);
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      for (; rem >= MT; rem -= MT, base += MT) {
        zw += tiled_tile_eq<MT, NGIA_SERVE_PF, Ring>(ring, req, base, je, nb1, cols, q4, cw, ncw);
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      if (rem > 0) zw += tiled_rem_eq<Ring, MT>(rem, ring, req, base, je, nb1, cols, q4, cw, ncw);
    } else {
      uint32_t cw = 0, ncw = 0;
      int base = js;
      for (int t = 0; t < full; t++, base += MT) {
        zw += tiled_tile<P, MT, Ring>(ring, rpl, base, je, cols, cur, cw, ncw);
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      for (; rem >= MT; rem -= MT, base += MT) {
        zw += tiled_tile<P, MT, Ring>(ring, rpl, base, je, cols, cur, cw, ncw);
        cw = ncw << (32 - cols);
        ncw = 0;
      }
      if (rem > 0) zw += tiled_rem<P, Ring, MT>(rem, ring, rpl, base, je, cols, cur, cw, ncw);
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
      for (int j = js; j <= je; j++) sum += __popc(~ring[j] & (j == nb1 - 1 ? vlast : 0xFFFFFFFFu));
      bool pass = !(sum < cutoff);
      if (pass && word_after && net1 >= 16 && net2 >= 16)
        pass = !(word_count<P>(qpl, net2, prm.w, rs.lists + (int64_t)r * rs.list_words) < word_min(L2, prm.w, s));
      if (pass) {
        if (MASK) {
          rb.score[(int64_t)r * rb.score_stride + q] = sum;
          atomicOr(&rb.mask[q], 1ull << r);
        } else {
          atomicMin(&rb.key[q], ((unsigned long long)r << 32) | (uint32_t)sum);
        }
      }
      active = false;
      state = -1;
      continue;
    }
    if (frozen + zw + (net2 - 32 * i) < cutoff) {  // cannot reach the cutoff any more
      active = false;
      state = -1;
      continue;
    }
#pragma unroll
    for (int p = 0; p < P; p++) cur[p] = nxt[p];
  }
  for (int o = 16; o; o >>= 1) {
    n_pairs += __shfl_down_sync(kFullMask, n_pairs, o);
    n_cells += __shfl_down_sync(kFullMask, n_cells, o);
  }
  if (lane == 0 && n_pairs) {
    atomicAdd(&rb.stats[0], n_pairs);
    atomicAdd(&rb.stats[1], n_cells);
  }
}

using AlignServeFn = void (*)(DevDB, RepStore, RunParams, RoundBufs, int, int, uint32_t *, int64_t, uint32_t);

template <bool MASK>
AlignServeFn serve_align_fn(int type, int cls) {
  if (type == 0)
    return cls == 0 ? k_serve_align<2, 64, MASK> : cls == 1 ? k_serve_align<2, 128, MASK> : k_serve_align<2, 0, MASK>;
  return cls == 0 ? k_serve_align<5, 64, MASK> : cls == 1 ? k_serve_align<5, 128, MASK> : k_serve_align<5, 0, MASK>;
}

// Dynamic shared memory of class cls: the row ring (shared classes) and, for
// DNA with staging, one match-table region of eq_stride words per warp.
inline size_t serve_align_smem(int type, int cls, int64_t eq_stride) {
  size_t b = cls == 2 ? 0 : (size_t)(cls == 0 ? 64 : 128) * kAlignThreads * 4;
  if (type == 0 && NGIA_SERVE_EQ && NGIA_SERVE_STAGE) b += 4 * (size_t)(kAlignThreads / 32) * (size_t)eq_stride;
  return b;
}

// Raises the kernel's dynamic shared memory limit to `bytes` (never lowers
// it: launches of other open servers or contexts may need more).
template <bool MASK>
cudaError_t serve_align_configure(int type, int cls, size_t bytes) {
  static std::mutex mu;
  static size_t have[64][2][kServeClasses] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  size_t &h = have[dev][type ? 1 : 0][cls];
  if (bytes <= h) return cudaSuccess;
  e = cudaFuncSetAttribute((const void *)serve_align_fn<MASK>(type, cls), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)bytes);
  if (e == cudaSuccess) h = bytes;
  return e;
}

}  // namespace
}  // namespace ngia
