// filter.cu — loader, per-representative preparation, the composition +
// short-word filter with work-queue compaction, and the next-representative
// reduction of the greedy driver.
//
// Reference counterparts (CUDA/signalNode/src/func.cu):
//   k_loader        readData device half (104-154): header arrays per sequence
//   k_prep          updateRepresent rep copy (213-235) + generateListGen/Pro (241-302)
//   k_filter        kernel_baseFilterGen/Pro (323-354) and kernel_wordFilterGen/Pro
//                   (357-447) fused, survivors compacted on the device instead of
//                   updateJobs (305-320)
//   k_next          updateRepresent assignment/selection (190-215): the next
//                   representative is the first unclustered sequence
#include <algorithm>
#include <climits>

#include "../host/host_common.h"
#include "ctx.h"
#include "kmer.cuh"
#include "steps.cuh"

namespace ngia {

// ---- loader ---------------------------------------------------------------
__global__ void k_loader(const uint32_t *__restrict__ words, const int64_t *__restrict__ off, int64_t n_words,
                         int n, int type, int32_t *len, int32_t *net, uint32_t *cnt, int32_t *max_nb,
                         int32_t *has_short, int32_t *bad) {
  const int A = type ? 28 : 4, hw = type ? 30 : 6, P = type ? 5 : 2;
  int local_max = 0, local_short = 0, local_bad = 0;
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < n; c += gridDim.x * blockDim.x) {
    const int64_t o = off[c];
    if (o < 0 || o + hw > n_words) {
      local_bad = 1;
      len[c] = 0;
      net[c] = 0;
      continue;
    }
    const uint32_t *r = words + o;
    const uint32_t L = r[0], N = r[1];
    const int64_t need = hw + (int64_t)((L + 31) / 32) * P;
    if (L > (uint32_t)kMaxLenDev || N > L || o + need > n_words) {
      local_bad = 1;
      len[c] = 0;
      net[c] = 0;
      continue;
    }
    len[c] = (int32_t)L;
    net[c] = (int32_t)N;
    for (int a = 0; a < A; a++) cnt[(int64_t)c * A + a] = r[2 + a];
    local_max = max(local_max, (int)((N + 31) / 32));
    local_short |= (N < 16);
  }
  atomicMax(max_nb, local_max);
  if (local_short) atomicOr(has_short, 1);
  if (local_bad) atomicOr(bad, 1);
}

// Protein residue-code streams, one warp per record (lanes over its
// blocks): each 32-residue block's five plane words become five stream
// words holding the block's residue codes (plane p = bit p of a code) as
// 5-bit groups, residue 0 at the top: residue j's code fills bits 155-5j ..
// 159-5j of the block's 160-bit value, whose bits 159..128 are stream word 0.
// Read across blocks, the stream holds every w-mer of the record in 5w
// contiguous bits with its last residue lowest, as the short-word test's
// rolling word holds it (func.cu:376-396).  Records the loader rejected have
// length 0 and are skipped.
__global__ void k_codes(const uint32_t *__restrict__ words, const int64_t *__restrict__ off,
                        const int32_t *__restrict__ len, int n, int hw, uint32_t *__restrict__ codes) {
  const int lane = threadIdx.x & 31;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t c = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; c < n; c += nw) {
    const int nb = (len[c] + 31) >> 5;
    const int64_t base = off[c] + hw;
    for (int b = lane; b < nb; b += 32) {
      uint32_t pl[5], st[5] = {0u, 0u, 0u, 0u, 0u};
#pragma unroll
      for (int p = 0; p < 5; p++) pl[p] = words[base + 5 * b + p];
#pragma unroll
      for (int j = 0; j < 32; j++) {
        uint32_t cj = 0;
#pragma unroll
        for (int p = 0; p < 5; p++) cj |= ((pl[p] >> j) & 1u) << p;
        const int t = 155 - 5 * j;  // the code's lowest bit in the 160-bit value
        const int k = 4 - (t >> 5), sh = t & 31;
        st[k] |= cj << sh;
        if (sh > 27) st[k - 1] |= cj >> (32 - sh);  // the group crosses into the word above
      }
#pragma unroll
      for (int k = 0; k < 5; k++) codes[base + 5 * b + k] = st[k];
    }
  }
}

cudaError_t launch_loader(ngia_ctx *c, int32_t *d_maxnb, int32_t *d_short, int32_t *d_bad) {
  int grid = c->num_sms * 4;
  k_loader<<<grid, 256, 0, c->stream>>>(c->d_words, c->d_off, c->n_words, c->db.n, c->db.type, c->d_len,
                                        c->d_net, c->d_cnt, d_maxnb, d_short, d_bad);
  if (c->db.type != 0 && c->d_codes)
    k_codes<<<grid, 256, 0, c->stream>>>(c->d_words, c->d_off, c->d_len, c->db.n, c->db.hw, c->d_codes);
  return cudaGetLastError();
}

// ---- run initialisation (initBench, func.cu:157-183) ------------------------
__global__ void k_init_run(DevDB db, RunBufs rb, RunParams prm) {
  const int n = db.n;
  const int nw = (n + 31) / 32;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    rb.cluster[i] = -1;
    rb.ident[i] = -1;
  }
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += gridDim.x * blockDim.x) {
    const int rem = n - i * 32;
    rb.alive[i] = rem >= 32 ? 0xFFFFFFFFu : ((1u << rem) - 1u);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    RunState *st = rb.st;
    st->rep = 0;
    st->done = n == 0;
    st->err = 0;
    st->err_where = 0;
    st->iter = 0;
    st->iter_limit = LLONG_MAX;
    for (int k = 0; k < kNumClasses; k++) st->qcount[k] = st->qhead[k] = 0;
    st->long_count = 0;
    st->word_first = word_first_of(db.type, prm);
    st->word_active = 0;
    st->rep_nb = st->rep_len = st->rep_net = 0;
    st->st_candidates = st->st_base_pass = st->st_align_pairs = st->st_members = 0;
    st->st_band_cells = st->st_filter_bytes = st->st_word_checks = st->st_word_pass = 0;
    st->st_done_cells = 0;
    for (int k = 0; k < kFilterStripes * kFilterStats; k++) rb.fstats[k] = 0;
    for (int k = 0; k < kNumClasses; k++) st->st_class_pairs[k] = st->st_class_done[k] = st->st_class_qwords[k] = 0;
  }
}

cudaError_t launch_init_run(ngia_ctx *c) {
  k_init_run<<<c->num_sms * 2, 256, 0, c->stream>>>(c->db, c->rb, c->prm);
  return cudaGetLastError();
}

// ---- representative preparation ----------------------------------------------
// score_rep >= 0: pair-score mode for that representative (no run state
// change); otherwise the representative is st->rep (steps.cuh).
__global__ void k_prep(DevDB db, RunBufs rb, RunParams prm, int score_rep) { prep_body(db, rb, prm, score_rep); }

cudaError_t launch_prep(ngia_ctx *c, int score_rep) {
  k_prep<<<1, 512, 0, c->stream>>>(c->db, c->rb, c->prm, score_rep);
  return cudaGetLastError();
}

// ---- fast short-word count (filter stage) --------------------------------------
// The filter looks words up in a byte table (tab[word] = 1 if the
// representative holds the word), expanded in shared memory from the k-mer
// bitset.  Positions q < w-1 have no full word (func.cu:376-396 counts from
// position w-1): the loops below count every position with a zero-filled
// history and then subtract those first w-1 lookups, recomputed the same way.

// Spreads the 16 low bits of x onto the even bits of a 32-bit word.
__device__ __forceinline__ uint32_t spread16(uint32_t x) {
  x = (x | (x << 8)) & 0x00FF00FFu;
  x = (x | (x << 4)) & 0x0F0F0F0Fu;
  x = (x | (x << 2)) & 0x33333333u;
  x = (x | (x << 1)) & 0x55555555u;
  return x;
}

// 2-bit code stream of one 32-residue DNA block as a 64-bit value (hi:lo),
// earliest residue in the highest bits: residue j's code at bits 2(31-j)
// (plane 0) and 2(31-j)+1 (plane 1).  With the previous block's low word
// above it, the word ending at residue j is the low 2w bits of
// (prev_lo:hi:lo) >> 2(31-j): one funnel shift and one mask.
__device__ __forceinline__ void dna_stream(uint32_t p0, uint32_t p1, uint32_t &hi, uint32_t &lo) {
  const uint32_t r0 = __brev(p0), r1 = __brev(p1);
  hi = spread16(r0 >> 16) | (spread16(r1 >> 16) << 1);
  lo = spread16(r0 & 0xFFFFu) | (spread16(r1 & 0xFFFFu) << 1);
}

// Occurrences of DNA block words in the table: all 32 positions (full) or
// the first lim positions.
__device__ __forceinline__ int dna_block_full(uint32_t prev, uint32_t hi, uint32_t lo, uint32_t mask,
                                              const uint8_t *tab) {
  int sum = 0;
#pragma unroll
  for (int j = 0; j < 16; j++) sum += tab[__funnelshift_r(hi, prev, 30 - 2 * j) & mask];
#pragma unroll
  for (int j = 16; j < 32; j++) sum += tab[__funnelshift_r(lo, hi, 62 - 2 * j) & mask];
  return sum;
}

__device__ __forceinline__ uint32_t dna_word_at(uint32_t prev, uint32_t hi, uint32_t lo, int j) {
  const int sh = 62 - 2 * j;
  return sh >= 32 ? __funnelshift_r(hi, prev, sh - 32) : __funnelshift_r(lo, hi, sh);
}

__device__ __forceinline__ int dna_block_part(uint32_t prev, uint32_t hi, uint32_t lo, int lim, uint32_t mask,
                                              const uint8_t *tab) {
  int sum = 0;
  for (int j = 0; j < lim; j++) sum += tab[dna_word_at(prev, hi, lo, j) & mask];
  return sum;
}

// First w-1 positions of DNA block 0 (zero-filled history), to subtract.
__device__ __forceinline__ int dna_head(const uint32_t *planes, int net2, int w, uint32_t mask, const uint8_t *tab) {
  const int head = min(w - 1, net2);
  if (head <= 0) return 0;
  uint32_t hi, lo;
  dna_stream(__ldg(planes), __ldg(planes + 1), hi, lo);
  int sum = 0;
  for (int j = 0; j < head; j++) sum += tab[dna_word_at(0u, hi, lo, j) & mask];
  return sum;
}

// Code of residue j of a block (P planes).
template <int P>
__device__ __forceinline__ uint32_t code_of(const uint32_t (&pl)[P], int j) {
  uint32_t c = 0;
#pragma unroll
  for (int p = 0; p < P; p++) c |= ((pl[p] >> j) & 1u) << p;
  return c;
}

// Protein: rolling word over the residues of one block.
template <int P>
__device__ __forceinline__ int roll_block(const uint32_t (&pl)[P], int lim, uint32_t &word, uint32_t mask,
                                          const uint8_t *tab) {
  constexpr int bits = P == 2 ? 2 : 5;
  int sum = 0;
  if (lim == 32) {
#pragma unroll
    for (int j = 0; j < 32; j++) {
      word = ((word << bits) | code_of<P>(pl, j)) & mask;
      sum += tab[word];
    }
  } else {
    for (int j = 0; j < lim; j++) {
      word = ((word << bits) | code_of<P>(pl, j)) & mask;
      sum += tab[word];
    }
  }
  return sum;
}

template <int P>
__device__ __forceinline__ int roll_head(const uint32_t *planes, int net2, int w, uint32_t mask, const uint8_t *tab) {
  constexpr int bits = P == 2 ? 2 : 5;
  const int head = min(w - 1, net2);
  if (head <= 0) return 0;
  uint32_t pl[P];
#pragma unroll
  for (int p = 0; p < P; p++) pl[p] = __ldg(planes + p);
  uint32_t word = 0;
  int sum = 0;
  for (int j = 0; j < head; j++) {
    word = ((word << bits) | code_of<P>(pl, j)) & mask;
    sum += tab[word];
  }
  return sum;
}

// Short-word count of one candidate by one thread.
template <int P>
__device__ int word_count_fast(const uint32_t *__restrict__ planes, int net2, int w, const uint8_t *tab) {
  constexpr int bits = P == 2 ? 2 : 5;
  const uint32_t mask = (1u << (w * bits)) - 1u;
  const int nfull = net2 >> 5, rest = net2 & 31;
  int sum = 0;
  if (P == 2) {
    uint32_t prev = 0, hi, lo;
    for (int b = 0; b < nfull; b++) {
      dna_stream(__ldg(planes + 2 * b), __ldg(planes + 2 * b + 1), hi, lo);
      sum += dna_block_full(prev, hi, lo, mask, tab);
      prev = lo;
    }
    if (rest) {
      dna_stream(__ldg(planes + 2 * nfull), __ldg(planes + 2 * nfull + 1), hi, lo);
      sum += dna_block_part(prev, hi, lo, rest, mask, tab);
    }
    return sum - dna_head(planes, net2, w, mask, tab);
  } else {
    uint32_t word = 0;
    for (int b = 0; b <= nfull; b++) {
      const int lim = b < nfull ? 32 : rest;
      if (!lim) break;
      uint32_t pl[P];
#pragma unroll
      for (int p = 0; p < P; p++) pl[p] = __ldg(planes + b * P + p);
      sum += roll_block<P>(pl, lim, word, mask, tab);
    }
    return sum - roll_head<P>(planes, net2, w, mask, tab);
  }
}

// ---- protein short-word count on the residue-code stream (k_codes) -----------
// The w-mer ending at residue j of a block: the 5w bits ending 5(j+1) bits
// below the top of the block's stream words st[], the previous block's last
// word above them (prev; 0 before the first block).  One funnel shift.
__device__ __forceinline__ uint32_t codes_word(const uint32_t (&st)[5], uint32_t prev, int j) {
  const int e = 5 * (j + 1), k = (e - 1) >> 5;
  return __funnelshift_r(st[k], k ? st[k - 1] : prev, 32 * (k + 1) - e);
}

// Lookups of the first lim (<= 32) positions of one block.
__device__ __forceinline__ int codes_block(const uint32_t *__restrict__ blk, uint32_t prev, int lim, uint32_t mask,
                                           const uint8_t *tab, uint32_t &last) {
  uint32_t st[5];
#pragma unroll
  for (int k = 0; k < 5; k++) st[k] = __ldg(blk + k);
  int sum = 0;
  if (lim == 32) {
#pragma unroll
    for (int j = 0; j < 32; j++) sum += tab[codes_word(st, prev, j) & mask];
  } else {
#pragma unroll
    for (int j = 0; j < 32; j++)
      if (j < lim) sum += tab[codes_word(st, prev, j) & mask];
  }
  last = st[4];
  return sum;
}

// The first w-1 positions (zero history), counted by the loops and subtracted.
__device__ __forceinline__ int codes_head(const uint32_t *__restrict__ codes, int net2, int w, uint32_t mask,
                                          const uint8_t *tab) {
  const int head = min(w - 1, net2);
  if (head <= 0) return 0;
  uint32_t st[5];
#pragma unroll
  for (int k = 0; k < 5; k++) st[k] = __ldg(codes + k);
  int sum = 0;
#pragma unroll
  for (int j = 0; j < 7; j++)
    if (j < head) sum += tab[codes_word(st, 0u, j) & mask];
  return sum;
}

// Short-word count of one protein candidate by one thread.
__device__ int word_count_codes(const uint32_t *__restrict__ codes, int net2, int w, const uint8_t *tab) {
  const uint32_t mask = (1u << (5 * w)) - 1u;
  const int nb = (net2 + 31) >> 5;
  uint32_t prev = 0;
  int sum = 0;
  for (int b = 0; b < nb; b++) sum += codes_block(codes + 5 * b, prev, min(32, net2 - 32 * b), mask, tab, prev);
  return sum - codes_head(codes, net2, w, mask, tab);
}

// The same by the whole warp: lane l takes blocks l, l+32, ..., the previous
// block's last stream word from the lane below.  All 32 lanes call it with
// the same arguments.
__device__ int word_count_codes_warp(const uint32_t *__restrict__ codes, int net2, int w, const uint8_t *tab) {
  const uint32_t mask = (1u << (5 * w)) - 1u;
  const int lane = threadIdx.x & 31;
  const int nb = (net2 + 31) >> 5;
  int sum = 0;
  uint32_t carry = 0;  // last stream word of the block below lane 0's
  for (int b0 = 0; b0 < nb; b0 += 32) {
    const int b = b0 + lane;
    const int lim = b < nb ? min(32, net2 - 32 * b) : 0;
    const uint32_t last_mine = b < nb ? __ldg(codes + 5 * b + 4) : 0u;
    uint32_t prev = __shfl_up_sync(kFullMask, last_mine, 1);
    if (lane == 0) prev = carry;
    uint32_t last = 0;
    if (lim > 0) sum += codes_block(codes + 5 * b, prev, lim, mask, tab, last);
    carry = __shfl_sync(kFullMask, last_mine, 31);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(kFullMask, sum, o);
  return sum - codes_head(codes, net2, w, mask, tab);
}

// Short-word count of candidate c for the filter: protein from the code
// stream when the database has one, otherwise from the planes.
template <int P>
__device__ __forceinline__ int word_count_cand(const DevDB &db, int c, int net2, int w, const uint8_t *tab) {
  const int64_t o = __ldg(db.off + c) + db.hw;
  if (P == 5 && db.codes) return word_count_codes(db.codes + o, net2, w, tab);
  return word_count_fast<P>(db.words + o, net2, w, tab);
}

// Short-word count of one candidate by the whole warp: lane l takes blocks
// l, l+32, ...; each lane's history (the previous block) comes from the lane
// below by a shuffle.  All 32 lanes call it with the same arguments.
template <int P>
__device__ int word_count_warp(const uint32_t *__restrict__ planes, int net2, int w, const uint8_t *tab) {
  constexpr int bits = P == 2 ? 2 : 5;
  const uint32_t mask = (1u << (w * bits)) - 1u;
  const int lane = threadIdx.x & 31;
  const int nb = (net2 + 31) >> 5;
  int sum = 0;
  uint32_t carry[P];  // planes (DNA: the stream's low word) of the block below lane 0's
#pragma unroll
  for (int p = 0; p < P; p++) carry[p] = 0u;
  for (int b0 = 0; b0 < nb; b0 += 32) {
    const int b = b0 + lane;
    const bool have = b < nb;
    const int lim = have ? min(32, net2 - 32 * b) : 0;
    uint32_t pl[P];
#pragma unroll
    for (int p = 0; p < P; p++) pl[p] = have ? __ldg(planes + b * P + p) : 0u;
    if (P == 2) {
      uint32_t hi, lo;
      dna_stream(pl[0], pl[1], hi, lo);
      uint32_t prev = __shfl_up_sync(kFullMask, lo, 1);
      if (lane == 0) prev = carry[0];
      if (lim == 32) sum += dna_block_full(prev, hi, lo, mask, tab);
      else if (lim > 0) sum += dna_block_part(prev, hi, lo, lim, mask, tab);
      carry[0] = __shfl_sync(kFullMask, lo, 31);
    } else {
      uint32_t pv[P];
#pragma unroll
      for (int p = 0; p < P; p++) {
        pv[p] = __shfl_up_sync(kFullMask, pl[p], 1);
        if (lane == 0) pv[p] = carry[p];
      }
      // history: the last w-1 residues of the block below
      uint32_t word = 0;
      for (int j = 32 - (w - 1); j < 32; j++) word = ((word << bits) | code_of<P>(pv, j)) & mask;
      if (lim > 0) sum += roll_block<P>(pl, lim, word, mask, tab);
#pragma unroll
      for (int p = 0; p < P; p++) carry[p] = __shfl_sync(kFullMask, pl[p], 31);
    }
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(kFullMask, sum, o);
  if (P == 2) return sum - dna_head(planes, net2, w, mask, tab);
  return sum - roll_head<P>(planes, net2, w, mask, tab);
}

template <int P>
__device__ __forceinline__ int word_count_cand_warp(const DevDB &db, int c, int net2, int w, const uint8_t *tab) {
  const int64_t o = __ldg(db.off + c) + db.hw;
  if (P == 5 && db.codes) return word_count_codes_warp(db.codes + o, net2, w, tab);
  return word_count_warp<P>(db.words + o, net2, w, tab);
}

// Candidates longer than this are counted by the whole warp.
constexpr int kWarpWordLen = 2048;


// Adds the filter counters of the calling CTA (every thread calls it) to one
// of kFilterStripes counter stripes; k_next folds the stripes into the run
// state.  One warp-level and one CTA-level reduction keep the global atomics
// at five per CTA, spread over 32 cache lines.
__device__ __forceinline__ void flush_stats(const RunBufs &rb, unsigned long long cand, unsigned long long base,
                                            unsigned long long bytes, unsigned long long wchk,
                                            unsigned long long wpass) {
  __shared__ unsigned long long s_acc[5];
  if (threadIdx.x < 5) s_acc[threadIdx.x] = 0;
  __syncthreads();
  for (int o = 16; o; o >>= 1) {
    cand += __shfl_down_sync(kFullMask, cand, o);
    base += __shfl_down_sync(kFullMask, base, o);
    bytes += __shfl_down_sync(kFullMask, bytes, o);
    wchk += __shfl_down_sync(kFullMask, wchk, o);
    wpass += __shfl_down_sync(kFullMask, wpass, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (cand) atomicAdd(&s_acc[0], cand);
    if (base) atomicAdd(&s_acc[1], base);
    if (bytes) atomicAdd(&s_acc[2], bytes);
    if (wchk) atomicAdd(&s_acc[3], wchk);
    if (wpass) atomicAdd(&s_acc[4], wpass);
  }
  __syncthreads();
  if (threadIdx.x < 5 && s_acc[threadIdx.x])
    atomicAdd(&rb.fstats[(blockIdx.x % kFilterStripes) * kFilterStats + threadIdx.x], s_acc[threadIdx.x]);
}

// Fused filter over the unclustered set, one tile of kFilterTileWords
// bitmap words (8 warps x kFilterWordsPerWarp words) per CTA pass: each warp takes
// kFilterWordsPerWarp consecutive words; lanes read the header arrays of 32
// consecutive sequences (coalesced), apply the composition test and, in
// word-first order, the short-word test (shared-memory k-mer bitset).
// Survivors are compacted into the alignment class queues in two levels:
// warp-aggregated shared-memory counters give each survivor its slot inside
// the tile, then one global atomic per class and tile reserves the tile's
// range, so the global queue counters see ~1/1,000 of the candidates.
// `exact` = 1 runs the composition stage only and records the survivors
// (bitmap in rb.flags) for the exact short-word path.
// Bitmap words per warp and tile pass.  Swept on GB300 (1M DNA s=0.85 and
// 200k protein s=0.9): the composition test alone is fastest with 8 (fewer,
// fuller CTAs: 20.7 us vs 23.1 us with 4), the short-word test in the filter
// with 1 (protein 0.21 ms vs 0.24 / 0.37 / 0.61 ms with 2 / 4 / 8: more
// tiles share the long candidates; DNA s=0.95 is the same for 1 to 4).
#ifndef NGIA_FILTER_WPW_BASE
#define NGIA_FILTER_WPW_BASE 8
#endif
#ifndef NGIA_FILTER_WPW_WORD
#define NGIA_FILTER_WPW_WORD 1
#endif
// (Issuing every header load of a warp's 8 bitmap words before the first
// use, unpredicated per lane, made the composition-only launch slower on
// GB300: 24.6 vs 18.1 us per iteration, 1M DNA s=0.85.)
// NGIA_FILTER_WARP_WORD: with the short-word test in the filter, warps take
// bitmap words independently (no tile barriers); 0 keeps the tiled loop.
#ifndef NGIA_FILTER_WARP_WORD
#define NGIA_FILTER_WARP_WORD 1
#endif

// NGIA_FILTER_SPLIT: launches that cannot run the short-word test in the
// filter (alignment-first order, the exact short-word path) use an instance
// compiled without it (kWord = false): each CTA runs its code once, so the
// kernel's size is paid in instruction fetches.
#ifndef NGIA_FILTER_SPLIT
#define NGIA_FILTER_SPLIT 1
#endif
// NGIA_FILTER_HOIST: in the composition-only DNA instance, load every header
// of the warp's words before the first test (predicated on the unclustered
// bit).  Off: on GB300 it ran at 24.2 against 17.8 us per iteration (80
// registers with spills against 57).
#ifndef NGIA_FILTER_HOIST
#define NGIA_FILTER_HOIST 0
#endif
template <int P, int kFilterWordsPerWarp, bool kWord = true>
__global__ void __launch_bounds__(256) k_filter(DevDB db, RunBufs rb, RunParams prm, int exact) {
  constexpr int kFilterTileWords = 8 * kFilterWordsPerWarp;  // 256 threads
  RunState *st = rb.st;
  extern __shared__ __align__(16) uint32_t s_list[];
  __shared__ uint64_t bar;
  __shared__ uint32_t s_rc[28];
  __shared__ int s_hdr[4];
  __shared__ uint32_t s_cnt[kNumClasses], s_base[kNumClasses];
  constexpr int A = P == 2 ? 4 : 28;
  if (threadIdx.x == 0) {
    const bool skip = st->done || st->iter >= st->iter_limit || st->err;
    s_hdr[0] = skip;
    s_hdr[1] = st->rep_len;
    s_hdr[2] = st->rep_nb;
    s_hdr[3] = (!exact && st->word_first && st->word_active) ? 1 : 0;
  }
  if (threadIdx.x < A) s_rc[threadIdx.x] = rb.rep_rec[2 + threadIdx.x];
  __syncthreads();
  if (s_hdr[0]) return;
  const int L1 = s_hdr[1], nb1 = s_hdr[2], word_here = kWord ? s_hdr[3] : 0;
  const int list_words = max(1, (int)((1u << (prm.w * (P == 2 ? 2 : 5))) / 32u));
  // byte table of the k-mer bitset, right after the bitset
  uint8_t *s_tab = reinterpret_cast<uint8_t *>(s_list + list_words);
  if (word_here) {
    if (!stage_to_smem(s_list, rb.rep_list, (uint32_t)list_words, &bar, st, 1)) return;
    for (int i = threadIdx.x; i < list_words * 8; i += blockDim.x) {
      const uint32_t nib = (s_list[i >> 3] >> (4 * (i & 7))) & 0xFu;  // 4 words -> 4 bytes
      reinterpret_cast<uint32_t *>(s_tab)[i] = (nib & 1u) | ((nib & 2u) << 7) | ((nib & 4u) << 14) | ((nib & 8u) << 21);
    }
    __syncthreads();
  }
  const float s = prm.s;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nbw = (db.n + 31) / 32;
  const int tiles = (nbw + kFilterTileWords - 1) / kFilterTileWords;
  // Bitmap word of slot k of a tile.  With the short-word test here, a
  // tile's words are spread over the (length-sorted) database so that every
  // tile holds a share of the long candidates; otherwise they are
  // consecutive, which keeps neighbouring queue entries of similar length.
  auto word_of = [&](int tile, int k) {
    return word_here ? k * tiles + tile : tile * kFilterTileWords + k;
  };
  unsigned long long cand = 0, base = 0, bytes = 0, wchk = 0, wpass = 0;
  if (word_here && NGIA_FILTER_WARP_WORD) {
    // Short-word test here: the work per candidate grows with its length, so
    // warps run independently — each takes every W-th bitmap word of the
    // length-sorted database (a share of every length) and queues its
    // survivors with one atomic per class and word; no CTA barrier makes a
    // warp wait for the CTA's longest candidates.
    const int W = gridDim.x * (blockDim.x >> 5);
    for (int wi = blockIdx.x * (blockDim.x >> 5) + warp; wi < nbw; wi += W) {
      const uint32_t bits = rb.alive[wi];
      if (!bits) continue;  // warp-uniform
      const int c = wi * 32 + lane;
      const bool alive = (bits >> lane) & 1u;
      bool pass = false, deferred = false;
      int cls = 0;
      if (alive) {
        cand++;
        bytes += 4 * (2 + A);
        const int L2 = __ldg(db.len + c);
        pass = !(base_sum<A>(db.cnt, c, s_rc) < cutoff_of(L2, s));
        if (pass) {
          base++;
          const int net2 = __ldg(db.net + c);
          wchk++;
          bytes += 4ull * P * ((net2 + 31) / 32);
          if (net2 <= kWarpWordLen) {
            pass = !(word_count_cand<P>(db, c, net2, prm.w, s_tab) < word_min(L2, prm.w, s));
            if (pass) wpass++;
          } else {
            deferred = true;
          }
        }
        if (pass) cls = class_of(db.type, window_of(band_blocks(L1, L2, s), nb1));
      }
      // long candidates go to k_filter_long, which gives each one a warp
      const unsigned dm = __ballot_sync(kFullMask, deferred);
      if (dm) {
        const int leader = __ffs(dm) - 1;
        uint32_t b = 0;
        if (lane == leader) b = atomicAdd(&st->long_count, (uint32_t)__popc(dm));
        b = __shfl_sync(kFullMask, b, leader);
        if (deferred) rb.long_list[b + __popc(dm & ((1u << lane) - 1u))] = c;
      }
      push_queue(rb, st, pass && !deferred, cls, c);
    }
    flush_stats(rb, cand, base, bytes, wchk, wpass);
    return;
  }
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    if (threadIdx.x < kNumClasses) s_cnt[threadIdx.x] = 0;
    __syncthreads();
    // The warp's bitmap words first, then every header load of all its
    // words (independent of one another), then the compaction.
    int slot[kFilterWordsPerWarp], cls_of[kFilterWordsPerWarp];
    uint32_t bits_of[kFilterWordsPerWarp];
#pragma unroll
    for (int k = 0; k < kFilterWordsPerWarp; k++) {
      const int wi = word_of(tile, warp * kFilterWordsPerWarp + k);
      bits_of[k] = wi < nbw ? rb.alive[wi] : 0u;
    }
    // Composition-only DNA instance: the headers of all the warp's words are
    // loaded before any test (predicated on the unclustered bit), so a warp
    // waits for one round of loads rather than one per word.
    constexpr bool kHoist = NGIA_FILTER_HOIST && !kWord && P == 2;
    constexpr int kH = kHoist ? kFilterWordsPerWarp : 1;
    int len_h[kH];
    uint4 cnt_h[kH];
    if constexpr (kHoist) {
#pragma unroll
      for (int k = 0; k < kFilterWordsPerWarp; k++) {
        const int c = word_of(tile, warp * kFilterWordsPerWarp + k) * 32 + lane;
        len_h[k] = 0;
        cnt_h[k] = make_uint4(0u, 0u, 0u, 0u);
        if ((bits_of[k] >> lane) & 1u) {
          len_h[k] = __ldg(db.len + c);
          cnt_h[k] = __ldg(reinterpret_cast<const uint4 *>(db.cnt) + c);
        }
      }
    }
    unsigned pass_of = 0;  // bit k: this lane's candidate of word k survives
#pragma unroll
    for (int k = 0; k < kFilterWordsPerWarp; k++) {
      cls_of[k] = 0;
      const uint32_t bits = bits_of[k];
      if (!bits) continue;  // warp-uniform
      const int wi = word_of(tile, warp * kFilterWordsPerWarp + k);
      const int c = wi * 32 + lane;
      const bool alive = (bits >> lane) & 1u;
      bool pass = false, deferred = false;
      if (alive) {
        cand++;
        bytes += 4 * (2 + A);
        int L2, sum;
        if constexpr (kHoist) {
          L2 = len_h[k];
          const uint4 q = cnt_h[k];
          sum = (int)(min(q.x, s_rc[0]) + min(q.y, s_rc[1]) + min(q.z, s_rc[2]) + min(q.w, s_rc[3]));
        } else {
          L2 = __ldg(db.len + c);
          sum = base_sum<A>(db.cnt, c, s_rc);
        }
        pass = !(sum < cutoff_of(L2, s));
        if (pass) base++;
        if (pass && word_here) {
          const int net2 = __ldg(db.net + c);
          wchk++;
          bytes += 4ull * P * ((net2 + 31) / 32);
          if (net2 <= kWarpWordLen) {
            pass = !(word_count_cand<P>(db, c, net2, prm.w, s_tab) < word_min(L2, prm.w, s));
            if (pass) wpass++;
          } else {
            deferred = true;
          }
        }
        if (pass && !exact) cls_of[k] = class_of(db.type, window_of(band_blocks(L1, L2, s), nb1));
      }
      // long candidates: the whole warp counts each one
      for (unsigned dm = __ballot_sync(kFullMask, deferred); dm; dm &= dm - 1) {
        const int src = __ffs(dm) - 1;
        const int cc = wi * 32 + src;
        const int ws = word_count_cand_warp<P>(db, cc, __ldg(db.net + cc), prm.w, s_tab);
        if (lane == src) {
          const int L2 = __ldg(db.len + cc);
          pass = !(ws < word_min(L2, prm.w, s));
          if (pass) {
            wpass++;
            if (!exact) cls_of[k] = class_of(db.type, window_of(band_blocks(L1, L2, s), nb1));
          }
        }
      }
      if (pass) pass_of |= 1u << k;
    }
#pragma unroll
    for (int k = 0; k < kFilterWordsPerWarp; k++) {
      slot[k] = -1;
      const int wi = word_of(tile, warp * kFilterWordsPerWarp + k);
      if (wi >= nbw) continue;  // warp-uniform
      const bool pass = (pass_of >> k) & 1u;
      const unsigned pm = __ballot_sync(kFullMask, pass);
      if (exact) {
        if (lane == 0) reinterpret_cast<uint32_t *>(rb.flags)[wi] = pm;
        continue;
      }
      if (pass) {
        const int cls = cls_of[k];
        const unsigned peers = __match_any_sync(pm, cls);
        const int leader = __ffs(peers) - 1;
        uint32_t b = 0;
        if (lane == leader) b = atomicAdd(&s_cnt[cls], (uint32_t)__popc(peers));
        b = __shfl_sync(peers, b, leader);
        slot[k] = (int)(b + __popc(peers & ((1u << lane) - 1u)));
      }
    }
    __syncthreads();
    if (threadIdx.x < kNumClasses)
      s_base[threadIdx.x] = s_cnt[threadIdx.x] ? atomicAdd(&st->qcount[threadIdx.x], s_cnt[threadIdx.x]) : 0u;
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kFilterWordsPerWarp; k++) {
      if (slot[k] >= 0) {
        const int c = word_of(tile, warp * kFilterWordsPerWarp + k) * 32 + lane;
        rb.queue[cls_of[k]][s_base[cls_of[k]] + (uint32_t)slot[k]] = c;
      }
    }
  }
  flush_stats(rb, cand, base, bytes, wchk, wpass);
}

// ---- exact short-word path ---------------------------------------------------
// For databases holding records with net length < 16 the reference's word
// kernel returns a whole thread at such a job (func.cu:375, 420), so whether
// a job is tested depends on its position p in the compacted job list and on
// the 16,384-thread map p -> p mod 16384.  These kernels reproduce that: the
// base-survivor bitmap (rb.flags as uint32 words) is prefix-counted to give p,
// first_short[t] is the first position of thread t holding a short query,
// and a job at p >= first_short[p mod 16384] passes untested.
__global__ void k_scan_words(const uint32_t *bm, int nbw, uint32_t *prefix) {
  // single CTA of 1024 threads: exclusive prefix of popcounts
  __shared__ uint32_t s_part[1024];
  const int per = (nbw + 1023) / 1024;
  const int b = threadIdx.x * per, e = min(nbw, b + per);
  uint32_t acc = 0;
  for (int i = b; i < e; i++) acc += __popc(bm[i]);
  s_part[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {
    uint32_t v = threadIdx.x >= o ? s_part[threadIdx.x - o] : 0;
    __syncthreads();
    s_part[threadIdx.x] += v;
    __syncthreads();
  }
  uint32_t run = threadIdx.x ? s_part[threadIdx.x - 1] : 0;
  for (int i = b; i < e; i++) {
    prefix[i] = run;
    run += __popc(bm[i]);
  }
}

__global__ void k_first_short(DevDB db, RunBufs rb, int reset) {
  const int nbw = (db.n + 31) / 32;
  const uint32_t *bm = reinterpret_cast<const uint32_t *>(rb.flags);
  if (reset) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < kRefGridThreads; t += gridDim.x * blockDim.x)
      rb.first_short[t] = INT_MAX;
    return;
  }
  for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nbw * 32; c += gridDim.x * blockDim.x) {
    if (c >= db.n) break;
    const uint32_t w = bm[c >> 5];
    if (!((w >> (c & 31)) & 1u)) continue;
    if (db.net[c] >= 16) continue;
    const int p = (int)(rb.scan_part[c >> 5] + __popc(w & ((1u << (c & 31)) - 1u)));
    atomicMin(&rb.first_short[p % kRefGridThreads], p);
  }
}

template <int P>
__global__ void __launch_bounds__(256) k_word_exact(DevDB db, RunBufs rb, RunParams prm) {
  RunState *st = rb.st;
  extern __shared__ __align__(16) uint32_t s_list[];
  __shared__ uint64_t bar;
  __shared__ int s_hdr[3];
  if (threadIdx.x == 0) {
    s_hdr[0] = st->done || st->iter >= st->iter_limit || st->err;
    s_hdr[1] = st->rep_len;
    s_hdr[2] = st->rep_nb;
  }
  __syncthreads();
  if (s_hdr[0]) return;
  const int L1 = s_hdr[1], nb1 = s_hdr[2];
  const int list_words = max(1, (int)((1u << (prm.w * (P == 2 ? 2 : 5))) / 32u));
  if (!stage_to_smem(s_list, rb.rep_list, (uint32_t)list_words, &bar, st, 2)) return;
  const uint32_t *bm = reinterpret_cast<const uint32_t *>(rb.flags);
  const int lane = threadIdx.x & 31;
  const int nbw = (db.n + 31) / 32;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long bytes = 0, wchk = 0, wpass = 0;
  for (int wi = gw; wi < nbw; wi += nwarps) {
    const uint32_t w = bm[wi];
    if (!w) continue;
    const int c = wi * 32 + lane;
    bool pass = (w >> lane) & 1u;
    int cls = 0;
    if (pass) {
      const int p = (int)(rb.scan_part[wi] + __popc(w & ((1u << lane) - 1u)));
      const bool skipped = p >= rb.first_short[p % kRefGridThreads];
      const int L2 = db.len[c];
      if (!skipped) {
        const int net2 = db.net[c];
        const uint32_t *planes = db.words + db.off[c] + db.hw;
        wchk++;
        bytes += 4ull * P * ((net2 + 31) / 32);
        pass = !(word_count<P>(planes, net2, prm.w, s_list) < word_min(L2, prm.w, prm.s));
      }
      if (pass) {
        wpass++;
        cls = class_of(db.type, window_of(band_blocks(L1, L2, prm.s), nb1));
      }
    }
    push_queue(rb, st, pass, cls, c);
  }
  flush_stats(rb, 0, 0, bytes, wchk, wpass);
}

// Largest filter shared memory: DNA w=8 bitset (8 KB) + byte table (64 KB).
// Short-word test of the candidates longer than kWarpWordLen residues that
// k_filter queued in rb.long_list (word-first order): one warp per
// candidate, spread over the grid, so that the longest sequences of the
// length-sorted database (which share the first bitmap words) are counted
// side by side; survivors join the alignment class queues.
template <int P>
__global__ void __launch_bounds__(256) k_filter_long(DevDB db, RunBufs rb, RunParams prm) {
  RunState *st = rb.st;
  extern __shared__ __align__(16) uint32_t s_list[];
  __shared__ uint64_t bar;
  __shared__ int s_hdr[4];
  if (threadIdx.x == 0) {
    const bool skip = st->done || st->iter >= st->iter_limit || st->err;
    s_hdr[0] = skip ? 0 : (int)st->long_count;
    s_hdr[1] = st->rep_len;
    s_hdr[2] = st->rep_nb;
  }
  __syncthreads();
  const int nlong = s_hdr[0];
  if (nlong == 0) return;
  const int L1 = s_hdr[1], nb1 = s_hdr[2];
  const int list_words = max(1, (int)((1u << (prm.w * (P == 2 ? 2 : 5))) / 32u));
  uint8_t *s_tab = reinterpret_cast<uint8_t *>(s_list + list_words);
  if (!stage_to_smem(s_list, rb.rep_list, (uint32_t)list_words, &bar, st, 2)) return;
  for (int i = threadIdx.x; i < list_words * 8; i += blockDim.x) {
    const uint32_t nib = (s_list[i >> 3] >> (4 * (i & 7))) & 0xFu;
    reinterpret_cast<uint32_t *>(s_tab)[i] = (nib & 1u) | ((nib & 2u) << 7) | ((nib & 4u) << 14) | ((nib & 8u) << 21);
  }
  __syncthreads();
  const float s = prm.s;
  const int lane = threadIdx.x & 31;
  const int W = gridDim.x * (blockDim.x >> 5);
  unsigned long long wpass = 0;
  for (int k = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); k < nlong; k += W) {
    const int c = rb.long_list[k];
    const int ws = word_count_cand_warp<P>(db, c, __ldg(db.net + c), prm.w, s_tab);
    const int L2 = __ldg(db.len + c);
    const bool pass = lane == 0 && !(ws < word_min(L2, prm.w, s));
    if (pass) wpass++;
    push_queue(rb, st, pass, pass ? class_of(db.type, window_of(band_blocks(L1, L2, s), nb1)) : 0, c);
  }
  flush_stats(rb, 0, 0, 0, 0, wpass);
}

cudaError_t filter_configure() {
  const int most = 9 * (1 << 16) / 8;
  const void *fns[] = {(const void *)k_filter<2, NGIA_FILTER_WPW_WORD>, (const void *)k_filter<5, NGIA_FILTER_WPW_WORD>,
                       (const void *)k_filter_long<2>, (const void *)k_filter_long<5>};
  for (const void *f : fns) {
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, most);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_filter(ngia_ctx *c) {
  const int P = c->db.P;
  const int bits = c->db.type ? 5 : 2;
  const int list_words = std::max(1, (int)((1u << (c->prm.w * bits)) / 32u));
  const size_t smem = (size_t)list_words * 4;
  // Exact path only matters when the short-word filter can run and some
  // record is shorter than 16 residues.
  const bool exact = c->db.has_short && !c->prm.precise;
  const int nbw = (c->db.n + 31) / 32;
  constexpr int kB = NGIA_FILTER_WPW_BASE, kW = NGIA_FILTER_WPW_WORD;
  const int grid_b = std::max(1, std::min(c->grid_filter, (nbw + 8 * kB - 1) / (8 * kB)));
  const int grid_w = std::max(1, std::min(c->grid_filter, (nbw + 8 * kW - 1) / (8 * kW)));
  if (!exact) {
    // word-first order also holds the byte table (8 bytes per bitset byte)
    if (word_first_of(c->db.type, c->prm)) {
      if (P == 2)
        k_filter<2, kW><<<grid_w, 256, smem * 9, c->stream>>>(c->db, c->rb, c->prm, 0);
      else
        k_filter<5, kW><<<grid_w, 256, smem * 9, c->stream>>>(c->db, c->rb, c->prm, 0);
      if (NGIA_FILTER_WARP_WORD && c->db.max_nb * 32 > kWarpWordLen) {  // some record is long
        const int grid_l = std::max(1, std::min(c->grid_filter, c->num_sms));
        if (P == 2)
          k_filter_long<2><<<grid_l, 256, smem * 9, c->stream>>>(c->db, c->rb, c->prm);
        else
          k_filter_long<5><<<grid_l, 256, smem * 9, c->stream>>>(c->db, c->rb, c->prm);
      }
    } else if (c->filter_tile == kW) {  // the tuner's choice: one bitmap word per warp and tile
      if (P == 2)
        k_filter<2, kW, !NGIA_FILTER_SPLIT><<<grid_w, 256, smem, c->stream>>>(c->db, c->rb, c->prm, 0);
      else
        k_filter<5, kW, !NGIA_FILTER_SPLIT><<<grid_w, 256, smem, c->stream>>>(c->db, c->rb, c->prm, 0);
    } else {
      if (P == 2)
        k_filter<2, kB, !NGIA_FILTER_SPLIT><<<grid_b, 256, smem, c->stream>>>(c->db, c->rb, c->prm, 0);
      else
        k_filter<5, kB, !NGIA_FILTER_SPLIT><<<grid_b, 256, smem, c->stream>>>(c->db, c->rb, c->prm, 0);
    }
    return cudaGetLastError();
  }
  if (P == 2)
    k_filter<2, kB, !NGIA_FILTER_SPLIT><<<grid_b, 256, smem, c->stream>>>(c->db, c->rb, c->prm, 1);
  else
    k_filter<5, kB, !NGIA_FILTER_SPLIT><<<grid_b, 256, smem, c->stream>>>(c->db, c->rb, c->prm, 1);
  k_scan_words<<<1, 1024, 0, c->stream>>>(reinterpret_cast<const uint32_t *>(c->rb.flags), nbw, c->rb.scan_part);
  k_first_short<<<64, 256, 0, c->stream>>>(c->db, c->rb, 1);
  k_first_short<<<c->num_sms * 2, 256, 0, c->stream>>>(c->db, c->rb, 0);
  if (P == 2)
    k_word_exact<2><<<c->grid_filter, 256, smem, c->stream>>>(c->db, c->rb, c->prm);
  else
    k_word_exact<5><<<c->grid_filter, 256, smem, c->stream>>>(c->db, c->rb, c->prm);
  return cudaGetLastError();
}

// ---- next representative (steps.cuh) ----------------------------------------
__global__ void k_next(DevDB db, RunBufs rb, unsigned long long cond, int use_cond) {
  next_body(db, rb, cond, use_cond);
}


// Start of a run over a subset of the sequences (the unclustered set was
// loaded into rb.alive): the first member of the subset is the first
// representative; an empty subset is done at once.
__global__ void k_subset_start(DevDB db, RunBufs rb) {
  RunState *st = rb.st;
  __shared__ int s_min[32];
  const int nbw = (db.n + 31) / 32;
  int v = INT_MAX;
  for (int wi = threadIdx.x; wi < nbw; wi += blockDim.x)
    if (rb.alive[wi]) {
      v = wi;
      break;
    }
  for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(kFullMask, v, o));
  if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x < 32) {
    int u = threadIdx.x < (int)(blockDim.x >> 5) ? s_min[threadIdx.x] : INT_MAX;
    for (int o = 16; o; o >>= 1) u = min(u, __shfl_xor_sync(kFullMask, u, o));
    if (threadIdx.x == 0) {
      if (u == INT_MAX) {
        st->done = 1;
      } else {
        st->rep = u * 32 + __ffs(rb.alive[u]) - 1;
        st->done = 0;
      }
    }
  }
}

cudaError_t launch_subset_start(ngia_ctx *c, const uint32_t *d_alive) {
  const int nbw = (c->db.n + 31) / 32;
  cudaError_t e = cudaMemcpyAsync(c->rb.alive, d_alive, sizeof(uint32_t) * (size_t)nbw, cudaMemcpyDeviceToDevice,
                                  c->stream);
  if (e != cudaSuccess) return e;
  k_subset_start<<<1, 1024, 0, c->stream>>>(c->db, c->rb);
  return cudaGetLastError();
}

cudaError_t launch_next(ngia_ctx *c, unsigned long long cond, int use_cond) {
  k_next<<<1, 1024, 0, c->stream>>>(c->db, c->rb, cond, use_cond);
  return cudaGetLastError();
}

// ---- pair-score mode: per-pair composition / word values and queueing ----------
template <int P>
__global__ void k_score_classify(DevDB db, RunBufs rb, RunParams prm, int n) {
  RunState *st = rb.st;
  constexpr int A = P == 2 ? 4 : 28;
  __shared__ uint32_t s_rc[28];
  if (threadIdx.x < A) s_rc[threadIdx.x] = rb.rep_rec[2 + threadIdx.x];
  __syncthreads();
  const int L1 = st->rep_len, nb1 = st->rep_nb, net1 = st->rep_net;
  const int iters = (n + blockDim.x * gridDim.x - 1) / (blockDim.x * gridDim.x);
  for (int it = 0; it < iters; it++) {
    const int k = it * blockDim.x * gridDim.x + blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = k < n;
    int cls = 0;
    if (valid) {
      const int c = rb.score_cands[k];
      const int L2 = db.len[c], net2 = db.net[c];
      rb.score_out[4 * k + 0] = base_sum<A>(db.cnt, c, s_rc);
      if (net1 < 16 || net2 < 16)
        rb.score_out[4 * k + 1] = -1;
      else
        rb.score_out[4 * k + 1] = word_count<P>(db.words + db.off[c] + db.hw, net2, prm.w, rb.rep_list);
      const int B = band_blocks(L1, L2, prm.s);
      rb.score_out[4 * k + 3] = B;
      cls = class_of(db.type, window_of(B, nb1));
    }
    push_queue(rb, st, valid, cls, k);
  }
}

cudaError_t launch_score_classify(ngia_ctx *c, int n) {
  const int grid = std::max(1, std::min(c->num_sms * 4, (n + 255) / 256));
  if (c->db.P == 2)
    k_score_classify<2><<<grid, 256, 0, c->stream>>>(c->db, c->rb, c->prm, n);
  else
    k_score_classify<5><<<grid, 256, 0, c->stream>>>(c->db, c->rb, c->prm, n);
  return cudaGetLastError();
}

}  // namespace ngia

namespace ngia {
// ---- the floor under the composition filter's time ---------------------------
// Two kernels with the composition filter's grid and tiles: one that does
// nothing, and one that only reads what the filter reads (each warp's bitmap
// words, then the length and counts of every unclustered sequence of them),
// folding the values so the loads are kept.  Their times on the context's
// stream bound the filter's: launch and one round of dependent loads.
namespace {

__global__ void k_floor_empty(const RunBufs rb) {
  if (threadIdx.x == 0 && blockIdx.x == 0 && rb.st == nullptr) rb.fstats[0] = 1;
}

__global__ void __launch_bounds__(256) k_floor_read(DevDB db, RunBufs rb, unsigned long long *sink) {
  constexpr int kW = NGIA_FILTER_WPW_BASE, kTileWords = 8 * kW;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nbw = (db.n + 31) / 32;
  const int tiles = (nbw + kTileWords - 1) / kTileWords;
  uint32_t acc = 0;
  for (int tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
    uint32_t bits_of[kW];
#pragma unroll
    for (int k = 0; k < kW; k++) {
      const int wi = tile * kTileWords + warp * kW + k;
      bits_of[k] = wi < nbw ? rb.alive[wi] : 0u;
    }
#pragma unroll
    for (int k = 0; k < kW; k++) {
      const int c = (tile * kTileWords + warp * kW + k) * 32 + lane;
      if ((bits_of[k] >> lane) & 1u) {
        const uint4 q = __ldg(reinterpret_cast<const uint4 *>(db.cnt) + c);
        acc += (uint32_t)__ldg(db.len + c) + q.x + q.y + q.z + q.w;
      }
    }
  }
  // A thread sums at most 8 x 5 values below 2^16 (< 2^22), so this never
  // holds; the compiler cannot know that and keeps the loads.
  if (acc == 0xFFFFFFFFu) atomicAdd(sink, 1ull);
}

}  // namespace
}  // namespace ngia

extern "C" int ngia_measure_filter_floor(ngia_ctx *c, double *launch_us, double *read_us) {
  ngia::clear_error();
  if (!c || !launch_us || !read_us) return ngia::fail(NGIA_E_ARG, "ngia_measure_filter_floor: null argument");
  if (!c->begun) return ngia::fail(NGIA_E_STATE, "ngia_measure_filter_floor before ngia_cluster_begin");
  if (c->db.type != 0) return ngia::fail(NGIA_E_ARG, "ngia_measure_filter_floor: DNA databases only");
  const int nbw = (c->db.n + 31) / 32;
  constexpr int kB = NGIA_FILTER_WPW_BASE;
  const int grid = std::max(1, std::min(c->grid_filter, (nbw + 8 * kB - 1) / (8 * kB)));
  constexpr int kReps = 20;
  cudaEvent_t e0 = nullptr, e1 = nullptr, e2 = nullptr;
  cudaError_t e = cudaEventCreate(&e0);
  if (e == cudaSuccess) e = cudaEventCreate(&e1);
  if (e == cudaSuccess) e = cudaEventCreate(&e2);
  // the sink (written only in the impossible case above): the last counter
  // of the filter-statistics stripes
  unsigned long long *sink = c->rb.fstats + ngia::kFilterStripes * ngia::kFilterStats - 1;
  if (e == cudaSuccess) {
    ngia::k_floor_empty<<<grid, 256, 0, c->stream>>>(c->rb);  // warm-up
    ngia::k_floor_read<<<grid, 256, 0, c->stream>>>(c->db, c->rb, sink);
    cudaEventRecord(e0, c->stream);
    for (int r = 0; r < kReps; r++) ngia::k_floor_empty<<<grid, 256, 0, c->stream>>>(c->rb);
    cudaEventRecord(e1, c->stream);
    for (int r = 0; r < kReps; r++) ngia::k_floor_read<<<grid, 256, 0, c->stream>>>(c->db, c->rb, sink);
    cudaEventRecord(e2, c->stream);
    e = cudaEventSynchronize(e2);
  }
  float a = 0.f, b = 0.f;
  if (e == cudaSuccess) e = cudaEventElapsedTime(&a, e0, e1);
  if (e == cudaSuccess) e = cudaEventElapsedTime(&b, e1, e2);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  if (e2) cudaEventDestroy(e2);
  if (e != cudaSuccess) return ngia::fail(NGIA_E_CUDA, "ngia_measure_filter_floor: %s", cudaGetErrorString(e));
  *launch_us = 1e3 * a / kReps;
  *read_us = 1e3 * b / kReps;
  return NGIA_OK;
}
