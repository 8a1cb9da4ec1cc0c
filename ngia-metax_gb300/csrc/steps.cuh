// steps.cuh — the per-iteration steps of the greedy driver that work on one
// job's run state: preparing the representative, queueing a filter survivor
// and choosing the next representative.  The single-job kernels (filter.cu)
// run them on one context; the pooled batch kernels (pool.cu) run them once
// per job of the pool, one CTA each.
//
// Reference counterparts (CUDA/signalNode/src/func.cu): updateRepresent
// (186-238) and generateListGen/Pro (241-302).
#pragma once
#include <climits>
#include <stdint.h>

#include "common.cuh"
#include "kmer.cuh"

namespace ngia {

// Rep buffer layout: header words at [0, hw), planes from word kRepPlanes
// (16-byte aligned for the bulk copy).
constexpr int kRepPlanes = 32;

// Copies the representative's record into rb.rep_rec, builds its k-mer
// presence bitset (rb.rep_list) and resets the iteration's queues; every
// thread of the CTA calls it.  A finished run (done, at its iteration limit
// or failed) only clears the queues.
// score_rep >= 0: pair-score mode for that representative (no run state
// change); otherwise the representative is st->rep.
__device__ __forceinline__ void prep_body(const DevDB &db, const RunBufs &rb, const RunParams &prm, int score_rep) {
  RunState *st = rb.st;
  __shared__ int s_skip;
  __shared__ uint32_t s_list[kListWords];
  if (threadIdx.x == 0) {
    int skip = 0;
    if (score_rep < 0) skip = st->done || st->iter >= st->iter_limit || st->err;
    s_skip = skip;
  }
  __syncthreads();
  if (s_skip) {  // loop finished: nothing queued for the kernels after this one
    if (threadIdx.x == 0) {
      for (int k = 0; k < kNumClasses; k++) st->qcount[k] = st->qhead[k] = 0;
      st->long_count = 0;
    }
    return;
  }
  const int r = score_rep >= 0 ? score_rep : st->rep;
  const uint32_t *rec = db.words + db.off[r];
  const int L1 = (int)rec[0], net1 = (int)rec[1];
  const int nb1 = (net1 + 31) / 32;
  const int hw = db.hw, P = db.P;
  for (int i = threadIdx.x; i < hw; i += blockDim.x) rb.rep_rec[i] = rec[i];
  for (int i = threadIdx.x; i < nb1 * P; i += blockDim.x) rb.rep_rec[kRepPlanes + i] = rec[hw + i];
  // pair-score mode reports the short-word count whatever the precise flag
  const int word_active = (score_rep >= 0 || !prm.precise) && net1 >= 16;
  if (word_active) {
    const int bits = db.type ? 5 : 2;
    const int nbits_words = (int)((1u << (prm.w * bits)) / 32u);
    const int list_words = nbits_words < 1 ? 1 : nbits_words;
    for (int i = threadIdx.x; i < list_words; i += blockDim.x) s_list[i] = 0;
    __syncthreads();
    const uint32_t *planes = rec + hw;
    const uint32_t mask = (1u << (prm.w * bits)) - 1u;
    for (int p = prm.w - 1 + threadIdx.x; p < net1; p += blockDim.x) {
      uint32_t word = 0;
      for (int t = p - prm.w + 1; t <= p; t++)
        word = (word << bits) | (P == 2 ? code_at<2>(planes, t) : code_at<5>(planes, t));
      word &= mask;
      atomicOr(&s_list[word >> 5], 1u << (word & 31));
    }
    __syncthreads();
    for (int i = threadIdx.x; i < list_words; i += blockDim.x) rb.rep_list[i] = s_list[i];
  }
  if (threadIdx.x == 0) {
    st->rep_len = L1;
    st->rep_net = net1;
    st->rep_nb = nb1;
    st->word_active = word_active;
    for (int k = 0; k < kNumClasses; k++) st->qcount[k] = st->qhead[k] = 0;
    st->long_count = 0;
    if (score_rep < 0) {
      rb.cluster[r] = r;  // updateRepresent marks the representative (func.cu:235)
      rb.ident[r] = -1;
    }
  }
}


// Clears the finished representative from the unclustered set and finds the
// first unclustered sequence at or after it (the longest remaining one,
// func.cu:215).  In graph form it also sets the while-node condition.
__device__ __forceinline__ void next_body(const DevDB &db, const RunBufs &rb, unsigned long long cond, int use_cond) {
  RunState *st = rb.st;
  __shared__ int s_found, s_skip;
  __shared__ int s_min[32];
  if (threadIdx.x == 0) {
    s_skip = st->done || st->iter >= st->iter_limit || st->err;
    s_found = -1;
  }
  __syncthreads();
  if (s_skip) {
    if (use_cond && threadIdx.x == 0) cudaGraphSetConditional((cudaGraphConditionalHandle)cond, 0);
    return;
  }
  const int r = st->rep;
  const int nbw = (db.n + 31) / 32;
  if (threadIdx.x == 0) atomicAnd(&rb.alive[r >> 5], ~(1u << (r & 31)));
  if (threadIdx.x < 5) {  // fold this iteration's filter counters
    unsigned long long sum = 0;
    for (int k = 0; k < kFilterStripes; k++) {
      unsigned long long &f = rb.fstats[k * kFilterStats + threadIdx.x];
      sum += f;
      f = 0;
    }
    unsigned long long *dst[5] = {&st->st_candidates, &st->st_base_pass, &st->st_filter_bytes,
                                  &st->st_word_checks, &st->st_word_pass};
    *dst[threadIdx.x] += sum;
  }
  __syncthreads();
  for (int base = r >> 5; base < nbw; base += blockDim.x) {
    const int wi = base + threadIdx.x;
    const uint32_t w = wi < nbw ? rb.alive[wi] : 0u;
    int v = w ? wi : INT_MAX;
    for (int o = 16; o; o >>= 1) v = min(v, __shfl_xor_sync(kFullMask, v, o));
    if ((threadIdx.x & 31) == 0) s_min[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x < 32) {
      int u = threadIdx.x < (int)(blockDim.x >> 5) ? s_min[threadIdx.x] : INT_MAX;
      for (int o = 16; o; o >>= 1) u = min(u, __shfl_xor_sync(kFullMask, u, o));
      if (threadIdx.x == 0 && u != INT_MAX) s_found = u * 32 + __ffs(rb.alive[u]) - 1;
    }
    __syncthreads();
    if (s_found >= 0) break;
  }
  if (threadIdx.x == 0) {
    st->iter += 1;
    for (int k = 0; k < kNumClasses; k++) st->st_class_pairs[k] += st->qcount[k];
    if (s_found >= 0) {
      st->rep = s_found;
    } else {
      st->done = 1;
    }
    if (use_cond) {
      const int more = !st->done && st->iter < st->iter_limit && !st->err;
      cudaGraphSetConditional((cudaGraphConditionalHandle)cond, more ? 1u : 0u);
    }
  }
}

// Pushes candidate `c` of lane into work queue `cls` with one atomic per
// class and warp (warp-aggregated compaction).
__device__ __forceinline__ void push_queue(const RunBufs &rb, RunState *st, bool pass, int cls, int c) {
  const unsigned pm = __ballot_sync(kFullMask, pass);
  if (!pass) return;
  const unsigned peers = __match_any_sync(pm, cls);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (lane == leader) base = atomicAdd(&st->qcount[cls], (uint32_t)__popc(peers));
  base = __shfl_sync(peers, base, leader);
  rb.queue[cls][base + __popc(peers & ((1u << lane) - 1u))] = c;
}

}  // namespace ngia
