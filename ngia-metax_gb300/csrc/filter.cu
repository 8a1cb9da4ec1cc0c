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
#include <climits>

#include "ctx.h"

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

cudaError_t launch_loader(ngia_ctx *c, int32_t *d_maxnb, int32_t *d_short, int32_t *d_bad) {
  int grid = c->num_sms * 4;
  k_loader<<<grid, 256, 0, c->stream>>>(c->d_words, c->d_off, c->n_words, c->db.n, c->db.type, c->d_len,
                                        c->d_net, c->d_cnt, d_maxnb, d_short, d_bad);
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
    // Order of the two cheap-to-expensive tests.  Both orders give the same
    // members (a candidate joins iff all three tests pass); the short-word
    // filter goes first when it is expected to reject most candidates.
    int wf;
    if (prm.word_order == 1) wf = 1;
    else if (prm.word_order == 2) wf = 0;
    else wf = db.type == 0 ? (prm.s >= 0.93f) : 1;
    st->word_first = wf;
    st->word_active = 0;
    st->rep_nb = st->rep_len = st->rep_net = 0;
    st->st_candidates = st->st_base_pass = st->st_align_pairs = st->st_members = 0;
    st->st_band_cells = st->st_filter_bytes = st->st_word_checks = st->st_word_pass = 0;
    st->st_done_cells = 0;
    for (int k = 0; k < kNumClasses; k++) st->st_class_pairs[k] = 0;
  }
}

cudaError_t launch_init_run(ngia_ctx *c) {
  k_init_run<<<c->num_sms * 2, 256, 0, c->stream>>>(c->db, c->rb, c->prm);
  return cudaGetLastError();
}

// ---- representative preparation ----------------------------------------------
// Residue code of net position q of a record's planes.
template <int P>
__device__ __forceinline__ uint32_t code_at(const uint32_t *planes, int q) {
  const uint32_t *b = planes + (q >> 5) * P;
  uint32_t c = 0;
#pragma unroll
  for (int p = 0; p < P; p++) c |= ((b[p] >> (q & 31)) & 1u) << p;
  return c;
}

// Rep buffer layout: header words at [0, hw), planes from word kRepPlanes
// (16-byte aligned for the bulk copy).
constexpr int kRepPlanes = 32;

// score_rep >= 0: pair-score mode for that representative (no run state
// change); otherwise the representative is st->rep.
__global__ void k_prep(DevDB db, RunBufs rb, RunParams prm, int score_rep) {
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
    if (threadIdx.x == 0)
      for (int k = 0; k < kNumClasses; k++) st->qcount[k] = st->qhead[k] = 0;
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
    if (score_rep < 0) {
      rb.cluster[r] = r;  // updateRepresent marks the representative (func.cu:235)
      rb.ident[r] = -1;
    }
  }
}

cudaError_t launch_prep(ngia_ctx *c, int score_rep) {
  k_prep<<<1, 512, 0, c->stream>>>(c->db, c->rb, c->prm, score_rep);
  return cudaGetLastError();
}

// ---- short-word count of one candidate (kernel_wordFilter job body) ----------
template <int P>
__device__ int word_count(const uint32_t *__restrict__ planes, int net2, int w, const uint32_t *list) {
  constexpr int bits = P == 2 ? 2 : 5;
  const uint32_t mask = (1u << (w * bits)) - 1u;
  uint32_t word = 0;
  int sum = 0;
  for (int i = 0; i < net2; i += 32) {
    uint32_t pl[P];
#pragma unroll
    for (int p = 0; p < P; p++) pl[p] = __ldg(planes + (i >> 5) * P + p);
    const int lim = min(32, net2 - i);
    for (int j = 0; j < lim; j++) {
      uint32_t c = 0;
#pragma unroll
      for (int p = 0; p < P; p++) c |= ((pl[p] >> j) & 1u) << p;
      word = ((word << bits) | c) & mask;
      if (i + j >= w - 1) sum += (list[word >> 5] >> (word & 31)) & 1u;
    }
  }
  return sum;
}

// Composition sum of candidate c against the representative counts rc[].
template <int A>
__device__ __forceinline__ int base_sum(const uint32_t *__restrict__ cnt, int c, const uint32_t *rc) {
  int sum = 0;
  if (A == 4) {
    const uint4 q = __ldg(reinterpret_cast<const uint4 *>(cnt) + c);
    sum = (int)(min(q.x, rc[0]) + min(q.y, rc[1]) + min(q.z, rc[2]) + min(q.w, rc[3]));
  } else {
    const uint4 *q4 = reinterpret_cast<const uint4 *>(cnt + (int64_t)c * 28);
#pragma unroll
    for (int k = 0; k < 7; k++) {
      const uint4 q = __ldg(q4 + k);
      sum += (int)(min(q.x, rc[4 * k]) + min(q.y, rc[4 * k + 1]) + min(q.z, rc[4 * k + 2]) + min(q.w, rc[4 * k + 3]));
    }
  }
  return sum;
}

// Pushes candidate `c` of lane into work queue `cls` with one atomic per
// class and warp (warp-aggregated compaction).
__device__ __forceinline__ void push_queue(RunBufs &rb, RunState *st, bool pass, int cls, int c) {
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

__device__ __forceinline__ void flush_stats(RunState *st, unsigned long long cand, unsigned long long base,
                                            unsigned long long bytes, unsigned long long wchk,
                                            unsigned long long wpass) {
  for (int o = 16; o; o >>= 1) {
    cand += __shfl_down_sync(kFullMask, cand, o);
    base += __shfl_down_sync(kFullMask, base, o);
    bytes += __shfl_down_sync(kFullMask, bytes, o);
    wchk += __shfl_down_sync(kFullMask, wchk, o);
    wpass += __shfl_down_sync(kFullMask, wpass, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (cand) atomicAdd(&st->st_candidates, cand);
    if (base) atomicAdd(&st->st_base_pass, base);
    if (bytes) atomicAdd(&st->st_filter_bytes, bytes);
    if (wchk) atomicAdd(&st->st_word_checks, wchk);
    if (wpass) atomicAdd(&st->st_word_pass, wpass);
  }
}

// Fused filter over the unclustered set.  One warp per 32-sequence bitmap
// word: lanes read the header arrays of 32 consecutive sequences (coalesced),
// apply the composition test and, in word-first order, the short-word test
// (shared-memory k-mer bitset), then compact survivors into the alignment
// class queues.  `exact` = 1 runs the composition stage only and records the
// survivors (bitmap in rb.flags) for the exact short-word path.
template <int P>
__global__ void __launch_bounds__(256) k_filter(DevDB db, RunBufs rb, RunParams prm, int exact) {
  RunState *st = rb.st;
  extern __shared__ __align__(16) uint32_t s_list[];
  __shared__ uint64_t bar;
  __shared__ uint32_t s_rc[28];
  __shared__ int s_hdr[4];
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
  const int L1 = s_hdr[1], nb1 = s_hdr[2], word_here = s_hdr[3];
  const int list_words = max(1, (int)((1u << (prm.w * (P == 2 ? 2 : 5))) / 32u));
  if (word_here) {
    if (!stage_to_smem(s_list, rb.rep_list, (uint32_t)list_words, &bar, st, 1)) return;
  }
  const float s = prm.s;
  const int lane = threadIdx.x & 31;
  const int nbw = (db.n + 31) / 32;
  const int gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int nwarps = (gridDim.x * blockDim.x) >> 5;
  unsigned long long cand = 0, base = 0, bytes = 0, wchk = 0, wpass = 0;
  for (int wi = gw; wi < nbw; wi += nwarps) {
    const uint32_t bits = rb.alive[wi];
    if (!bits) {
      if (exact && lane == 0) reinterpret_cast<uint32_t *>(rb.flags)[wi] = 0;
      continue;
    }
    const int c = wi * 32 + lane;
    const bool alive = (bits >> lane) & 1u;
    bool pass = false;
    int cls = 0;
    if (alive) {
      cand++;
      bytes += 4 * (2 + A);
      const int L2 = __ldg(db.len + c);
      pass = !(base_sum<A>(db.cnt, c, s_rc) < cutoff_of(L2, s));
      if (pass) base++;
      if (pass && word_here) {
        const int net2 = __ldg(db.net + c);
        const uint32_t *planes = db.words + __ldg(db.off + c) + db.hw;
        const int ws = word_count<P>(planes, net2, prm.w, s_list);
        wchk++;
        bytes += 4ull * P * ((net2 + 31) / 32);
        pass = !(ws < word_min(L2, prm.w, s));
        if (pass) wpass++;
      }
      if (pass && !exact) cls = class_of(db.type, window_of(band_blocks(L1, L2, s), nb1));
    }
    if (exact) {
      const unsigned m = __ballot_sync(kFullMask, pass);
      if (lane == 0) reinterpret_cast<uint32_t *>(rb.flags)[wi] = m;
    } else {
      push_queue(rb, st, pass, cls, c);
    }
  }
  flush_stats(st, cand, base, bytes, wchk, wpass);
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
  flush_stats(st, 0, 0, bytes, wchk, wpass);
}

cudaError_t launch_filter(ngia_ctx *c) {
  const int P = c->db.P;
  const int bits = c->db.type ? 5 : 2;
  const int list_words = std::max(1, (int)((1u << (c->prm.w * bits)) / 32u));
  const size_t smem = (size_t)list_words * 4;
  // Exact path only matters when the short-word filter can run and some
  // record is shorter than 16 residues.
  const bool exact = c->db.has_short && !c->prm.precise;
  if (!exact) {
    if (P == 2)
      k_filter<2><<<c->grid_filter, 256, smem, c->stream>>>(c->db, c->rb, c->prm, 0);
    else
      k_filter<5><<<c->grid_filter, 256, smem, c->stream>>>(c->db, c->rb, c->prm, 0);
    return cudaGetLastError();
  }
  if (P == 2)
    k_filter<2><<<c->grid_filter, 256, smem, c->stream>>>(c->db, c->rb, c->prm, 1);
  else
    k_filter<5><<<c->grid_filter, 256, smem, c->stream>>>(c->db, c->rb, c->prm, 1);
  const int nbw = (c->db.n + 31) / 32;
  k_scan_words<<<1, 1024, 0, c->stream>>>(reinterpret_cast<const uint32_t *>(c->rb.flags), nbw, c->rb.scan_part);
  k_first_short<<<64, 256, 0, c->stream>>>(c->db, c->rb, 1);
  k_first_short<<<c->num_sms * 2, 256, 0, c->stream>>>(c->db, c->rb, 0);
  if (P == 2)
    k_word_exact<2><<<c->grid_filter, 256, smem, c->stream>>>(c->db, c->rb, c->prm);
  else
    k_word_exact<5><<<c->grid_filter, 256, smem, c->stream>>>(c->db, c->rb, c->prm);
  return cudaGetLastError();
}

// ---- next representative -----------------------------------------------------
// Clears the finished representative from the unclustered set and finds the
// first unclustered sequence at or after it (the longest remaining one,
// func.cu:215).  In graph form it also sets the while-node condition.
__global__ void k_next(DevDB db, RunBufs rb, unsigned long long cond, int use_cond) {
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
