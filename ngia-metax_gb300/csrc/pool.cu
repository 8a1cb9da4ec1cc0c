// pool.cu — the pooled form of a batch: the jobs of a batch that share a
// record type advance together, one representative each per round, and every
// stage of a round is ONE launch over all of them.
//
// A round:
//   k_pool_prep     one CTA per job: the job's representative (rep record,
//                   k-mer bitset, queue reset; steps.cuh) and the round's
//                   per-job header (rep length, blocks, composition counts,
//                   test order)
//   k_pool_filter   the composition test (and, in word-first order, the
//                   short-word test) of every unclustered sequence of every
//                   job: warps take bitmap words of the pool's word space (the
//                   jobs' bitmaps end to end) and queue survivors into their
//                   job's length buckets (alignment classes, by band window)
//                   and, in its last CTA, per bucket: the pairs of all jobs
//                   cut into chunks and a prefix of chunks over the jobs (the
//                   cross-job work queue)
//   k_pool_align    per bucket, one persistent launch: a CTA claims the next
//                   chunk of the bucket, whichever job it belongs to, stages
//                   that job's representative (planes, k-mer bitset, DNA
//                   match table) in shared memory when it differs from the one
//                   staged, and its lanes run the chunk's pairs through the
//                   tiled banded LCS (tile.cuh), thread per pair
//   k_pool_next     one CTA per job: retire the representative, next one;
//                   the last CTA sets the graph's WHILE condition (any job
//                   left)
//
// The batch graph (batch.cu) holds one WHILE node per pool (DNA, protein)
// beside the per-job nodes of jobs the pool does not take: a job whose
// database holds records of net length < 16 while the short-word test is on
// (the reference's word kernel then returns a whole thread, func.cu:375,
// 420, and whether a job is tested depends on its position in that job's
// list; filter.cu reproduces it per job).  Every job's result is the same as
// clustering it alone: the per-pair tests are the reference's
// (func.cu:323-604) and each job's greedy order is untouched.
#include <algorithm>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "../host/host_common.h"
#include "ctx.h"
#include "kmer.cuh"
#include "steps.cuh"
#include "tile.cuh"

namespace ngia {
namespace pool {

// Device table entry of one job (copied from its context before a run).
struct PoolJob {
  DevDB db;
  RunBufs rb;
  RunParams prm;
};

// Per-job header of the current round, written by k_pool_prep.
struct PoolHdr {
  int32_t active, L1, nb1, net1, word_here, word_after, rep, pad;
  uint32_t rc[28];
};

struct PoolDev {
  const PoolJob *jobs;
  PoolHdr *hdr;
  const int32_t *wbase;  // n_jobs + 1: first bitmap word of every job in the pool's word space
  int32_t *chunk_base;   // kNumClasses x (n_jobs + 1): first chunk of every job, per bucket
  int32_t *chunk_size;   // kNumClasses: pairs per chunk this round
  uint32_t *ctr;         // kNumClasses: chunks claimed this round
  uint32_t *done;        // [0] filter CTAs finished, [1] next CTAs finished (last one resets)
  uint32_t *scratch;     // global ring of the widest bucket
  int64_t scratch_words;
  uint32_t ring_mask;
  int32_t n_jobs, type, total_words;
  int32_t grid_align[kNumClasses];
};

constexpr int kPoolWarpWordLen = 2048;  // longer candidates are word-counted by a whole warp
constexpr int kPoolMaxJobs = 8192;       // the filter keeps the word prefix in shared memory
static_assert(sizeof(PoolJob) % 4 == 0, "job entries are copied as words");

// Copies a job's table entry into shared memory with the whole CTA.
__device__ __forceinline__ void load_job(const PoolJob *src, PoolJob *dst) {
  const uint32_t *s = reinterpret_cast<const uint32_t *>(src);
  uint32_t *d = reinterpret_cast<uint32_t *>(dst);
  for (int i = threadIdx.x; i < (int)(sizeof(PoolJob) / 4); i += blockDim.x) d[i] = s[i];
  __syncthreads();
}

__device__ __forceinline__ bool job_running(const RunState *st) {
  return !(st->done || st->iter >= st->iter_limit || st->err);
}

// ---- prep -------------------------------------------------------------------
// Shared storage for one job's table entry (raw words: the entry is copied
// in by load_job, nothing is constructed).
#define NGIA_POOL_SHARED_JOB(name)                                            \
  __shared__ __align__(16) uint32_t name##_raw[sizeof(PoolJob) / 4];          \
  PoolJob &name = *reinterpret_cast<PoolJob *>(name##_raw)

__global__ void __launch_bounds__(512) k_pool_prep(PoolDev pd) {
  NGIA_POOL_SHARED_JOB(s_job);
  const int j = blockIdx.x;
  load_job(pd.jobs + j, &s_job);
  prep_body(s_job.db, s_job.rb, s_job.prm, -1);
  __syncthreads();
  const RunState *st = s_job.rb.st;
  PoolHdr *H = pd.hdr + j;
  if (threadIdx.x == 0) {
    const bool act = job_running(st);
    H->active = act;
    H->L1 = st->rep_len;
    H->nb1 = st->rep_nb;
    H->net1 = st->rep_net;
    H->rep = st->rep;
    H->word_here = act && st->word_first && st->word_active;
    H->word_after = act && !st->word_first && st->word_active;
  }
  if (threadIdx.x < s_job.db.A) H->rc[threadIdx.x] = s_job.rb.rep_rec[2 + threadIdx.x];
}

// ---- chunks -------------------------------------------------------------------
// Per bucket: the chunk size of this round (about eight chunks per CTA of the
// bucket's launch, 128 to 4,096 pairs) and the exclusive prefix of every
// job's chunk count.  Run by the last CTA of the filter (NT threads).
// Chunk size of a bucket: its pairs over NGIA_POOL_CHUNK_DIV chunks per CTA
// of the alignment grid, at least NGIA_POOL_CHUNK_MIN and at most 4,096
// pairs.  A CTA's warps meet at a barrier between chunks.  Swept on GB300
// (256-job batch, 8 iterations per job): 16/64, 8/128, 4/256 and 2/512 gave
// 13.7M, 17.0M, 16.2M and 15.3M candidate seqs/s.
#ifndef NGIA_POOL_CHUNK_DIV
#define NGIA_POOL_CHUNK_DIV 8
#endif
#ifndef NGIA_POOL_CHUNK_MIN
#define NGIA_POOL_CHUNK_MIN 128
#endif
template <int NT>
__device__ void chunks_body(const PoolDev &pd, int ncls) {
  __shared__ long long s_red[NT / 32];
  __shared__ int32_t s_part[NT];
  __shared__ int32_t s_C;
  const int nj = pd.n_jobs, t = threadIdx.x;
  const int per = (nj + NT - 1) / NT;
  const int j0 = min(nj, t * per), j1 = min(nj, j0 + per);
  for (int k = 0; k < ncls; k++) {
    long long tot = 0;
    for (int j = j0; j < j1; j++) tot += pd.jobs[j].rb.st->qcount[k];
#pragma unroll
    for (int o = 16; o; o >>= 1) tot += __shfl_xor_sync(kFullMask, tot, o);
    if ((t & 31) == 0) s_red[t >> 5] = tot;
    __syncthreads();
    if (t == 0) {
      long long T = 0;
      for (int i = 0; i < NT / 32; i++) T += s_red[i];
      const long long per = (long long)NGIA_POOL_CHUNK_DIV * pd.grid_align[k];
      const long long want = (T + per - 1) / per;
      s_C = (int)max((long long)NGIA_POOL_CHUNK_MIN, min(4096ll, want));
    }
    __syncthreads();
    const int C = s_C;
    int mine = 0;
    for (int j = j0; j < j1; j++) mine += (int)((pd.jobs[j].rb.st->qcount[k] + C - 1) / C);
    s_part[t] = mine;
    __syncthreads();
    for (int o = 1; o < NT; o <<= 1) {  // inclusive scan of the partials
      const int v = t >= o ? s_part[t - o] : 0;
      __syncthreads();
      s_part[t] += v;
      __syncthreads();
    }
    int32_t *cb = pd.chunk_base + k * (nj + 1);
    int run = s_part[t] - mine;
    for (int j = j0; j < j1; j++) {
      cb[j] = run;
      run += (int)((pd.jobs[j].rb.st->qcount[k] + C - 1) / C);
    }
    if (t == NT - 1) {
      cb[nj] = s_part[NT - 1];
      pd.chunk_size[k] = C;
      pd.ctr[k] = 0;
    }
    __syncthreads();
  }
}

// True in exactly one CTA of the grid: the last to finish (its view of the
// other CTAs' global writes is complete after the fence).  Resets *done.
__device__ __forceinline__ bool last_cta(uint32_t *done) {
  __shared__ int s_last;
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(done, 1u) == gridDim.x - 1;
    if (s_last) *done = 0;  // every other CTA has counted: ready for the next round
  }
  __syncthreads();
  if (s_last) __threadfence();
  return s_last;
}

// ---- filter -------------------------------------------------------------------
// Short-word count of one candidate by the whole warp against a k-mer
// bitset in global memory: lane l takes blocks l, l+32, ...; each block's
// history (the last w-1 residues of the block below) comes from the lane
// below by a shuffle.  Counts positions q >= w-1 (func.cu:376-396).  All 32
// lanes call it with the same arguments.
template <int P>
__device__ int word_count_warp_bits(const uint32_t *__restrict__ planes, int net2, int w, const uint32_t *list) {
  constexpr int bits = P == 2 ? 2 : 5;
  const uint32_t mask = (1u << (w * bits)) - 1u;
  const int lane = threadIdx.x & 31;
  const int nb = (net2 + 31) >> 5;
  int sum = 0;
  uint32_t carry[P];
#pragma unroll
  for (int p = 0; p < P; p++) carry[p] = 0u;
  for (int b0 = 0; b0 < nb; b0 += 32) {
    const int b = b0 + lane;
    const bool have = b < nb;
    const int lim = have ? min(32, net2 - 32 * b) : 0;
    uint32_t pl[P], pv[P];
#pragma unroll
    for (int p = 0; p < P; p++) {
      pl[p] = have ? __ldg(planes + b * P + p) : 0u;
      pv[p] = __shfl_up_sync(kFullMask, pl[p], 1);
      if (lane == 0) pv[p] = carry[p];
    }
    uint32_t word = 0;
    for (int k = 32 - (w - 1); k < 32; k++) {  // history: the block below's last w-1 residues
      uint32_t c = 0;
#pragma unroll
      for (int p = 0; p < P; p++) c |= ((pv[p] >> k) & 1u) << p;
      word = ((word << bits) | c) & mask;
    }
    for (int k = 0; k < lim; k++) {
      uint32_t c = 0;
#pragma unroll
      for (int p = 0; p < P; p++) c |= ((pl[p] >> k) & 1u) << p;
      word = ((word << bits) | c) & mask;
      if (32 * b + k >= w - 1) sum += (list[word >> 5] >> (word & 31)) & 1u;
    }
#pragma unroll
    for (int p = 0; p < P; p++) carry[p] = __shfl_sync(kFullMask, pl[p], 31);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) sum += __shfl_xor_sync(kFullMask, sum, o);
  return sum;
}

template <int P>
__global__ void __launch_bounds__(256) k_pool_filter(PoolDev pd, int ncls) {
  constexpr int A = P == 2 ? 4 : 28;
  constexpr int type = P == 2 ? 0 : 1;
  extern __shared__ int32_t s_wbase[];  // n_jobs + 1
  for (int i = threadIdx.x; i <= pd.n_jobs; i += blockDim.x) s_wbase[i] = pd.wbase[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int W = gridDim.x * (blockDim.x >> 5);
  for (int gw = blockIdx.x * (blockDim.x >> 5) + warp; gw < pd.total_words; gw += W) {
    int lo = 0, hi = pd.n_jobs;  // s_wbase[lo] <= gw < s_wbase[hi]
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (s_wbase[mid] <= gw) lo = mid;
      else hi = mid;
    }
    const int j = lo;
    const PoolHdr *H = pd.hdr + j;
    if (!H->active) continue;  // warp-uniform
    const PoolJob *J = pd.jobs + j;
    const int wi = gw - s_wbase[j];
    const uint32_t bits = J->rb.alive[wi];
    if (!bits) continue;  // warp-uniform
    const float s = J->prm.s;
    const int w = J->prm.w;
    const int L1 = H->L1, nb1 = H->nb1, word_here = H->word_here;
    const int c = wi * 32 + lane;
    bool pass = false, deferred = false;
    int cls = 0;
    unsigned long long cand = 0, base = 0, bytes = 0, wchk = 0, wpass = 0;
    if ((bits >> lane) & 1u) {
      cand = 1;
      bytes = 4 * (2 + A);
      const int L2 = __ldg(J->db.len + c);
      pass = !(base_sum<A>(J->db.cnt, c, H->rc) < cutoff_of(L2, s));
      if (pass) {
        base = 1;
        if (word_here) {
          const int net2 = __ldg(J->db.net + c);
          wchk = 1;
          bytes += 4ull * P * ((net2 + 31) / 32);
          if (net2 <= kPoolWarpWordLen) {
            const uint32_t *planes = J->db.words + __ldg(J->db.off + c) + J->db.hw;
            pass = !(word_count<P>(planes, net2, w, J->rb.rep_list) < word_min(L2, w, s));
            wpass = pass;
          } else {
            deferred = true;
          }
        }
        if (pass && !deferred) cls = class_of(type, window_of(band_blocks(L1, L2, s), nb1));
      }
    }
    for (unsigned dm = __ballot_sync(kFullMask, deferred); dm; dm &= dm - 1) {
      const int src = __ffs(dm) - 1;
      const int cc = wi * 32 + src;
      const uint32_t *planes = J->db.words + __ldg(J->db.off + cc) + J->db.hw;
      const int ws = word_count_warp_bits<P>(planes, __ldg(J->db.net + cc), w, J->rb.rep_list);
      if (lane == src) {
        const int L2 = __ldg(J->db.len + cc);
        pass = !(ws < word_min(L2, w, s));
        wpass = pass;
        if (pass) cls = class_of(type, window_of(band_blocks(L1, L2, s), nb1));
      }
    }
    push_queue(J->rb, J->rb.st, pass, cls, c);
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      cand += __shfl_down_sync(kFullMask, cand, o);
      base += __shfl_down_sync(kFullMask, base, o);
      bytes += __shfl_down_sync(kFullMask, bytes, o);
      wchk += __shfl_down_sync(kFullMask, wchk, o);
      wpass += __shfl_down_sync(kFullMask, wpass, o);
    }
    if (lane == 0) {  // folded into the run state by the job's next step
      unsigned long long *f = J->rb.fstats + (gw % kFilterStripes) * kFilterStats;
      if (cand) atomicAdd(f + 0, cand);
      if (base) atomicAdd(f + 1, base);
      if (bytes) atomicAdd(f + 2, bytes);
      if (wchk) atomicAdd(f + 3, wchk);
      if (wpass) atomicAdd(f + 4, wpass);
    }
  }
  // the last CTA cuts every bucket's pairs into chunks (the pairs' counts
  // are final once every CTA has queued its survivors)
  if (last_cta(pd.done)) chunks_body<256>(pd, ncls);
}

// ---- alignment -------------------------------------------------------------------
// Shared memory: rep planes | k-mer bitset | row ring (RING > 0) | DNA match
// table; the same layout as k_align_tiled (align.cu).
template <int P, int RING>
__global__ void __launch_bounds__(kAlignThreads, tiled_min_blocks(P)) k_pool_align(PoolDev pd, int cls, int max_nb) {
  extern __shared__ __align__(16) uint32_t smem[];
  __shared__ uint64_t bar;
  __shared__ int s_j, s_a, s_b;
  __shared__ uint32_t s_next;
  __shared__ unsigned long long s_qw;
  constexpr bool kEq = P == 2 && NGIA_ALIGN_EQ;
  constexpr int MT = tiled_main(P);
  const int nj = pd.n_jobs;
  const int32_t *cb = pd.chunk_base + cls * (nj + 1);
  const int lane = threadIdx.x & 31;
  uint32_t *s_pl = smem;
  uint32_t *s_list = smem + ((max_nb * P + 3) & ~3);
  uint32_t *s_eq = smem + tiled_eq_off(P, max_nb, RING);
  const uint32_t s_eq_s = smem_u32(s_eq);
  (void)s_eq_s;
  typename RingOf<RING>::T ring;
  if constexpr (RING > 0) {
    ring.base = smem + (((max_nb * P + 3) & ~3) + kListWords) + threadIdx.x;
  } else {
    const int64_t TL = (int64_t)gridDim.x * blockDim.x;
    if ((int64_t)(pd.ring_mask + 1) * TL > pd.scratch_words) return;  // the host sizes the grid to the scratch
    ring.base = pd.scratch + (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    ring.mask = pd.ring_mask;
    ring.stride = TL;
  }
  if (threadIdx.x == 0) mbar_init(&bar, 1);
  __syncthreads();
  uint32_t phase = 0;
  int staged = -1;
  bool broken = false;  // a staging copy of this CTA did not land
  // the staged job's representative
  int L1 = 0, net1 = 0, nb1 = 0, rep = 0, word_after = 0;
  uint32_t vlast = 0;
  // 1 and 4 as values ptxas cannot fold (the FMA-pipe bookkeeping of tile.cuh)
  const uint32_t one_rt = 1u + (uint32_t)(max_nb < 0);
  const FmaK fk{one_rt, one_rt << 2};
  (void)fk;
  for (;;) {
    if (threadIdx.x == 0) {
      const uint32_t u = atomicAdd(&pd.ctr[cls], 1u);
      int j = -1, a = 0, b = 0;
      if ((int)u < cb[nj]) {
        int lo = 0, hi = nj;  // cb[lo] <= u < cb[hi]
        while (hi - lo > 1) {
          const int mid = (lo + hi) >> 1;
          if (cb[mid] <= (int)u) lo = mid;
          else hi = mid;
        }
        j = lo;
        const int C = pd.chunk_size[cls];
        a = ((int)u - cb[j]) * C;
        b = min(a + C, (int)pd.jobs[j].rb.st->qcount[cls]);
      }
      s_j = j;
      s_a = a;
      s_b = b;
      s_next = (uint32_t)a;
      s_qw = 0;
    }
    __syncthreads();
    const int j = s_j;
    if (j < 0) break;
    const PoolJob *J = pd.jobs + j;
    RunState *st = J->rb.st;
    if (broken) {  // the chunk's job stops with an error instead of losing pairs silently
      if (threadIdx.x == 0) set_error(st, NGIA_ERR_MBAR_TIMEOUT, 40 + cls);
      __syncthreads();
      continue;
    }
    if (j != staged) {
      const PoolHdr *H = pd.hdr + j;
      L1 = H->L1;
      net1 = H->net1;
      nb1 = H->nb1;
      rep = H->rep;
      word_after = H->word_after;
      vlast = (net1 & 31) ? ((1u << (net1 & 31)) - 1u) : 0xFFFFFFFFu;
      const int bits = P == 2 ? 2 : 5;
      const uint32_t plane_words = (uint32_t)((nb1 * P + 3) & ~3);
      const uint32_t list_words = word_after ? (uint32_t)max(4, (int)((1u << (J->prm.w * bits)) / 32u)) : 0u;
      if (threadIdx.x == 0) {
        // the planes and bitset regions were last read through the generic proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        const uint32_t bytes = 4u * (plane_words + list_words);
        if (bytes) {
          mbar_expect_tx(&bar, bytes);
          if (plane_words) bulk_g2s(s_pl, J->rb.rep_rec + kRepPlanes, 4u * plane_words, &bar);
          if (list_words) bulk_g2s(s_list, J->rb.rep_list, 4u * list_words, &bar);
        } else {
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&bar)) : "memory");
        }
      }
      const bool ok = mbar_wait_bounded(&bar, phase & 1u, J->prm.wait_polls);
      if (!ok) mbar_wait_bounded(&bar, phase & 1u, kWaitPolls);  // let the copy in flight land
      phase++;
      if (!__syncthreads_and(ok)) {
        if (threadIdx.x == 0) set_error(st, NGIA_ERR_MBAR_TIMEOUT, 40 + cls);
        broken = true;
        __syncthreads();
        continue;
      }
      if constexpr (kEq) {
        build_eq(s_pl, nb1, s_eq);
        __syncthreads();
      }
      staged = j;
    }
    // the chunk's pairs: one thread per pair, lockstep refill (align.cu)
    const float s = J->prm.s;
    const int w = J->prm.w, refill = J->prm.refill;
    const int32_t *queue = J->rb.queue[cls];
    const DevDB db = J->db;
    int32_t *cluster = J->rb.cluster, *ident = J->rb.ident;
    uint32_t *alive = J->rb.alive;
    const int b_end = s_b;
    int state = -1, cand = 0;
    int i = 0, nq = 0, B = 0, js = 0, je = -1, net2 = 0, L2 = 0, cutoff = 0, lastcols = 32, frozen = 0, zw = 0;
    bool active = false;
    const uint32_t *qpl = nullptr;
    uint32_t cur[P], nxt[P];
    unsigned long long n_pairs = 0, n_members = 0, n_cells = 0, n_done = 0;
    for (;;) {
      {
        const unsigned idle = __ballot_sync(kFullMask, state == -1);
        const bool any_busy = __any_sync(kFullMask, state >= 0);  // every lane votes
        if (__popc(idle) >= refill || !any_busy) {
          const bool need = state == -1;
          const unsigned nm = __ballot_sync(kFullMask, need);
          if (nm) {
            const int leader = __ffs(nm) - 1;
            uint32_t base = 0;
            if (lane == leader) base = atomicAdd(&s_next, (uint32_t)__popc(nm));
            base = __shfl_sync(kFullMask, base, leader);
            if (need) {
              const uint32_t idx = base + (uint32_t)__popc(nm & ((1u << lane) - 1u));
              state = idx < (uint32_t)b_end ? (int)idx : -2;
            }
          }
        }
      }
      if (__all_sync(kFullMask, state == -2)) break;
      bool busy = state >= 0;
      if (busy && !active) {
        cand = queue[state];
        L2 = __ldg(db.len + cand);
        net2 = __ldg(db.net + cand);
        nq = (net2 + 31) >> 5;
        lastcols = (net2 & 31) ? (net2 & 31) : 32;
        B = band_blocks(L1, L2, s);
        cutoff = cutoff_of(L2, s);
        qpl = db.words + __ldg(db.off + cand) + db.hw;
        i = 0;
        js = 0;
        je = min(B, nb1 - 1);
        frozen = 0;
        zw = 0;
        n_pairs++;
        n_cells += (unsigned long long)band_cells(B, nb1, net2);
        atomicAdd(&s_qw, (unsigned long long)(nq * P));
        if (B < 0 || je < 0 || nq == 0) {
          // no band: score 0 (func.cu never updates the rows)
          if (!(0 < cutoff) && !(word_after && word_count<P>(qpl, net2, w, s_list) < word_min(L2, w, s))) {
            cluster[cand] = rep;
            ident[cand] = 0;
            atomicAnd(&alive[cand >> 5], ~(1u << (cand & 31)));
            n_members++;
          }
          state = -1;
          busy = false;
        } else {
          for (int jj = 0; jj <= je; jj++) ring[jj] = 0xFFFFFFFFu;
#pragma unroll
          for (int p = 0; p < P; p++) cur[p] = __ldg(qpl + p);
          active = true;
        }
      }
      const int n = busy ? je - js + 1 : 0;
      const int full = (int)__reduce_min_sync(kFullMask, busy ? (unsigned)(n / MT) : 0xFFFFFFFFu);
      int rem = (int)__reduce_max_sync(kFullMask, busy ? (unsigned)(n - MT * full) : 0u);
      if (!busy) continue;
      const int cols = (i == nq - 1) ? lastcols : 32;
      n_done += (unsigned long long)n * cols;
      if (i + 1 < nq) {
#pragma unroll
        for (int p = 0; p < P; p++) nxt[p] = __ldg(qpl + (i + 1) * P + p);
      }
      using Ring = typename RingOf<RING>::T;
      if constexpr (kEq && NGIA_EQ_FMA) {
        uint32_t wc[2];
        eq_codes_top(cur, wc);
        uint32_t cw = 0, ncw = 0;
        int base = js;
        if (NGIA_EQ_NOZOLD) zw = 0;  // the tiles return their rows' zero counts
        for (int t = 0; t < full; t++, base += MT) {
          zw += tiled_tile_eqf<MT, NGIA_EQ_PF_MAIN, Ring>(ring, s_eq_s, base, je, nb1, cols, wc, cw, ncw, fk);
          cw = ncw << (32 - cols);  // column 0's carry at bit 31
          ncw = 0;
        }
        for (; rem >= MT; rem -= MT, base += MT) {
          zw += tiled_tile_eqf<MT, NGIA_EQ_PF_MAIN, Ring>(ring, s_eq_s, base, je, nb1, cols, wc, cw, ncw, fk);
          cw = ncw << (32 - cols);
          ncw = 0;
        }
        if (rem > 0) zw += tiled_rem_eqf<Ring, MT>(rem, ring, s_eq_s, base, je, nb1, cols, wc, cw, ncw, fk);
      } else if constexpr (kEq) {
        uint32_t q[4];
        eq_codes(cur, q);
        uint32_t cw = 0, ncw = 0;
        int base = js;
        for (int t = 0; t < full; t++, base += MT) {
          zw += tiled_tile_eq<MT, NGIA_EQ_PF_MAIN, Ring>(ring, s_eq, base, je, nb1, cols, q, cw, ncw);
          cw = ncw << (32 - cols);
          ncw = 0;
        }
        for (; rem >= MT; rem -= MT, base += MT) {
          zw += tiled_tile_eq<MT, NGIA_EQ_PF_MAIN, Ring>(ring, s_eq, base, je, nb1, cols, q, cw, ncw);
          cw = ncw << (32 - cols);
          ncw = 0;
        }
        if (rem > 0) zw += tiled_rem_eq<Ring, MT>(rem, ring, s_eq, base, je, nb1, cols, q, cw, ncw);
      } else {
        uint32_t cw = 0, ncw = 0;
        int base = js;
        for (int t = 0; t < full; t++, base += MT) {
          zw += tiled_tile<P, MT, Ring>(ring, s_pl, base, je, cols, cur, cw, ncw);
          cw = ncw << (32 - cols);
          ncw = 0;
        }
        for (; rem >= MT; rem -= MT, base += MT) {
          zw += tiled_tile<P, MT, Ring>(ring, s_pl, base, je, cols, cur, cw, ncw);
          cw = ncw << (32 - cols);
          ncw = 0;
        }
        if (rem > 0) zw += tiled_rem<P, Ring, MT>(rem, ring, s_pl, base, je, cols, cur, cw, ncw);
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
        for (int jj = js; jj <= je; jj++) sum += __popc(~ring[jj] & (jj == nb1 - 1 ? vlast : 0xFFFFFFFFu));
        bool pass = !(sum < cutoff);
        // short-word test after the alignment (func.cu:376-396), members only
        if (pass && word_after) pass = !(word_count<P>(qpl, net2, w, s_list) < word_min(L2, w, s));
        if (pass) {
          cluster[cand] = rep;
          ident[cand] = sum;
          atomicAnd(&alive[cand >> 5], ~(1u << (cand & 31)));
          n_members++;
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
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      n_pairs += __shfl_down_sync(kFullMask, n_pairs, o);
      n_members += __shfl_down_sync(kFullMask, n_members, o);
      n_cells += __shfl_down_sync(kFullMask, n_cells, o);
      n_done += __shfl_down_sync(kFullMask, n_done, o);
    }
    if (lane == 0) {
      if (n_pairs) atomicAdd(&st->st_align_pairs, n_pairs);
      if (n_members) atomicAdd(&st->st_members, n_members);
      if (n_cells) atomicAdd(&st->st_band_cells, n_cells);
      if (n_done) {
        atomicAdd(&st->st_done_cells, n_done * 32ull);
        atomicAdd(&st->st_class_done[cls], n_done * 32ull);
      }
    }
    __syncthreads();  // every warp is done with the chunk (and the staged representative)
    if (threadIdx.x == 0 && s_qw) atomicAdd(&st->st_class_qwords[cls], s_qw);
  }
}

// ---- next representative, loop condition -----------------------------------------
// One CTA per job; the last CTA to finish sets the loop's condition: any job
// still running.
__global__ void __launch_bounds__(1024) k_pool_next(PoolDev pd, cudaGraphConditionalHandle cond) {
  NGIA_POOL_SHARED_JOB(s_job);
  load_job(pd.jobs + blockIdx.x, &s_job);
  next_body(s_job.db, s_job.rb, 0ull, 0);
  if (!last_cta(pd.done + 1)) return;
  int more = 0;
  for (int j = threadIdx.x; j < pd.n_jobs; j += blockDim.x) more |= job_running(pd.jobs[j].rb.st) ? 1 : 0;
  more = __syncthreads_or(more);
  if (threadIdx.x == 0) cudaGraphSetConditional(cond, more ? 1u : 0u);
}

// ---- host side -------------------------------------------------------------------
using PoolAlignFn = void (*)(PoolDev, int, int);

// Ring per bucket: every window up to 64 blocks in the 64-slot shared ring,
// then 128, then the global ring (the last bucket).
int ring_of(int type, int cls) {
  const int cap = class_cap(type, cls);
  return cap == 0 ? 0 : cap <= 64 ? 64 : 128;
}

PoolAlignFn align_fn(int type, int ring) {
  if (type == 0) return ring == 64 ? k_pool_align<2, 64> : ring == 128 ? k_pool_align<2, 128> : k_pool_align<2, 0>;
  return ring == 64 ? k_pool_align<5, 64> : ring == 128 ? k_pool_align<5, 128> : k_pool_align<5, 0>;
}

size_t align_smem(int type, int max_nb, int ring) {
  const int P = type ? 5 : 2;
  size_t words = (size_t)tiled_eq_off(P, max_nb, ring);
  if (P == 2 && NGIA_ALIGN_EQ) words += (size_t)eq_words(max_nb);
  return 4 * words;
}

struct Group {
  int type = 0;
  std::vector<ngia_ctx *> jobs;
  int max_nb = 1, num_sms = 1, grid_filter = 1;
  size_t smem[kNumClasses] = {0};
  PoolDev pd{};
  PoolJob *d_jobs = nullptr;
  PoolHdr *d_hdr = nullptr;
  int32_t *d_wbase = nullptr, *d_chunk_base = nullptr, *d_chunk_size = nullptr;
  uint32_t *d_ctr = nullptr, *d_scratch = nullptr, *d_done = nullptr;
  cudaStream_t side[kNumClasses] = {nullptr};
  cudaEvent_t fork = nullptr, join[kNumClasses] = {nullptr};
};

template <class T>
cudaError_t dalloc(T **p, size_t n) {
  return cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(n, 1));
}

// The dynamic shared memory limit of a pool kernel only grows (batches with
// shorter records cannot lower it under an open one with longer records).
cudaError_t configure(int type, int max_nb) {
  static std::mutex mu;
  static size_t have[64][2][3] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(mu);
  const int rings[3] = {64, 128, 0};
  for (int r = 0; r < 3; r++) {
    const size_t want = align_smem(type, max_nb, rings[r]);
    size_t &h = have[dev][type ? 1 : 0][r];
    if (want <= h) continue;
    e = cudaFuncSetAttribute((const void *)align_fn(type, rings[r]), cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)want);
    if (e != cudaSuccess) return e;
    h = want;
  }
  return cudaSuccess;
}

void group_close(Group *g) {
  if (!g) return;
  for (void *p : {(void *)g->d_jobs, (void *)g->d_hdr, (void *)g->d_wbase, (void *)g->d_chunk_base,
                  (void *)g->d_chunk_size, (void *)g->d_ctr, (void *)g->d_scratch, (void *)g->d_done})
    if (p) cudaFree(p);
  for (auto &s : g->side)
    if (s) cudaStreamDestroy(s);
  if (g->fork) cudaEventDestroy(g->fork);
  for (auto &e : g->join)
    if (e) cudaEventDestroy(e);
  delete g;
}

int group_open(const std::vector<ngia_ctx *> &jobs, Group **out) {
  *out = nullptr;
  if (jobs.empty() || (int)jobs.size() > kPoolMaxJobs)
    return fail(NGIA_E_LIMIT, "pool: %zu jobs of one record type (at most %d)", jobs.size(), kPoolMaxJobs);
  Group *g = new (std::nothrow) Group();
  if (!g) return fail(NGIA_E_NOMEM, "pool: out of host memory");
  g->jobs = jobs;
  g->type = jobs[0]->db.type;
  g->num_sms = jobs[0]->num_sms;
  std::vector<int32_t> wbase(jobs.size() + 1, 0);
  for (size_t j = 0; j < jobs.size(); j++) {
    g->max_nb = std::max(g->max_nb, jobs[j]->db.max_nb);
    wbase[j + 1] = wbase[j] + (jobs[j]->db.n + 31) / 32;
  }
  const int nj = (int)jobs.size(), type = g->type;
  bool ok = dalloc(&g->d_jobs, jobs.size()) == cudaSuccess && dalloc(&g->d_hdr, jobs.size()) == cudaSuccess &&
            dalloc(&g->d_wbase, jobs.size() + 1) == cudaSuccess &&
            dalloc(&g->d_chunk_base, (size_t)kNumClasses * (jobs.size() + 1)) == cudaSuccess &&
            dalloc(&g->d_chunk_size, kNumClasses) == cudaSuccess && dalloc(&g->d_ctr, kNumClasses) == cudaSuccess &&
            dalloc(&g->d_done, 2) == cudaSuccess && cudaMemset(g->d_done, 0, 2 * sizeof(uint32_t)) == cudaSuccess;
  if (!ok) {
    group_close(g);
    return fail(NGIA_E_NOMEM, "pool: device allocation of the job tables failed");
  }
  if (configure(type, g->max_nb) != cudaSuccess) {
    group_close(g);
    return fail(NGIA_E_CUDA, "pool: kernel attributes");
  }
  // grids: the filter over the whole GPU; per bucket a persistent grid of the
  // resident CTAs of its kernel (the global-ring bucket at most 2 per SM)
  g->grid_filter = std::max(1, std::min(g->num_sms * 8, (wbase[nj] + 7) / 8));
  PoolDev &pd = g->pd;
  for (int k = 0; k < num_classes(type); k++) {
    const int ring = ring_of(type, k);
    g->smem[k] = align_smem(type, g->max_nb, ring);
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)align_fn(type, ring), kAlignThreads,
                                                      g->smem[k]) != cudaSuccess || occ < 1)
      occ = 1;
    if (ring == 0) occ = std::min(occ, 2);
    pd.grid_align[k] = g->num_sms * occ;
  }
  uint32_t rs = 1;
  while ((int)rs < g->max_nb) rs <<= 1;
  const int gcls = generic_class(type);
  pd.scratch_words = (int64_t)pd.grid_align[gcls] * kAlignThreads * rs;
  pd.ring_mask = rs - 1;
  if (dalloc(&g->d_scratch, (size_t)pd.scratch_words) != cudaSuccess) {
    group_close(g);
    return fail(NGIA_E_NOMEM, "pool: device allocation of the alignment ring failed");
  }
  for (int k = 0; k < num_classes(type); k++)
    if (cudaStreamCreateWithFlags(&g->side[k], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&g->join[k], cudaEventDisableTiming) != cudaSuccess) {
      group_close(g);
      return fail(NGIA_E_CUDA, "pool: streams");
    }
  if (cudaEventCreateWithFlags(&g->fork, cudaEventDisableTiming) != cudaSuccess) {
    group_close(g);
    return fail(NGIA_E_CUDA, "pool: events");
  }
  if (cudaMemcpy(g->d_wbase, wbase.data(), 4 * wbase.size(), cudaMemcpyHostToDevice) != cudaSuccess) {
    group_close(g);
    return fail(NGIA_E_CUDA, "pool: copy of the word prefix");
  }
  pd.jobs = g->d_jobs;
  pd.hdr = g->d_hdr;
  pd.wbase = g->d_wbase;
  pd.chunk_base = g->d_chunk_base;
  pd.chunk_size = g->d_chunk_size;
  pd.ctr = g->d_ctr;
  pd.done = g->d_done;
  pd.scratch = g->d_scratch;
  pd.n_jobs = nj;
  pd.type = type;
  pd.total_words = wbase[nj];
  *out = g;
  return NGIA_OK;
}

// Copies every job's current database view, run buffers and parameters into
// the device table (after ngia_cluster_begin of each job), on stream s.
int group_fill(Group *g, cudaStream_t s) {
  std::vector<PoolJob> h(g->jobs.size());
  for (size_t j = 0; j < g->jobs.size(); j++) {
    std::memset(&h[j], 0, sizeof(PoolJob));
    h[j].db = g->jobs[j]->db;
    h[j].rb = g->jobs[j]->rb;
    h[j].prm = g->jobs[j]->prm;
  }
  cudaError_t e = cudaMemcpyAsync(g->d_jobs, h.data(), sizeof(PoolJob) * h.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(g->d_done, 0, 2 * sizeof(uint32_t), s);  // completion counters
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "pool: table copy: %s", cudaGetErrorString(e));
  return NGIA_OK;
}

// Enqueues one round of the pool on the capturing stream s; the last kernel
// sets `cond` (the WHILE node's condition) while any job is still running.
int group_enqueue_round(Group *g, cudaStream_t s, cudaGraphConditionalHandle cond) {
  const PoolDev &pd = g->pd;
  const int nj = pd.n_jobs, type = g->type, nc = num_classes(type);
  k_pool_prep<<<nj, 512, 0, s>>>(pd);
  const size_t fsm = 4 * (size_t)(nj + 1);
  if (type == 0)
    k_pool_filter<2><<<g->grid_filter, 256, fsm, s>>>(pd, nc);
  else
    k_pool_filter<5><<<g->grid_filter, 256, fsm, s>>>(pd, nc);
  cudaError_t e = cudaEventRecord(g->fork, s);
  for (int k = 0; e == cudaSuccess && k < nc; k++) {
    e = cudaStreamWaitEvent(g->side[k], g->fork, 0);
    if (e != cudaSuccess) break;
    PoolDev a = pd;
    int cls = k, mnb = g->max_nb;
    void *args[] = {&a, &cls, &mnb};
    e = cudaLaunchKernel((const void *)align_fn(type, ring_of(type, k)), dim3(pd.grid_align[k]), dim3(kAlignThreads),
                         args, g->smem[k], g->side[k]);
    if (e == cudaSuccess) e = cudaEventRecord(g->join[k], g->side[k]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, g->join[k], 0);
  }
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "pool: alignment launches: %s", cudaGetErrorString(e));
  k_pool_next<<<nj, 1024, 0, s>>>(pd, cond);
  e = cudaGetLastError();
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "pool: launches: %s", cudaGetErrorString(e));
  return NGIA_OK;
}

int group_size(const Group *g) { return g ? (int)g->jobs.size() : 0; }

}  // namespace pool
}  // namespace ngia
