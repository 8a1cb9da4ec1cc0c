// spec.cu — speculative rounds of the greedy loop (NGIA_MODE_SPEC).
//
// The greedy loop takes one representative per iteration: the longest
// unclustered sequence, whose members (every unclustered sequence passing
// the composition, short-word and banded-LCS tests against it) leave the set
// (the reference's clustering(), CUDA/signalNode/src/func.cu:607-677).  Once
// the unclustered set is small, an iteration no longer fills the GPU: its
// time is the latency of its slowest pair.  A speculative round takes the
// next K unclustered sequences c_0 < ... < c_{K-1} (sorted order) as
// candidate representatives at once and runs every pair (c_i, x), x an
// unclustered sequence with x >= c_i, through the same three tests; each
// accepted pair sets bit i of x's mask and records its score.  The round then
// replays the greedy order exactly:
//   c_i is a representative  iff  no representative c_j, j < i, accepts it
//     (c_0 always is) — in the greedy loop c_i would have joined that c_j
//     before its own turn, and otherwise it is the longest sequence left
//     when its turn comes, since every c_j, j < i, has been taken or absorbed;
//   x joins the first representative of the round that accepts it, with
//     that pair's score — exactly the representative whose iteration would
//     have absorbed it.
// Sequences accepted by no representative of the round stay unclustered.  The
// per-pair tests are pure functions of the pair, except the reference's
// short-word kernel, whose thread leaves at its first job of net length < 16
// (the job list of one iteration decides which later pairs skip the test):
// with such records, the short-word test on (precise off) and more sequences
// than the reference's 16,384 threads, the driver runs the plain loop
// instead.  K is sized so that a round's pairs stay within
// a budget (a few waves of the alignment kernels); while the unclustered set
// is larger than that budget the plain one-representative iteration runs.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>

#include "../host/host_common.h"
#include "assign.cuh"
#include "ctx.h"

using ngia::fail;

namespace ngia {
namespace {

constexpr int kSpecMax = 64;              // candidate representatives per round (one mask bit each)
constexpr int kSpecBudget = 1 << 20;      // pairs per round at most (K x unclustered)
// Rounds start once the unclustered set is this small: a one-representative
// iteration over a larger set fills the GPU, and the round kernels (the
// representative taken per pair) run at about half the clustering kernels'
// cell rate (GB300, 1M DNA s=0.85: 7.3 ms for 1M pairs in the clustering
// kernel; a greedy iteration over 32k sequences is bounded by the latency of
// its slowest pair, 0.2-0.3 ms).
constexpr int kSpecMaxAlive = 1 << 15;
constexpr int kSpecRecheck = 8;  // graph iterations between looks at the unclustered set
constexpr int64_t kSpecScoreWords = 1ll << 26;  // K x n scores at most (256 MB)

struct SpecCtl {
  int32_t k;                // candidates of this round (0: none, or the set is above the budget)
  int32_t alive;            // unclustered sequences at the round's start
  unsigned long long valid;  // bit i: candidate i is a representative
  int32_t left;             // unclustered sequences after the round
  int32_t err;              // 1: an inconsistent mask (never expected)
  uint32_t prev[8];         // the previous round's queue counters (RoundBufs ctl)
};

struct SpecDev {
  int32_t *c;               // the candidates' sorted indices
  SpecCtl *ctl;
  int64_t *rs_off;          // record offsets of the candidates (the RepStore's off)
  uint32_t *lists;          // k-mer bitsets of the candidates
  uint32_t *eq;             // DNA match tables of the candidates
};

__device__ __forceinline__ int block_sum_1024(int v, int *s_red) {
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(kFullMask, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) s_red[threadIdx.x >> 5] = v;
  __syncthreads();
  int t = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += s_red[w];
  return t;
}

// Round start (one CTA of 1,024 threads): counts the unclustered set, sizes
// K, takes the first K unclustered sequences as candidates and gathers their
// record offsets; zeroes the round's queue counters.  Marks the run done when
// nothing is left.
__global__ void __launch_bounds__(1024) k_spec_pick(DevDB db, RunBufs run, SpecDev sd, RoundBufs rb, int k_max,
                                                    int budget, int max_alive) {
  __shared__ int s_red[32];
  __shared__ int s_k, s_found;
  RunState *st = run.st;
  const int nbw = (db.n + 31) / 32;
  const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
  if (tid < 8) {
    sd.ctl->prev[tid] = rb.ctl[tid];
    rb.ctl[tid] = 0;
  }
  int cnt = 0;
  for (int wi = tid; wi < nbw; wi += blockDim.x) cnt += __popc(run.alive[wi]);
  const int total = block_sum_1024(cnt, s_red);
  if (tid == 0) {
    int k = 0;
    const int64_t rem = st->iter_limit - st->iter;
    // at least two candidates per round (one is a plain iteration, which
    // the clustering kernels run faster)
    if (total > 0 && total <= max_alive && (int64_t)total * 2 <= budget && k_max >= 2 && !st->err && rem > 0) {
      k = min(k_max, budget / total);
      k = min(k, total);
      if (rem < k) k = (int)rem;
    }
    if (total == 0) st->done = 1;
    sd.ctl->k = k;
    sd.ctl->alive = total;
    sd.ctl->valid = 0;
    sd.ctl->left = 0;
    s_k = total > 0 ? max(k, 1) : 0;  // the first unclustered sequence is always found
    s_found = 0;
  }
  __syncthreads();
  const int k = s_k;
  if (k == 0) return;
  for (int base = 0; base < nbw; base += blockDim.x) {
    const int wi = base + tid;
    const uint32_t w = wi < nbw ? run.alive[wi] : 0u;
    const int c = __popc(w);
    int x = c;  // inclusive scan within the warp
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFullMask, x, o);
      if (lane >= o) x += y;
    }
    __syncthreads();
    if (lane == 31) s_red[wid] = x;
    __syncthreads();
    if (wid == 0) {  // inclusive scan of the warp totals
      int v = s_red[lane];
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(kFullMask, v, o);
        if (lane >= o) v += y;
      }
      s_red[lane] = v;
    }
    __syncthreads();
    int r = s_found + (wid ? s_red[wid - 1] : 0) + x - c;  // rank of this word's first unclustered sequence
    for (uint32_t m = w; m && r < k; m &= m - 1) sd.c[r++] = wi * 32 + __ffs(m) - 1;
    __syncthreads();
    if (tid == 0) s_found += s_red[31];
    __syncthreads();
    if (s_found >= k) break;
  }
  __syncthreads();
  for (int i = tid; i < k; i += blockDim.x) sd.rs_off[i] = db.off[sd.c[i]];
  // the plain iteration (and a checkpoint) take the representative from here
  if (tid == 0) st->rep = sd.c[0];
}

// Filter of a round: every unclustered x against every candidate c_i <= x —
// composition test, and the short-word test when it goes first — with the
// surviving (i, x) pairs queued by band-window class (warp-aggregated
// atomics, one per class and warp step).
template <int P>
__global__ void __launch_bounds__(256) k_spec_filter(DevDB db, RunBufs run, SpecDev sd, RoundBufs rb,
                                                      RunParams prm, int word_first, int list_words) {
  constexpr int A = P == 2 ? 4 : 28;
  __shared__ uint32_t s_rc[kSpecMax * A];
  __shared__ int s_c[kSpecMax], s_L1[kSpecMax], s_net1[kSpecMax], s_nb1[kSpecMax];
  __shared__ int s_k;
  if (threadIdx.x == 0) s_k = sd.ctl->k;
  __syncthreads();
  const int k = s_k;
  if (k == 0) return;
  for (int t = threadIdx.x; t < k * A; t += blockDim.x) s_rc[t] = db.words[sd.rs_off[t / A] + 2 + t % A];
  for (int i = threadIdx.x; i < k; i += blockDim.x) {
    const int c = sd.c[i];
    s_c[i] = c;
    s_L1[i] = db.len[c];
    s_net1[i] = db.net[c];
    s_nb1[i] = (db.net[c] + 31) / 32;
  }
  __syncthreads();
  const float s = prm.s;
  const int nbw = (db.n + 31) / 32;
  const int lane = threadIdx.x & 31;
  const int warps = gridDim.x * (blockDim.x >> 5);
  const bool word_here = word_first && !prm.precise;
  for (int wi = (s_c[0] >> 5) + blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); wi < nbw; wi += warps) {
    const uint32_t bits = run.alive[wi];
    if (!bits) continue;  // warp-uniform
    const int x = wi * 32 + lane;
    const bool here = (bits >> lane) & 1u;
    int L2 = 0, net2 = 0;
    const uint32_t *qpl = nullptr;
    if (here) {
      L2 = __ldg(db.len + x);
      net2 = __ldg(db.net + x);
      qpl = db.words + __ldg(db.off + x) + db.hw;
    }
    const int cut = here ? cutoff_of(L2, s) : 0;
    for (int i = 0; i < k; i++) {
      bool pass = here && x >= s_c[i];
      if (pass) pass = !(base_sum<A>(db.cnt, x, s_rc + i * A) < cut);
      if (pass && word_here && s_net1[i] >= 16 && net2 >= 16)
        pass = !(word_count<P>(qpl, net2, prm.w, sd.lists + (int64_t)i * list_words) < word_min(L2, prm.w, s));
      const int res = pass ? 1 + serve_class(window_of(band_blocks(s_L1[i], L2, s), s_nb1[i])) : 0;
      const unsigned pm = __ballot_sync(kFullMask, res != 0);
      if (res) {
        const unsigned peers = __match_any_sync(pm, res);
        const int leader = __ffs(peers) - 1;
        uint32_t b = 0;
        if (lane == leader) b = atomicAdd(&rb.ctl[res - 1], (uint32_t)__popc(peers));
        b = __shfl_sync(peers, b, leader);
        const int64_t slot = (int64_t)b + __popc(peers & ((1u << lane) - 1u));
        if (slot < rb.cap) rb.queue[res - 1][slot] = make_int2(i, x);
      }
    }
  }
}

// Which candidates are representatives (in order: c_i is one iff no earlier
// representative accepted it).
__global__ void k_spec_resolve(SpecDev sd, RoundBufs rb) {
  if (threadIdx.x != 0) return;
  const int k = sd.ctl->k;
  unsigned long long v = 0;
  for (int i = 0; i < k; i++) {
    const unsigned long long below = i ? (~0ull >> (64 - i)) : 0ull;
    if (!(rb.mask[sd.c[i]] & below & v)) v |= 1ull << i;
  }
  sd.ctl->valid = v;
}

// Applies a round: representatives, members with their scores, the
// unclustered set; clears the masks it read and counts what is left.
__global__ void __launch_bounds__(256) k_spec_assign(DevDB db, RunBufs run, SpecDev sd, RoundBufs rb) {
  __shared__ int s_c[kSpecMax];
  __shared__ int s_k;
  __shared__ unsigned long long s_v;
  if (threadIdx.x == 0) {
    s_k = sd.ctl->k;
    s_v = sd.ctl->valid;
  }
  __syncthreads();
  const int k = s_k;
  if (k == 0) return;
  for (int i = threadIdx.x; i < k; i += blockDim.x) s_c[i] = sd.c[i];
  __syncthreads();
  const unsigned long long v = s_v;
  const int last = s_c[k - 1];
  const int nbw = (db.n + 31) / 32;
  int left = 0, members = 0, bad = 0;
  for (int wi = (s_c[0] >> 5) + blockIdx.x * blockDim.x + threadIdx.x; wi < nbw; wi += gridDim.x * blockDim.x) {
    const uint32_t bits = run.alive[wi];
    uint32_t keep = bits;
    for (uint32_t m = bits; m; m &= m - 1) {
      const int x = wi * 32 + __ffs(m) - 1;
      const unsigned long long acc = rb.mask[x];
      int to = -1, id = -1;
      if (x <= last) {  // a candidate of this round (the first k unclustered)
        int i = 0;
        while (i < k && s_c[i] != x) i++;
        if (i == k) {
          bad = 1;
        } else if ((v >> i) & 1ull) {
          to = x;
          if ((acc >> i) & 1ull) {
            id = rb.score[(int64_t)i * rb.score_stride + x];
            members++;
          }
        } else {
          const int j = __ffsll((long long)(acc & v)) - 1;
          if (j < 0) {
            bad = 1;
          } else {
            to = s_c[j];
            id = rb.score[(int64_t)j * rb.score_stride + x];
            members++;
          }
        }
      } else if (acc & v) {
        const int j = __ffsll((long long)(acc & v)) - 1;
        to = s_c[j];
        id = rb.score[(int64_t)j * rb.score_stride + x];
        members++;
      }
      if (to >= 0) {
        run.cluster[x] = to;
        run.ident[x] = id;
        keep &= ~(1u << (x & 31));
      }
      if (acc) rb.mask[x] = 0ull;
    }
    if (keep != bits) run.alive[wi] = keep;
    left += __popc(keep);
  }
  for (int o = 16; o; o >>= 1) {
    left += __shfl_xor_sync(kFullMask, left, o);
    members += __shfl_xor_sync(kFullMask, members, o);
    bad |= __shfl_xor_sync(kFullMask, bad, o);
  }
  if ((threadIdx.x & 31) == 0) {
    if (left) atomicAdd(&sd.ctl->left, left);
    if (members) atomicAdd(&run.st->st_members, (unsigned long long)members);
    if (bad) atomicExch(&sd.ctl->err, 1);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) run.st->iter += __popcll(v);
}

}  // namespace
}  // namespace ngia

// Per-context state of the speculative driver (allocated on first use).
struct ngia_spec {
  int64_t cap_n = 0;
  int k_max = 0;
  int type = -1;
  ngia::SpecDev d{};
  ngia::RoundBufs rb{};
  ngia::RepStore rs{};
  unsigned char *h_ctl = nullptr;  // pinned: RoundBufs ctl (8 words) + SpecCtl
  unsigned char *d_ctl = nullptr;
  uint32_t *scratch = nullptr;
  int64_t scratch_words = 0;
  uint32_t ring_mask = 0;
  int64_t eq_stride = 0;      // words per candidate match table
  int grid[ngia::kServeClasses] = {0, 0, 0};
  int budget = ngia::kSpecBudget;  // pairs per round (NGIA_SPEC_BUDGET lowers it)
  int max_alive = ngia::kSpecMaxAlive;  // rounds once this few are unclustered (NGIA_SPEC_MAX_ALIVE)
  bool big = false;           // the unclustered set was above the round budget at the last check
};

namespace ngia {
namespace drv {

namespace {

#define CKP(call)                                                                              \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return fail(NGIA_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

template <class T>
cudaError_t dmalloc(T **p, size_t count) {
  return cudaMalloc((void **)p, sizeof(T) * (count ? count : 1));
}

constexpr size_t kCtlBytes = 8 * sizeof(uint32_t) + sizeof(SpecCtl);

int spec_alloc(ngia_ctx *c) {
  ngia_spec *sp = c->spec;
  const int64_t n = std::max<int64_t>(c->cap_n, c->db.n);
  const int64_t eq_stride = (int64_t)eq_words(std::max(c->cap_nb, c->db.max_nb));
  if (sp && sp->cap_n >= n && sp->type == c->db.type && sp->ring_mask == c->rb.ring_mask &&
      sp->eq_stride >= eq_stride)
    return NGIA_OK;
  spec_free(c);
  sp = new (std::nothrow) ngia_spec();
  if (!sp) return fail(NGIA_E_NOMEM, "spec: out of host memory");
  c->spec = sp;
  sp->cap_n = n;
  sp->type = c->db.type;
  sp->k_max = (int)std::max<int64_t>(1, std::min<int64_t>(kSpecMax, kSpecScoreWords / std::max<int64_t>(1, n)));
  sp->ring_mask = c->rb.ring_mask;
  sp->eq_stride = eq_stride;
  const int lw = kListWords;
  if (dmalloc(&sp->d.c, kSpecMax) != cudaSuccess || dmalloc(&sp->d.rs_off, kSpecMax) != cudaSuccess ||
      dmalloc(&sp->d.lists, (size_t)kSpecMax * lw) != cudaSuccess || dmalloc(&sp->d_ctl, kCtlBytes) != cudaSuccess ||
      dmalloc(&sp->d.eq, (size_t)kSpecMax * (size_t)eq_stride) != cudaSuccess ||
      cudaMallocHost((void **)&sp->h_ctl, kCtlBytes) != cudaSuccess ||
      dmalloc(&sp->rb.mask, (size_t)n) != cudaSuccess ||
      dmalloc(&sp->rb.score, (size_t)sp->k_max * (size_t)n) != cudaSuccess ||
      dmalloc(&sp->rb.stats, 2) != cudaSuccess)
    return fail(NGIA_E_NOMEM, "spec: device allocation failed");
  for (auto *&q : sp->rb.queue)
    if (dmalloc(&q, (size_t)kSpecBudget) != cudaSuccess) return fail(NGIA_E_NOMEM, "spec: queue allocation failed");
  sp->rb.ctl = reinterpret_cast<uint32_t *>(sp->d_ctl);
  sp->d.ctl = reinterpret_cast<SpecCtl *>(sp->d_ctl + 8 * sizeof(uint32_t));
  sp->rb.cap = kSpecBudget;
  sp->rb.score_stride = n;
  sp->rb.key = nullptr;
  sp->rb.todo = nullptr;
  static std::mutex mu;
  {
    std::lock_guard<std::mutex> lock(mu);
    for (int k = 0; k < kServeClasses; k++) {
      const void *fn = (const void *)serve_align_fn<true>(sp->type, k);
      const size_t smem = serve_align_smem(sp->type, k, sp->eq_stride);
      CKP(serve_align_configure<true>(sp->type, k, smem));
      int occ = 0;
      if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, kAlignThreads, smem) != cudaSuccess ||
          occ < 1)
        occ = 1;
      sp->grid[k] = c->num_sms * occ;
    }
  }
  sp->scratch_words = (int64_t)sp->grid[2] * kAlignThreads * (sp->ring_mask + 1);
  if (dmalloc(&sp->scratch, (size_t)sp->scratch_words) != cudaSuccess)
    return fail(NGIA_E_NOMEM, "spec: scratch allocation failed");
  return NGIA_OK;
}

// Launches one round after k_spec_pick: k-mer lists, filter, the three
// alignment classes (mask form), resolve, assign; then the next round's pick.
int spec_launch_round(ngia_ctx *c, bool lists) {
  ngia_spec *sp = c->spec;
  cudaStream_t st = c->stream;
  const int P = c->db.type ? 5 : 2;
  const int lw = (int)std::max<uint32_t>(1u, (1u << (c->prm.w * (P == 2 ? 2 : 5))) / 32u);
  RepStore rs{c->db.words, sp->d.rs_off, nullptr, nullptr,     nullptr, sp->d.lists,
              kSpecMax,    lw,           &sp->d.ctl->k, sp->d.eq, sp->eq_stride};
  if (P == 2) {
    k_rep_eq<<<sp->k_max, 256, 0, st>>>(rs, sp->d.eq);
    CKP(cudaGetLastError());
  }
  if (lists) {
    if (P == 2)
      k_rep_lists<2><<<sp->k_max, 256, 0, st>>>(rs, c->prm.w, sp->d.lists);
    else
      k_rep_lists<5><<<sp->k_max, 256, 0, st>>>(rs, c->prm.w, sp->d.lists);
    CKP(cudaGetLastError());
  }
  const int word_first = word_first_of(c->db.type, c->prm);
  const int fgrid = c->num_sms * 8;
  if (P == 2)
    k_spec_filter<2><<<fgrid, 256, 0, st>>>(c->db, c->rb, sp->d, sp->rb, c->prm, word_first, lw);
  else
    k_spec_filter<5><<<fgrid, 256, 0, st>>>(c->db, c->rb, sp->d, sp->rb, c->prm, word_first, lw);
  CKP(cudaGetLastError());
  const int word_after = !word_first && !c->prm.precise;
  for (int k = 0; k < kServeClasses; k++) {
    DevDB db = c->db;
    RunParams prm = c->prm;
    RoundBufs rb = sp->rb;
    int cls = k, wa = word_after;
    uint32_t *scr = sp->scratch;
    int64_t sw = sp->scratch_words;
    uint32_t rm = sp->ring_mask;
    void *args[] = {&db, &rs, &prm, &rb, &cls, &wa, &scr, &sw, &rm};
    CKP(cudaLaunchKernel((const void *)serve_align_fn<true>(c->db.type, k), dim3(sp->grid[k]), dim3(kAlignThreads),
                         args, serve_align_smem(c->db.type, k, sp->eq_stride), st));
  }
  k_spec_resolve<<<1, 32, 0, st>>>(sp->d, sp->rb);
  CKP(cudaGetLastError());
  k_spec_assign<<<c->num_sms * 4, 256, 0, st>>>(c->db, c->rb, sp->d, sp->rb);
  CKP(cudaGetLastError());
  k_spec_pick<<<1, 1024, 0, st>>>(c->db, c->rb, sp->d, sp->rb, sp->k_max, sp->budget, sp->max_alive);
  CKP(cudaGetLastError());
  return NGIA_OK;
}

int spec_read(ngia_ctx *c) {
  ngia_spec *sp = c->spec;
  CKP(cudaMemcpyAsync(sp->h_ctl, sp->d_ctl, kCtlBytes, cudaMemcpyDeviceToHost, c->stream));
  return pull_state(c);  // synchronises the stream
}

}  // namespace

// With at most kRefGridThreads sequences every thread of the reference's
// short-word kernel holds at most one job, so its early return only leaves
// the short job itself untested — the pairwise rule of the round kernels.
bool spec_exact(const ngia_ctx *c) {
  return !c->db.has_short || c->prm.precise || c->db.n <= kRefGridThreads;
}

int spec_prepare(ngia_ctx *c) {
  int rc = spec_alloc(c);
  if (rc) return rc;
  ngia_spec *sp = c->spec;
  CKP(cudaMemsetAsync(sp->rb.mask, 0, sizeof(unsigned long long) * (size_t)c->db.n, c->stream));
  CKP(cudaMemsetAsync(sp->rb.stats, 0, 2 * sizeof(unsigned long long), c->stream));
  CKP(cudaMemsetAsync(sp->d_ctl, 0, kCtlBytes, c->stream));
  sp->big = false;
  sp->budget = kSpecBudget;
  if (const char *b = getenv("NGIA_SPEC_BUDGET")) sp->budget = std::max(1, std::min(kSpecBudget, atoi(b)));
  sp->max_alive = kSpecMaxAlive;
  if (const char *m = getenv("NGIA_SPEC_MAX_ALIVE")) sp->max_alive = std::max(2, atoi(m));
  return NGIA_OK;
}

void spec_free(ngia_ctx *c) {
  ngia_spec *sp = c->spec;
  if (!sp) return;
  cudaFree(sp->d.c);
  cudaFree(sp->d.rs_off);
  cudaFree(sp->d.lists);
  cudaFree(sp->d.eq);
  cudaFree(sp->d_ctl);
  if (sp->h_ctl) cudaFreeHost(sp->h_ctl);
  cudaFree(sp->rb.mask);
  cudaFree(sp->rb.score);
  cudaFree(sp->rb.stats);
  for (auto *q : sp->rb.queue) cudaFree(q);
  cudaFree(sp->scratch);
  delete sp;
  c->spec = nullptr;
}

// Runs up to max_iters representatives (all, for max_iters <= 0): plain
// iterations while the unclustered set is above the round budget (or when the
// rounds would not be exact), speculative rounds after that.
int spec_step(ngia_ctx *c, int64_t max_iters) {
  ngia_spec *sp = c->spec;
  if (!sp) return fail(NGIA_E_STATE, "spec: driver not prepared");
  const int64_t it0 = c->h_state->iter;
  const int64_t limit = max_iters > 0 ? it0 + max_iters : LLONG_MAX;
  c->h_state->iter_limit = limit;
  CKP(cudaMemcpyAsync(&c->rb.st->iter_limit, &c->h_state->iter_limit, sizeof(int64_t), cudaMemcpyHostToDevice,
                      c->stream));
  const bool exact = spec_exact(c);
  const bool lists = !c->prm.precise;
  bool picked = false;  // a pick for the next round is in flight
  for (int64_t guard = 0; !c->h_state->done && c->h_state->iter < limit; guard++) {
    if (guard > 2 * (int64_t)c->db.n + 8)
      return fail(NGIA_E_STATE, "spec: more steps than sequences");
    if (!exact || sp->big) {
      // one-representative iterations in the captured loop: the rest of the
      // step when rounds would not be exact, else a few before the next look
      // at the unclustered set
      const int64_t room = limit - c->h_state->iter;
      const int64_t n_it = exact ? std::min<int64_t>(room, kSpecRecheck) : room;
      // captured on first use (databases that start below the threshold,
      // such as serving leftovers, never need it)
      int rc0 = ensure_graph(c);
      if (rc0) return rc0;
      c->h_state->iter_limit = c->h_state->iter + n_it;
      CKP(cudaMemcpyAsync(&c->rb.st->iter_limit, &c->h_state->iter_limit, sizeof(int64_t), cudaMemcpyHostToDevice,
                          c->stream));
      CKP(cudaGraphLaunch(c->graph_exec, c->stream));
      int rc = pull_state(c);
      if (rc) return rc;
      c->h_state->iter_limit = limit;  // the rounds' own limit again
      CKP(cudaMemcpyAsync(&c->rb.st->iter_limit, &c->h_state->iter_limit, sizeof(int64_t), cudaMemcpyHostToDevice,
                          c->stream));
      picked = false;
      if (exact) sp->big = false;  // look at the unclustered set again
      continue;
    }
    if (!picked) {
      k_spec_pick<<<1, 1024, 0, c->stream>>>(c->db, c->rb, sp->d, sp->rb, sp->k_max, sp->budget, sp->max_alive);
      CKP(cudaGetLastError());
      int rc = spec_read(c);
      if (rc) return rc;
      picked = true;
    }
    const SpecCtl *ctl = reinterpret_cast<const SpecCtl *>(sp->h_ctl + 8 * sizeof(uint32_t));
    if (ctl->k == 0) {
      picked = false;
      if (ctl->alive == 0 || c->h_state->done) break;
      if (c->h_state->iter >= limit || c->h_state->err) break;
      sp->big = true;  // above the budget: plain iterations for a while
      continue;
    }
    int rc = spec_launch_round(c, lists);
    if (rc) return rc;
    rc = spec_read(c);  // this round applied, the next one picked
    if (rc) return rc;
    const uint32_t *qc = ctl->prev;  // this round's queue counters
    if (qc[7]) return fail(NGIA_E_DEVICE, "spec: alignment loop bound exceeded");
    if (qc[0] > sp->rb.cap || qc[1] > sp->rb.cap || qc[2] > sp->rb.cap)
      return fail(NGIA_E_LIMIT, "spec: a round queued more pairs than its budget");
    if (ctl->err) return fail(NGIA_E_DEVICE, "spec: inconsistent acceptance masks");
  }
  return NGIA_OK;
}

void spec_stats(const ngia_ctx *c, int64_t *pairs, int64_t *cells) {
  *pairs = *cells = 0;
  if (!c->spec) return;
  unsigned long long h[2] = {0, 0};
  if (cudaMemcpy(h, c->spec->rb.stats, sizeof(h), cudaMemcpyDeviceToHost) == cudaSuccess) {
    *pairs = (int64_t)h[0];
    *cells = (int64_t)h[1];
  }
}

}  // namespace drv
}  // namespace ngia
