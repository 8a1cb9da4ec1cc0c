// serve.cu — continuous-batching service: query batches are assigned to a
// resident representative set, then each batch's leftovers are clustered
// among themselves.  The reference has no serving mode; the per-pair tests
// are its own (composition, func.cu:323-354; short words, 357-447; banded
// LCS, 450-604), applied with the representative in the reference role.
//
// Resident state (ngia_serve_open): the representatives as a device
// database (records and header arrays, loaded by the same loader as
// ngia_open) plus one k-mer bitset and, for DNA, one match table per
// representative, built on the device.  The per-pair kernels are shared with
// the speculative rounds (assign.cuh).
//
// One batch runs on one slot — a context of fixed capacity with its own
// stream, driven by its own host thread:
//  1. assignment, in rounds over chunks of representatives in creation order
//     (64, 128, ... doubling up to 1,024): k_serve_filter tests every unassigned
//     query against every representative of the chunk (composition, and the
//     short-word test when it goes first) and queues the surviving pairs by
//     band-window width; k_serve_align runs the banded LCS of each pair with
//     the tiled register update (tile.cuh, lanes in lockstep) and keeps per
//     query the smallest accepting representative with its score (one 64-bit
//     atomicMin of rep << 32 | score); k_serve_round_end drops assigned
//     queries and counts the rest.  A later round only holds later
//     representatives, so a query assigned in a round is final and the
//     rounds stop once no query is left (or the set is exhausted);
//  2. the leftovers are clustered by the greedy driver over the batch's
//     database restricted to them (begin_subset), which equals clustering a
//     database of only the leftovers — by default with the speculative
//     rounds (spec.cu).
// Slots run side by side on the GPU; a batch waits in a FIFO until a slot is
// free.  The number of slots is capped by the memory budget.
#include <algorithm>
#include <chrono>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../host/host_common.h"
#include "ctx.h"
#include "kmer.cuh"
#include "assign.cuh"
#include "tile.cuh"

using ngia::fail;

namespace ngia {
namespace {

constexpr int kFirstChunk = 64;     // representatives in the first round
constexpr int kMaxChunk = 1024;     // ... doubling up to this many per round

__global__ void k_serve_init(int n, RoundBufs rb) {
  const int nbw = (n + 31) / 32;
  if (blockIdx.x == 0 && threadIdx.x < 2) rb.stats[threadIdx.x] = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) rb.key[i] = kNoRep;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nbw; i += gridDim.x * blockDim.x) {
    const int rem = n - i * 32;
    rb.todo[i] = rem >= 32 ? 0xFFFFFFFFu : ((1u << rem) - 1u);
  }
}

// Drops the queries assigned in this round from the unassigned set and
// counts the rest.
__global__ void k_serve_round_end(int n, RoundBufs rb) {
  const int nbw = (n + 31) / 32;
  uint32_t left = 0;
  for (int wi = blockIdx.x * blockDim.x + threadIdx.x; wi < nbw; wi += gridDim.x * blockDim.x) {
    uint32_t bits = rb.todo[wi];
    for (uint32_t m = bits; m; m &= m - 1) {
      const int q = wi * 32 + __ffs(m) - 1;
      if (rb.key[q] != kNoRep) bits &= ~(1u << (q & 31));
    }
    rb.todo[wi] = bits;
    left += __popc(bits);
  }
  for (int o = 16; o; o >>= 1) left += __shfl_xor_sync(kFullMask, left, o);
  if ((threadIdx.x & 31) == 0 && left) atomicAdd(&rb.ctl[6], left);
}

// NGIA_SERVE_TRACE=1 prints the phases of every batch to stderr.
bool trace() {
  static const bool on = [] {
    const char *t = getenv("NGIA_SERVE_TRACE");
    return t && *t && *t != '0';
  }();
  return on;
}

// Driver of the leftover clustering (NGIA_SERVE_LEFTOVERS=spec|plain|graph).
// The speculative rounds are the default: a batch's leftovers are a few
// hundred to a few thousand sequences, far from filling the GPU one
// representative at a time, so a round takes up to 64 representatives at
// once.  The graph form would be captured and instantiated per batch (a
// slot's database changes with every batch); with several slots doing that
// at once it served 2.2x fewer queries per second than the plain host loop
// on GB300 (200 batches of the serving workload, 8 slots).
int leftover_mode() {
  static const int m = [] {
    const char *t = getenv("NGIA_SERVE_LEFTOVERS");
    if (t && std::strcmp(t, "graph") == 0) return NGIA_MODE_GRAPH;
    if (t && std::strcmp(t, "plain") == 0) return NGIA_MODE_PLAIN;
    return NGIA_MODE_SPEC;
  }();
  return m;
}

double now_ms() {
  return std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
  int64_t ticket = 0;
  std::vector<uint32_t> words;
  std::vector<int64_t> off;
  int32_t n = 0, longest = 0;
  std::vector<int32_t> rep, ident;
  int status = 0;  // 0 waiting or running, 1 done, < 0 error code
  std::string error;
  double t_submit = 0, t_start = 0, t_done = 0;
  int slot = -1, rounds = 0, resident = 0, new_reps = 0;
  int64_t pairs = 0, cells = 0;
};

}  // namespace
}  // namespace ngia

struct ngia_server;

namespace ngia {
namespace {

struct Slot {
  int index = 0;
  ngia_ctx *ctx = nullptr;
  RoundBufs rb{};
  uint32_t *h_ctl = nullptr;                  // pinned
  unsigned long long *h_key = nullptr;        // pinned, cap_n
  unsigned long long *h_stats = nullptr;      // pinned, 2
  uint32_t *scratch = nullptr;
  int64_t scratch_words = 0;
  int grid[kServeClasses] = {0, 0, 0};
  std::vector<int32_t> cl, id;
  std::thread worker;
};

}  // namespace
}  // namespace ngia

struct ngia_server {
  int device = 0, type = 0, num_sms = 0;
  ngia_params params{};
  ngia::RunParams prm{};
  int word_first = 0;
  ngia_ctx *reps = nullptr;  // the resident representatives' database
  uint32_t *d_lists = nullptr;
  uint32_t *d_eq = nullptr;  // DNA match tables of the representatives
  ngia::RepStore store{};
  int64_t cap_n = 0, cap_words = 0;
  int32_t cap_nb = 0;
  uint32_t ring_mask = 0;
  std::vector<std::unique_ptr<ngia::Slot>> slots;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<ngia::Request *> fifo;
  std::unordered_map<int64_t, std::unique_ptr<ngia::Request>> requests;
  int64_t next_ticket = 1;
  bool stop = false;
};

namespace ngia {
namespace {

#define CKS(call)                                                                              \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return fail(NGIA_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
  } while (0)

// One batch on one slot.  Returns a status; results land in rq.
int run_batch(ngia_server *sv, Slot &sl, Request &rq) {
  ngia_db_view v{};
  v.n = rq.n;
  v.type = sv->type;
  v.longest = rq.longest;
  v.words = rq.words.data();
  v.n_words = (int64_t)rq.words.size();
  v.rec_off = rq.off.data();
  ngia_ctx *c = sl.ctx;
  if (trace()) fprintf(stderr, "[serve] slot %d ticket %lld start n=%d\n", sl.index, (long long)rq.ticket, rq.n);
  int rc = drv::reload_ctx(c, &v);
  if (rc) return rc;
  const int n = rq.n, nbw = (n + 31) / 32;
  cudaStream_t st = c->stream;
  RoundBufs rb = sl.rb;
  k_serve_init<<<std::max(1, std::min(c->num_sms, (n + 255) / 256)), 256, 0, st>>>(n, rb);
  CKS(cudaGetLastError());
  const int word_after = !sv->word_first && !sv->prm.precise;
  // largest round (NGIA_SERVE_MAX_CHUNK, at most kMaxChunk, which sizes the
  // slot's pair queues): a query accepted by a representative of a round can
  // still have its pairs with the round's later representatives aligned.
  // Swept on GB300 (200 DNA query batches, 14,077 representatives): 1,024,
  // 512, 256 and 128 aligned 300.2M, 299.3M, 298.5M and 298.0M pairs at
  // 53.1k, 53.0k, 52.3k and 51.3k queries/s: nearly every pair is one the
  // first-match rule needs.
  static const int max_chunk = [] {
    const char *m = getenv("NGIA_SERVE_MAX_CHUNK");
    return m ? std::max(kFirstChunk, std::min(kMaxChunk, atoi(m))) : kMaxChunk;
  }();
  int r0 = 0, chunk = std::min(kFirstChunk, max_chunk);
  uint32_t left = (uint32_t)n;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  if (trace())
    for (auto &e : ev) cudaEventCreate(&e);
  while (r0 < sv->store.n && left > 0) {
    const int nr = std::min(chunk, sv->store.n - r0);
    CKS(cudaMemsetAsync(rb.ctl, 0, 8 * sizeof(uint32_t), st));
    if (ev[0]) cudaEventRecord(ev[0], st);
    if (sv->type == 0)
      k_serve_filter<2><<<nr, 256, (size_t)nbw * 32, st>>>(c->db, sv->store, sv->prm, rb, r0, sv->word_first);
    else
      k_serve_filter<5><<<nr, 256, (size_t)nbw * 32, st>>>(c->db, sv->store, sv->prm, rb, r0, sv->word_first);
    CKS(cudaGetLastError());
    if (ev[1]) cudaEventRecord(ev[1], st);
    for (int k = 0; k < kServeClasses; k++) {
      AlignServeFn fn = serve_align_fn<false>(sv->type, k);
      DevDB db = c->db;
      RepStore rs = sv->store;
      RunParams prm = sv->prm;
      int cls = k, wa = word_after;
      uint32_t *scr = sl.scratch;
      int64_t sw = sl.scratch_words;
      uint32_t rm = sv->ring_mask;
      void *args[] = {&db, &rs, &prm, &rb, &cls, &wa, &scr, &sw, &rm};
      CKS(cudaLaunchKernel((const void *)fn, dim3(sl.grid[k]), dim3(kAlignThreads), args,
                           serve_align_smem(sv->type, k, sv->store.eq_stride), st));
    }
    if (ev[2]) cudaEventRecord(ev[2], st);
    k_serve_round_end<<<std::max(1, std::min(c->num_sms, (nbw + 255) / 256)), 256, 0, st>>>(n, rb);
    CKS(cudaGetLastError());
    if (ev[3]) cudaEventRecord(ev[3], st);
    CKS(cudaMemcpyAsync(sl.h_ctl, rb.ctl, 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, st));
    CKS(cudaStreamSynchronize(st));
    if (sl.h_ctl[7]) return fail(NGIA_E_DEVICE, "serve: alignment loop bound exceeded (round at rep %d)", r0);
    if (sl.h_ctl[0] > rb.cap || sl.h_ctl[1] > rb.cap || sl.h_ctl[2] > rb.cap)
      return fail(NGIA_E_LIMIT, "serve: %u pairs in one round exceed the queue capacity", sl.h_ctl[0]);
    left = sl.h_ctl[6];
    if (trace()) {
      float f = 0, a = 0, e = 0;
      cudaEventElapsedTime(&f, ev[0], ev[1]);
      cudaEventElapsedTime(&a, ev[1], ev[2]);
      cudaEventElapsedTime(&e, ev[2], ev[3]);
      fprintf(stderr,
              "[serve] slot %d ticket %lld round %d reps %d..%d pairs %u/%u/%u left %u  filter %.3f align %.3f end "
              "%.3f ms\n",
              sl.index, (long long)rq.ticket, rq.rounds, r0, r0 + nr - 1, sl.h_ctl[0], sl.h_ctl[1], sl.h_ctl[2], left,
              f, a, e);
    }
    r0 += nr;
    chunk = std::min(chunk * 2, max_chunk);
    rq.rounds++;
  }
  for (auto &e : ev)
    if (e) cudaEventDestroy(e);
  CKS(cudaMemcpyAsync(sl.h_key, rb.key, sizeof(unsigned long long) * (size_t)n, cudaMemcpyDeviceToHost, st));
  CKS(cudaMemcpyAsync(sl.h_stats, rb.stats, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st));
  CKS(cudaStreamSynchronize(st));
  rq.pairs = (int64_t)sl.h_stats[0];
  rq.cells = (int64_t)sl.h_stats[1];
  rq.rep.assign(n, 0);
  rq.ident.assign(n, -1);
  if (trace()) fprintf(stderr, "[serve] slot %d ticket %lld leftovers %u\n", sl.index, (long long)rq.ticket, left);
  if (left > 0) {  // greedy clustering of the leftovers
    const double t0 = now_ms();
    const int mode = leftover_mode();
    rc = drv::begin_subset(c, &sv->params, mode, rb.todo);
    if (rc) return rc;
    const double t1 = now_ms();
    int32_t done = 0;
    rc = ngia_cluster_step(c, 0, &done);
    if (rc) return rc;
    sl.cl.resize(n);
    sl.id.resize(n);
    ngia_stats gst;
    rc = ngia_cluster_end(c, sl.cl.data(), sl.id.data(), &gst);
    if (rc) return rc;
    if (trace())
      fprintf(stderr, "[serve] slot %d ticket %lld greedy %s: %lld iterations, begin %.2f ms, loop %.2f ms\n",
              sl.index, (long long)rq.ticket,
              mode == NGIA_MODE_GRAPH ? "graph" : mode == NGIA_MODE_SPEC ? "spec" : "plain", (long long)gst.iterations,
              t1 - t0, now_ms() - t1);
  }
  rq.resident = 0;
  rq.new_reps = 0;
  for (int q = 0; q < n; q++) {
    const unsigned long long k = sl.h_key[q];
    if (k != kNoRep) {
      rq.rep[q] = (int32_t)(k >> 32);
      rq.ident[q] = (int32_t)(uint32_t)k;
      rq.resident++;
    } else {
      rq.rep[q] = -1 - sl.cl[q];
      rq.ident[q] = sl.id[q];
      if (sl.cl[q] == q) rq.new_reps++;
    }
  }
  return NGIA_OK;
}

void worker_main(ngia_server *sv, Slot *sl) {
  cudaSetDevice(sv->device);
  for (;;) {
    Request *rq = nullptr;
    {
      std::unique_lock<std::mutex> lk(sv->mu);
      sv->cv_work.wait(lk, [&] { return sv->stop || !sv->fifo.empty(); });
      if (sv->fifo.empty()) return;  // stopping and nothing left
      rq = sv->fifo.front();
      sv->fifo.pop_front();
      rq->t_start = now_ms();
      rq->slot = sl->index;
    }
    ngia::clear_error();
    const int rc = run_batch(sv, *sl, *rq);
    std::string msg;
    if (rc) {
      char buf[512];
      ngia_last_error(buf, sizeof(buf));
      msg = buf;
    }
    {
      std::lock_guard<std::mutex> lk(sv->mu);
      rq->t_done = now_ms();
      rq->status = rc ? rc : 1;
      rq->error = msg;
    }
    sv->cv_done.notify_all();
  }
}

void free_slot(Slot &sl) {
  if (sl.ctx) ngia_close(sl.ctx);
  for (auto *q : sl.rb.queue) cudaFree(q);
  cudaFree(sl.rb.ctl);
  cudaFree(sl.rb.key);
  cudaFree(sl.rb.todo);
  cudaFree(sl.rb.stats);
  if (sl.h_stats) cudaFreeHost(sl.h_stats);
  cudaFree(sl.scratch);
  if (sl.h_ctl) cudaFreeHost(sl.h_ctl);
  if (sl.h_key) cudaFreeHost(sl.h_key);
  sl = Slot{};
}

// Device bytes of one slot (context, round buffers, scratch).
int64_t slot_bytes(const ngia_server *sv, int grid2) {
  const int A = sv->type ? 28 : 4;
  const int64_t ctx = 4 * sv->cap_words + sv->cap_n * (8 + 4 + 4 + 4 * A) +
                      sv->cap_n * (4 + 4 + 4 * ngia::kNumClasses) + (int64_t)sv->cap_n / 8 * 3;
  const int64_t rounds = (int64_t)kServeClasses * kMaxChunk * sv->cap_n * 8 + sv->cap_n * 8 + sv->cap_n / 8;
  const int64_t scratch = (int64_t)grid2 * kAlignThreads * (sv->ring_mask + 1) * 4;
  // speculative leftover rounds: masks, up to 64 scores per record, pair
  // queues of 2^20 pairs per class, their own global ring
  const int64_t spec = sv->cap_n * (8 + 64 * 4) + (int64_t)kServeClasses * (1 << 20) * 8 + scratch;
  return ctx + rounds + scratch + spec + (16 << 20);
}

int open_slot(ngia_server *sv, Slot &sl, int index) {
  sl.index = index;
  int rc = drv::open_ctx_capacity(sv->type, sv->cap_n, sv->cap_words, sv->cap_nb, &sl.ctx);
  if (rc) return rc;
  const int64_t cap = (int64_t)kMaxChunk * sv->cap_n;
  for (auto *&q : sl.rb.queue)
    if (cudaMalloc((void **)&q, sizeof(int2) * (size_t)cap) != cudaSuccess)
      return fail(NGIA_E_NOMEM, "serve: queue allocation failed");
  if (cudaMalloc((void **)&sl.rb.ctl, 8 * sizeof(uint32_t)) != cudaSuccess ||
      cudaMalloc((void **)&sl.rb.key, sizeof(unsigned long long) * (size_t)sv->cap_n) != cudaSuccess ||
      cudaMalloc((void **)&sl.rb.todo, 4 * (size_t)((sv->cap_n + 31) / 32)) != cudaSuccess ||
      cudaMallocHost((void **)&sl.h_ctl, 8 * sizeof(uint32_t)) != cudaSuccess ||
      cudaMallocHost((void **)&sl.h_key, sizeof(unsigned long long) * (size_t)sv->cap_n) != cudaSuccess ||
      cudaMalloc((void **)&sl.rb.stats, 2 * sizeof(unsigned long long)) != cudaSuccess ||
      cudaMallocHost((void **)&sl.h_stats, 2 * sizeof(unsigned long long)) != cudaSuccess)
    return fail(NGIA_E_NOMEM, "serve: slot allocation failed");
  sl.rb.cap = cap;
  for (int k = 0; k < kServeClasses; k++) {
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, (const void *)serve_align_fn<false>(sv->type, k), kAlignThreads,
                                                      serve_align_smem(sv->type, k, sv->store.eq_stride)) != cudaSuccess ||
        occ < 1)
      occ = 1;
    sl.grid[k] = sv->num_sms * occ;
  }
  sl.scratch_words = (int64_t)sl.grid[2] * kAlignThreads * (sv->ring_mask + 1);
  if (cudaMalloc((void **)&sl.scratch, 4 * (size_t)sl.scratch_words) != cudaSuccess)
    return fail(NGIA_E_NOMEM, "serve: scratch allocation failed");
  if (leftover_mode() == NGIA_MODE_SPEC) {  // the leftover driver's buffers, before any request
    rc = drv::spec_prepare(sl.ctx);
    if (rc) return rc;
  }
  return NGIA_OK;
}

void destroy(ngia_server *sv) {
  {
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->stop = true;
  }
  sv->cv_work.notify_all();
  for (auto &sl : sv->slots)
    if (sl->worker.joinable()) sl->worker.join();
  for (auto &sl : sv->slots) free_slot(*sl);
  if (sv->reps) ngia_close(sv->reps);
  cudaFree(sv->d_lists);
  cudaFree(sv->d_eq);
  delete sv;
}

// Largest plane-block count of the records of a host view.
int view_max_blocks(const ngia_db_view *v) {
  int nb = 0;
  for (int32_t i = 0; i < v->n; i++) {
    const int64_t o = v->rec_off[i];
    if (o < 0 || o + 2 > v->n_words) return INT_MAX;
    nb = std::max(nb, (int)((v->words[o + 1] + 31) / 32));
  }
  return nb;
}

}  // namespace
}  // namespace ngia

extern "C" int ngia_serve_open(const ngia_db_view *reps, const ngia_params *params, const ngia_serve_config *cfg,
                               ngia_server **out) {
  ngia::clear_error();
  if (!reps || !params || !out) return fail(NGIA_E_ARG, "ngia_serve_open: null argument");
  *out = nullptr;
  int rc = ngia::drv::validate_params(reps->type, params);
  if (rc) return rc;
  ngia_serve_config cf = cfg ? *cfg : ngia_serve_config{};
  if (cf.slots <= 0) cf.slots = 4;
  if (cf.max_batch <= 0) cf.max_batch = 4096;
  if (cf.max_record_blocks <= 0) cf.max_record_blocks = 128;
  if (cf.max_record_blocks > ngia::kMaxBlocks)
    return fail(NGIA_E_LIMIT, "ngia_serve_open: records of more than %d blocks", ngia::kMaxBlocks);
  const int hw = reps->type ? 30 : 6, P = reps->type ? 5 : 2;
  if (cf.max_batch_words <= 0) cf.max_batch_words = (int64_t)cf.max_batch * (hw + P * cf.max_record_blocks);
  ngia_server *sv = new (std::nothrow) ngia_server();
  if (!sv) return fail(NGIA_E_NOMEM, "ngia_serve_open: out of host memory");
  cudaGetDevice(&sv->device);
  cudaDeviceGetAttribute(&sv->num_sms, cudaDevAttrMultiProcessorCount, sv->device);
  sv->type = reps->type;
  sv->params = *params;
  sv->prm.s = params->similarity;
  sv->prm.w = params->word_length;
  sv->prm.precise = params->precise;
  sv->prm.word_order = 0;
  if (const char *wo = getenv("NGIA_SERVE_WORD_ORDER")) sv->prm.word_order = std::max(0, std::min(2, atoi(wo)));
  // lockstep refill (NGIA_SERVE_REFILL: idle lanes a warp waits for before it
  // claims); swept on GB300 (200 DNA query batches, 14,077
  // representatives): 32, 24, 16, 8 lanes gave 53.4k, 52.2k, 48.8k, 49.9k
  // queries/s
  sv->prm.refill = 32;
  if (const char *rf = getenv("NGIA_SERVE_REFILL")) sv->prm.refill = std::max(1, std::min(32, atoi(rf)));
  sv->word_first = ngia::word_first_of(sv->type, sv->prm);
  sv->cap_n = cf.max_batch;
  sv->cap_words = cf.max_batch_words;
  sv->cap_nb = cf.max_record_blocks;
  // resident representatives and their k-mer bitsets
  rc = ngia::drv::open_ctx(reps, true, &sv->reps);
  if (rc) {
    ngia::destroy(sv);
    return rc;
  }
  const int bits = sv->type ? 5 : 2;
  const int lw = std::max(1, (int)((1u << (params->word_length * bits)) / 32u));
  ngia_ctx *rc_ctx = sv->reps;
  if (cudaMalloc((void **)&sv->d_lists, 4 * (size_t)lw * (size_t)reps->n) != cudaSuccess) {
    ngia::destroy(sv);
    return fail(NGIA_E_NOMEM, "ngia_serve_open: k-mer table allocation failed");
  }
  sv->store = ngia::RepStore{rc_ctx->db.words, rc_ctx->db.off, rc_ctx->db.len, rc_ctx->db.net, rc_ctx->db.cnt,
                             sv->d_lists, rc_ctx->db.n, lw};
  if (sv->type == 0) {
    sv->store.eq_stride = (int64_t)ngia::eq_words(rc_ctx->db.max_nb);
    if (cudaMalloc((void **)&sv->d_eq, 4 * (size_t)sv->store.eq_stride * (size_t)reps->n) != cudaSuccess) {
      ngia::destroy(sv);
      return fail(NGIA_E_NOMEM, "ngia_serve_open: match table allocation failed");
    }
    sv->store.eq = sv->d_eq;
    ngia::k_rep_eq<<<reps->n, 256, 0, rc_ctx->stream>>>(sv->store, sv->d_eq);
    ngia::k_rep_lists<2><<<reps->n, 256, 0, rc_ctx->stream>>>(sv->store, params->word_length, sv->d_lists);
  } else {
    ngia::k_rep_lists<5><<<reps->n, 256, 0, rc_ctx->stream>>>(sv->store, params->word_length, sv->d_lists);
  }
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(rc_ctx->stream);
  if (e != cudaSuccess) {
    ngia::destroy(sv);
    return fail(NGIA_E_CUDA, "ngia_serve_open: k-mer tables: %s", cudaGetErrorString(e));
  }
  uint32_t ring = 1;
  while ((int)ring < rc_ctx->db.max_nb) ring <<= 1;
  sv->ring_mask = ring - 1;
  for (int k = 0; k < ngia::kServeClasses; k++) {
    e = ngia::serve_align_configure<false>(sv->type, k, ngia::serve_align_smem(sv->type, k, sv->store.eq_stride));
    if (e != cudaSuccess) {
      ngia::destroy(sv);
      return fail(NGIA_E_CUDA, "ngia_serve_open: kernel attributes: %s", cudaGetErrorString(e));
    }
  }
  // slots: as many as asked for and as fit the memory budget
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  const int64_t budget = cf.memory_budget > 0 ? cf.memory_budget : (int64_t)(free_b / 2);
  int occ2 = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, (const void *)ngia::serve_align_fn<false>(sv->type, 2),
                                                ngia::kAlignThreads,
                                                ngia::serve_align_smem(sv->type, 2, sv->store.eq_stride));
  const int64_t per = ngia::slot_bytes(sv, sv->num_sms * std::max(1, occ2));
  const int n_slots = (int)std::min<int64_t>(cf.slots, budget / per);
  if (n_slots < 1) {
    ngia::destroy(sv);
    return fail(NGIA_E_NOMEM, "ngia_serve_open: one slot needs %lld bytes, the budget is %lld", (long long)per,
                (long long)budget);
  }
  for (int k = 0; k < n_slots; k++) {
    sv->slots.push_back(std::make_unique<ngia::Slot>());
    rc = ngia::open_slot(sv, *sv->slots.back(), k);
    if (rc) {
      ngia::destroy(sv);
      return rc;
    }
  }
  for (auto &sl : sv->slots) sl->worker = std::thread(ngia::worker_main, sv, sl.get());
  *out = sv;
  return NGIA_OK;
}

extern "C" int ngia_serve_slots(const ngia_server *s, int32_t *slots) {
  if (!s || !slots) return fail(NGIA_E_ARG, "ngia_serve_slots: null argument");
  *slots = (int32_t)s->slots.size();
  return NGIA_OK;
}

extern "C" int ngia_serve_submit(ngia_server *s, const ngia_db_view *batch, int64_t *ticket) {
  ngia::clear_error();
  if (!s || !batch || !ticket) return fail(NGIA_E_ARG, "ngia_serve_submit: null argument");
  if (batch->type != s->type) return fail(NGIA_E_ARG, "ngia_serve_submit: batch type %d, service type %d", batch->type,
                                          s->type);
  if (batch->n <= 0 || !batch->words || !batch->rec_off || batch->n_words <= 0)
    return fail(NGIA_E_ARG, "ngia_serve_submit: empty or malformed batch");
  if (batch->n > s->cap_n || batch->n_words > s->cap_words)
    return fail(NGIA_E_LIMIT, "ngia_serve_submit: %d records / %lld words exceed a slot (%lld / %lld)", batch->n,
                (long long)batch->n_words, (long long)s->cap_n, (long long)s->cap_words);
  const int nb = ngia::view_max_blocks(batch);
  if (nb > s->cap_nb)
    return fail(NGIA_E_LIMIT, "ngia_serve_submit: a record of %d blocks exceeds a slot (%d)", nb, s->cap_nb);
  auto rq = std::make_unique<ngia::Request>();
  rq->n = batch->n;
  rq->longest = batch->longest;
  rq->words.assign(batch->words, batch->words + batch->n_words);
  rq->off.assign(batch->rec_off, batch->rec_off + batch->n);
  rq->t_submit = ngia::now_ms();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return fail(NGIA_E_STATE, "ngia_serve_submit: service is closing");
    rq->ticket = s->next_ticket++;
    *ticket = rq->ticket;
    s->fifo.push_back(rq.get());
    s->requests.emplace(rq->ticket, std::move(rq));
  }
  s->cv_work.notify_one();
  return NGIA_OK;
}

extern "C" int ngia_serve_poll(ngia_server *s, int64_t ticket, int32_t wait_ms, int32_t *rep_out,
                               int32_t *ident_out, ngia_serve_result *res) {
  ngia::clear_error();
  if (!s || !res) return fail(NGIA_E_ARG, "ngia_serve_poll: null argument");
  std::memset(res, 0, sizeof(*res));
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->requests.find(ticket);
  if (it == s->requests.end()) return fail(NGIA_E_ARG, "ngia_serve_poll: unknown ticket %lld", (long long)ticket);
  ngia::Request *rq = it->second.get();
  auto ready = [&] { return rq->status != 0; };
  if (!ready() && wait_ms != 0) {
    if (wait_ms < 0)
      s->cv_done.wait(lk, ready);
    else
      s->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), ready);
  }
  if (!ready()) return NGIA_OK;
  res->slot = rq->slot;
  res->rounds = rq->rounds;
  res->queued_ms = rq->t_start - rq->t_submit;
  res->run_ms = rq->t_done - rq->t_start;
  if (rq->status < 0) {
    const int code = rq->status;
    const std::string msg = rq->error;
    s->requests.erase(it);
    return fail(code, "serve batch %lld: %s", (long long)ticket, msg.c_str());
  }
  if (rep_out) std::memcpy(rep_out, rq->rep.data(), sizeof(int32_t) * rq->rep.size());
  if (ident_out) std::memcpy(ident_out, rq->ident.data(), sizeof(int32_t) * rq->ident.size());
  res->done = 1;
  res->resident = rq->resident;
  res->new_reps = rq->new_reps;
  res->pairs = rq->pairs;
  res->cells = rq->cells;
  s->requests.erase(it);
  return NGIA_OK;
}

extern "C" int ngia_serve_close(ngia_server *s) {
  if (!s) return NGIA_OK;
  ngia::destroy(s);
  return NGIA_OK;
}
