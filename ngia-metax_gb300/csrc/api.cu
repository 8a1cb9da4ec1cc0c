// api.cu — device half of the C ABI (include/ngia.h): context lifetime, the
// greedy driver in its two forms, and the pair-score entry point.
//
// Reference counterparts (CUDA/signalNode/src/func.cu):
//   ngia_open            readData device copy (104-154)
//   ngia_cluster_begin   initBench (157-183)
//   ngia_cluster_step    the while(true) loop of clustering (616-675)
//   ngia_cluster_end     the cluster[] hand-off to saveResult (692-705)
//   ngia_close           finish (767-781)
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstring>
#include <new>

#include "../host/host_common.h"
#include "ctx.h"

using ngia::fail;
using namespace ngia::drv;

#define CK(call)                                                                                  \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) return fail(NGIA_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_));     \
  } while (0)

namespace ngia {
namespace drv {

template <class T>
cudaError_t dalloc(T **p, size_t count) {
  return cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(count, 1));
}

int check_device_error(ngia_ctx *c) {
  if (c->h_state->err)
    return fail(NGIA_E_DEVICE, "device error %d in kernel %d (bounded wait expired or scratch too small)",
                c->h_state->err, c->h_state->err_where);
  return NGIA_OK;
}

int pull_state(ngia_ctx *c) {
  CK(cudaMemcpyAsync(c->h_state, c->rb.st, sizeof(ngia::RunState), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return check_device_error(c);
}

// One greedy iteration: prepare the representative, filter the unclustered
// set into class queues, align every class, pick the next representative.
// In graph form the class kernels of a single job run as parallel branches;
// batch members keep them on one stream (the batch runs jobs side by side).
int enqueue_iteration(ngia_ctx *c, bool graph, cudaGraphConditionalHandle cond) {
  const bool prof = c->profiling && !graph;
  CK(ngia::launch_prep(c, -1));
  if (prof) CK(cudaEventRecord(c->ev_p0, c->stream));
  CK(ngia::launch_filter(c));
  if (prof) CK(cudaEventRecord(c->ev_p1, c->stream));
  const int nc = ngia::num_classes(c->db.type);
  if (graph && !c->batch_member) {
    // classes run as parallel branches of the body graph
    CK(cudaEventRecord(c->fork_ev, c->stream));
    for (int k = 0; k < nc; k++) {
      CK(cudaStreamWaitEvent(c->side[k], c->fork_ev, 0));
      CK(ngia::launch_align(c, k, c->side[k], 0));
      CK(cudaEventRecord(c->join_ev[k], c->side[k]));
      CK(cudaStreamWaitEvent(c->stream, c->join_ev[k], 0));
    }
  } else {
    for (int k = 0; k < nc; k++) {
      if (prof) CK(cudaEventRecord(c->ev_cls[k], c->stream));
      CK(ngia::launch_align(c, k, c->stream, 0));
    }
    if (prof) CK(cudaEventRecord(c->ev_cls[nc], c->stream));
  }
  if (prof) CK(cudaEventRecord(c->ev_p2, c->stream));
  CK(ngia::launch_next(c, (unsigned long long)cond, graph ? 1 : 0));
  return NGIA_OK;
}

// Adds the stage times of the iteration just synchronised (profiling).
void account_stages(ngia_ctx *c) {
  float a = 0.f, b = 0.f;
  if (cudaEventElapsedTime(&a, c->ev_p0, c->ev_p1) == cudaSuccess) c->ms_filter += a;
  if (cudaEventElapsedTime(&b, c->ev_p1, c->ev_p2) == cudaSuccess) c->ms_align += b;
  for (int k = 0; k < ngia::num_classes(c->db.type); k++) {
    float m = 0.f;
    if (cudaEventElapsedTime(&m, c->ev_cls[k], c->ev_cls[k + 1]) == cudaSuccess) c->ms_class[k] += m;
  }
}

void fill_stats(const ngia_ctx *c, ngia_stats *stats) {
  const ngia::RunState &s = *c->h_state;
  stats->iterations = s.iter;
  stats->candidates = (int64_t)s.st_candidates;
  stats->base_pass = (int64_t)s.st_base_pass;
  stats->align_pairs = (int64_t)s.st_align_pairs;
  stats->members = (int64_t)s.st_members;
  stats->band_cells = (int64_t)s.st_band_cells;
  stats->filter_bytes = (int64_t)s.st_filter_bytes;
  stats->word_checks = (int64_t)s.st_word_checks;
  stats->done_cells = (int64_t)s.st_done_cells;
  if (c->mode == NGIA_MODE_SPEC) {  // pairs and cells of the speculative rounds
    int64_t pairs = 0, cells = 0;
    spec_stats(c, &pairs, &cells);
    stats->align_pairs += pairs;
    stats->done_cells += cells;
  }
  stats->ms_filter = c->ms_filter;
  stats->ms_align = c->ms_align;
  for (int k = 0; k < 8; k++) {
    stats->class_pairs[k] = k < ngia::kNumClasses ? (int64_t)s.st_class_pairs[k] : 0;
    stats->class_ms[k] = k < ngia::kNumClasses ? c->ms_class[k] : 0.0;
    stats->class_cells[k] = k < ngia::kNumClasses ? (int64_t)s.st_class_done[k] : 0;
    stats->class_bytes[k] = k < ngia::kNumClasses ? 4 * (int64_t)s.st_class_qwords[k] : 0;
  }
}

void destroy_graph(ngia_ctx *c) {
  if (c->graph_exec) cudaGraphExecDestroy(c->graph_exec);
  if (c->graph) cudaGraphDestroy(c->graph);
  c->graph_exec = nullptr;
  c->graph = nullptr;
  c->graph_ready = false;
}

// Captures the loop body once into the body of a conditional WHILE node; the
// node re-runs it until k_next clears the condition.
int build_graph(ngia_ctx *c) {
  destroy_graph(c);
  CK(cudaGraphCreate(&c->graph, 0));
  cudaGraphConditionalHandle cond;
  CK(cudaGraphConditionalHandleCreate(&cond, c->graph, 1, cudaGraphCondAssignDefault));
  cudaGraphNodeParams np = {cudaGraphNodeTypeConditional};
  np.conditional.handle = cond;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  CK(cudaGraphAddNode(&node, c->graph, nullptr, nullptr, 0, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  CK(cudaStreamBeginCaptureToGraph(c->stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_iteration(c, true, cond);
  cudaGraph_t captured = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->stream, &captured);
  if (rc != NGIA_OK || e != cudaSuccess) {
    destroy_graph(c);  // a body whose capture failed is never instantiated
    return rc != NGIA_OK ? rc : fail(NGIA_E_CUDA, "graph capture: %s", cudaGetErrorString(e));
  }
  cudaGraphExec_t exec = nullptr;
  e = cudaGraphInstantiate(&exec, c->graph, 0);
  if (e != cudaSuccess) {
    destroy_graph(c);
    return fail(NGIA_E_CUDA, "graph instantiate: %s", cudaGetErrorString(e));
  }
  c->graph_exec = exec;
  c->graph_warp_pairs = c->warp_pairs;
  c->graph_tune_gen = c->tune_gen;
  c->graph_ready = true;
  c->graph_prm = c->prm;
  return NGIA_OK;
}

bool same_params(const ngia::RunParams &a, const ngia::RunParams &b) {
  return a.s == b.s && a.w == b.w && a.precise == b.precise && a.word_order == b.word_order && a.refill == b.refill &&
         a.wait_polls == b.wait_polls;
}

// The captured loop for the context's current parameters and tuning,
// captured again only when they changed.
int ensure_graph(ngia_ctx *c) {
  if (c->graph_ready && same_params(c->graph_prm, c->prm) && c->graph_warp_pairs == c->warp_pairs &&
      c->graph_tune_gen == c->tune_gen)
    return NGIA_OK;
  return build_graph(c);
}

int validate_params(int type, const ngia_params *p) {
  if (!p) return fail(NGIA_E_ARG, "null params");
  if (!(p->similarity >= 0.1f && p->similarity <= 1.0f))
    return fail(NGIA_E_ARG, "similarity %g outside [0.1, 1.0] (apply ngia_params_clamp)", (double)p->similarity);
  const int lo = type == 0 ? 4 : 2, hi = type == 0 ? 8 : 3;
  if (p->word_length < lo || p->word_length > hi)
    return fail(NGIA_E_ARG, "word length %d outside [%d, %d] (apply ngia_params_clamp)", p->word_length, lo, hi);
  if (p->precise != 0 && p->precise != 1) return fail(NGIA_E_ARG, "precise must be 0 or 1");
  return NGIA_OK;
}

}  // namespace drv
}  // namespace ngia

extern "C" int ngia_open(const ngia_db_view *v, ngia_ctx **out) { return ngia::drv::open_ctx(v, false, out); }

namespace {

using ngia::drv::dalloc;

// Streams and events of a context.
int create_streams(ngia_ctx *c) {
  cudaError_t e = cudaGetDevice(&c->device);
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "no CUDA device: %s", cudaGetErrorString(e));
  if (cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device) != cudaSuccess)
    return fail(NGIA_E_CUDA, "cannot query SM count");
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess)
    return fail(NGIA_E_CUDA, "cannot create stream");
  for (int k = 0; k < ngia::kNumClasses; k++) {
    if (cudaStreamCreateWithFlags(&c->side[k], cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&c->join_ev[k], cudaEventDisableTiming) != cudaSuccess)
      return fail(NGIA_E_CUDA, "cannot create side streams");
  }
  if (cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreate(&c->ev_step0) != cudaSuccess || cudaEventCreate(&c->ev_step1) != cudaSuccess ||
      cudaEventCreate(&c->ev_p0) != cudaSuccess || cudaEventCreate(&c->ev_p1) != cudaSuccess ||
      cudaEventCreate(&c->ev_p2) != cudaSuccess)
    return fail(NGIA_E_CUDA, "cannot create event");
  for (auto &ev : c->ev_cls)
    if (cudaEventCreate(&ev) != cudaSuccess) return fail(NGIA_E_CUDA, "cannot create event");
  if (dalloc(&c->d_flags, 3) != cudaSuccess || cudaMallocHost((void **)&c->h_flags, 3 * sizeof(int32_t)) != cudaSuccess)
    return fail(NGIA_E_NOMEM, "ngia_open: allocation failed");
  if (cudaMallocHost((void **)&c->h_state, sizeof(ngia::RunState)) != cudaSuccess)
    return fail(NGIA_E_NOMEM, "ngia_open: pinned allocation failed");
  std::memset(c->h_state, 0, sizeof(ngia::RunState));
  return NGIA_OK;
}

// Device arrays of a database of up to cap_n records and cap_words words.
int alloc_db(ngia_ctx *c, int type, int64_t cap_n, int64_t cap_words) {
  const int A = ngia::count_words(type);
  // protein residue-code streams for the short-word test (NGIA_PROTEIN_CODES=0:
  // the test reads the planes instead)
  const char *pc = getenv("NGIA_PROTEIN_CODES");
  const bool codes = type != 0 && !(pc && atoi(pc) == 0);
  if (dalloc(&c->d_words, (size_t)cap_words + 4) != cudaSuccess || dalloc(&c->d_off, (size_t)cap_n) != cudaSuccess ||
      dalloc(&c->d_len, (size_t)cap_n) != cudaSuccess || dalloc(&c->d_net, (size_t)cap_n) != cudaSuccess ||
      dalloc(&c->d_cnt, (size_t)cap_n * A) != cudaSuccess ||
      (codes && dalloc(&c->d_codes, (size_t)cap_words + 4) != cudaSuccess))
    return fail(NGIA_E_NOMEM, "ngia_open: device allocation of the database failed");
  c->cap_n = cap_n;
  c->cap_words = cap_words;
  c->db.words = c->d_words;
  c->db.off = c->d_off;
  c->db.len = c->d_len;
  c->db.net = c->d_net;
  c->db.cnt = c->d_cnt;
  c->db.codes = c->d_codes;
  c->db.n = 0;
  c->db.type = type;
  c->db.hw = ngia::header_words(type);
  c->db.P = ngia::plane_count(type);
  c->db.A = A;
  c->db.max_nb = 1;
  return NGIA_OK;
}

// Copies a database view into the context's arrays (one host-to-device copy
// of the records and offsets) and builds the header arrays on the device.
int load_db(ngia_ctx *c, const ngia_db_view *v) {
  cudaError_t e =
      cudaMemcpyAsync(c->d_words, v->words, sizeof(uint32_t) * (size_t)v->n_words, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(c->d_off, v->rec_off, sizeof(int64_t) * (size_t)v->n, cudaMemcpyHostToDevice, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(c->d_flags, 0, 3 * sizeof(int32_t), c->stream);
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "ngia_open: copy: %s", cudaGetErrorString(e));
  c->n_words = v->n_words;
  c->longest = v->longest;
  c->db.n = v->n;
  e = ngia::launch_loader(c, c->d_flags, c->d_flags + 1, c->d_flags + 2);
  if (e == cudaSuccess) e = cudaMemcpyAsync(c->h_flags, c->d_flags, 3 * sizeof(int32_t), cudaMemcpyDeviceToHost, c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "ngia_open: loader: %s", cudaGetErrorString(e));
  if (c->h_flags[2]) return fail(NGIA_E_FORMAT, "ngia_open: a record offset or header is out of range");
  c->db.max_nb = std::max(1, c->h_flags[0]);
  c->db.has_short = c->h_flags[1];
  return NGIA_OK;
}

// Launch grids for the loaded database: persistent grids over the whole GPU,
// or (batch members and serving slots, which share the GPU with other jobs)
// one CTA per 128 candidates and one warp per bitmap word.
void size_grids(ngia_ctx *c, bool by_size) {
  const int type = c->db.type;
  for (int k = 0; k < ngia::num_classes(type); k++)
    c->grid_align[k] = c->num_sms * ngia::align_occupancy(type, k, c->cap_nb);
  c->grid_filter = c->num_sms * 8;
  // warp-per-pair: the whole GPU's warps; a class goes warp-per-pair when it
  // has at most one pair per warp (a wide pair's latency on a warp is a few
  // times shorter than on a thread, at ~6x the instructions per cell; swept
  // on GB300: 0.25, 0.5, 1 and 2 pairs per warp gave 41, 47, 47 and 40M
  // candidate seqs/s on the 20,000-sequence DNA workload and within 1% of
  // each other on the 1M DNA and 200k protein workloads)
  c->grid_warp = c->num_sms * ngia::align_occupancy(type, ngia::kNumClasses, c->cap_nb);
  c->warp_pairs = c->grid_warp * (ngia::align_threads() / 32);
  if (by_size) {
    const int64_t n = std::max(1, c->db.n), nbw = (n + 31) / 32;
    const int by_n = (int)std::min<int64_t>((n + 127) / 128, INT32_MAX);
    for (int k = 0; k < ngia::num_classes(type); k++) c->grid_align[k] = std::max(1, std::min(c->grid_align[k], by_n));
    c->grid_filter = std::max(1, std::min(c->grid_filter, (int)((nbw + 7) / 8)));
    // warp-per-pair: no more warps than the job has sequences
    const int wpc = ngia::align_threads() / 32;
    c->grid_warp = std::max(1, std::min(c->grid_warp, (int)((n + wpc - 1) / wpc)));
    c->warp_pairs = c->grid_warp * wpc;
  }
  if (const char *w = getenv("NGIA_WARP_PAIRS")) c->warp_pairs = atoi(w);
  c->warp_pairs_default = c->warp_pairs;
}

// Run buffers for up to cap_n sequences whose records have up to cap_nb
// plane blocks (grids sized for that capacity).
int alloc_run(ngia_ctx *c, int64_t cap_n, int cap_nb) {
  const int type = c->db.type;
  c->cap_nb = std::max(1, cap_nb);
  const size_t nbw = (size_t)(cap_n + 31) / 32;
  ngia::RunBufs &rb = c->rb;
  bool ok = dalloc(&rb.st, 1) == cudaSuccess && dalloc(&rb.cluster, (size_t)cap_n) == cudaSuccess &&
            dalloc(&rb.ident, (size_t)cap_n) == cudaSuccess && dalloc(&rb.alive, nbw) == cudaSuccess &&
            dalloc(&rb.rep_rec, 32 + (size_t)ngia::kMaxBlocks * 5 + 64) == cudaSuccess &&
            dalloc(&rb.rep_list, ngia::kListWords) == cudaSuccess &&
            dalloc(&rb.first_short, ngia::kRefGridThreads) == cudaSuccess &&
            dalloc(&rb.scan_part, nbw) == cudaSuccess && dalloc(&rb.long_list, (size_t)cap_n) == cudaSuccess;
  ok = ok && cudaMalloc((void **)&rb.flags, 4 * std::max<size_t>(nbw, 1)) == cudaSuccess;
  ok = ok && dalloc(&rb.fstats, (size_t)ngia::kFilterStripes * ngia::kFilterStats) == cudaSuccess;
  for (int k = 0; ok && k < ngia::num_classes(type); k++) ok = dalloc(&rb.queue[k], (size_t)cap_n) == cudaSuccess;
  if (!ok) return fail(NGIA_E_NOMEM, "ngia_open: device allocation of run buffers failed");
  cudaMemsetAsync(rb.rep_list, 0, 4 * ngia::kListWords, c->stream);
  cudaMemsetAsync(rb.fstats, 0, 8 * ngia::kFilterStripes * ngia::kFilterStats, c->stream);
  if (ngia::align_configure(type, c->cap_nb) != cudaSuccess || ngia::filter_configure() != cudaSuccess)
    return fail(NGIA_E_CUDA, "ngia_open: kernel attributes");
  // the widest class keeps its rows in global scratch, sized for this
  // context's grid at capacity (every later grid of the context is within)
  const int32_t saved_n = c->db.n;
  c->db.n = (int32_t)cap_n;
  size_grids(c, c->batch_member);
  c->db.n = saved_n;
  const int g = ngia::generic_class(type);
  rb.generic_lanes = c->grid_align[g] * ngia::align_threads();
  uint32_t ring = 1;
  while ((int)ring < c->cap_nb) ring <<= 1;
  rb.ring_mask = ring - 1;
  rb.scratch_words = (int64_t)rb.generic_lanes * ring;
  if (dalloc(&rb.scratch, (size_t)rb.scratch_words) != cudaSuccess)
    return fail(NGIA_E_NOMEM, "ngia_open: device allocation of alignment scratch failed");
  return NGIA_OK;
}

}  // namespace

int ngia::drv::open_ctx(const ngia_db_view *v, bool batch_member, ngia_ctx **out) {
  ngia::clear_error();
  if (!v || !out) return fail(NGIA_E_ARG, "ngia_open: null argument");
  if (v->n <= 0 || (v->type != 0 && v->type != 1) || !v->words || !v->rec_off || v->n_words <= 0)
    return fail(NGIA_E_ARG, "ngia_open: empty or malformed database view (n=%d type=%d)", v->n, v->type);
  ngia_ctx *c = new (std::nothrow) ngia_ctx();
  if (!c) return fail(NGIA_E_NOMEM, "ngia_open: out of host memory");
  c->batch_member = batch_member;
  *out = nullptr;
  int rc = create_streams(c);
  if (!rc) rc = alloc_db(c, v->type, v->n, v->n_words);
  if (!rc) rc = load_db(c, v);
  if (!rc) rc = alloc_run(c, v->n, c->db.max_nb);
  if (!rc) {
    size_grids(c, batch_member);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = fail(NGIA_E_CUDA, "ngia_open: %s", cudaGetErrorString(e));
  }
  if (rc) {
    ngia_close(c);
    return rc;
  }
  *out = c;
  return NGIA_OK;
}

int ngia::drv::open_ctx_capacity(int type, int64_t cap_n, int64_t cap_words, int cap_nb, ngia_ctx **out) {
  if (!out || (type != 0 && type != 1) || cap_n <= 0 || cap_words <= 0 || cap_nb <= 0 || cap_nb > ngia::kMaxBlocks)
    return fail(NGIA_E_ARG, "open_ctx_capacity: bad argument");
  ngia_ctx *c = new (std::nothrow) ngia_ctx();
  if (!c) return fail(NGIA_E_NOMEM, "out of host memory");
  c->batch_member = true;
  *out = nullptr;
  int rc = create_streams(c);
  if (!rc) rc = alloc_db(c, type, cap_n, cap_words);
  if (!rc) rc = alloc_run(c, cap_n, cap_nb);
  if (!rc) {
    cudaError_t e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) rc = fail(NGIA_E_CUDA, "open_ctx_capacity: %s", cudaGetErrorString(e));
  }
  if (rc) {
    ngia_close(c);
    return rc;
  }
  *out = c;
  return NGIA_OK;
}

int ngia::drv::reload_ctx(ngia_ctx *c, const ngia_db_view *v) {
  if (!c || !v || v->type != c->db.type || v->n <= 0 || !v->words || !v->rec_off || v->n_words <= 0)
    return fail(NGIA_E_ARG, "reload: bad database view");
  if (v->n > c->cap_n || v->n_words > c->cap_words)
    return fail(NGIA_E_LIMIT, "reload: %d records / %lld words exceed the capacity (%lld / %lld)", v->n,
                (long long)v->n_words, (long long)c->cap_n, (long long)c->cap_words);
  // longest record, checked on the host before anything is copied
  int nb = 0;
  for (int32_t i = 0; i < v->n; i++) {
    const int64_t o = v->rec_off[i];
    if (o < 0 || o + 2 > v->n_words) return fail(NGIA_E_FORMAT, "reload: record %d offset out of range", i);
    nb = std::max(nb, (int)((v->words[o + 1] + 31) / 32));
  }
  if (nb > c->cap_nb)
    return fail(NGIA_E_LIMIT, "reload: a record of %d blocks exceeds the capacity of %d", nb, c->cap_nb);
  const ngia::DevDB before = c->db;
  const int grids_before = c->grid_filter, warp_before = c->grid_warp;
  c->begun = false;
  int rc = load_db(c, v);
  if (rc) {
    destroy_graph(c);
    return rc;
  }
  if (c->db.max_nb > c->cap_nb) {
    destroy_graph(c);
    return fail(NGIA_E_LIMIT, "reload: a record of %d blocks exceeds the capacity of %d", c->db.max_nb, c->cap_nb);
  }
  size_grids(c, c->batch_member);
  // a captured graph holds the kernel arguments (sizes) and grids: it stays
  // valid when the database has the same shape
  const bool same = before.n == c->db.n && before.max_nb == c->db.max_nb && before.has_short == c->db.has_short &&
                    grids_before == c->grid_filter && warp_before == c->grid_warp;
  if (!same) destroy_graph(c);
  return NGIA_OK;
}

extern "C" int ngia_reload(ngia_ctx *c, const ngia_db_view *v) {
  ngia::clear_error();
  return ngia::drv::reload_ctx(c, v);
}

extern "C" int ngia_close(ngia_ctx *c) {
  if (!c) return NGIA_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  destroy_graph(c);
  ngia::drv::spec_free(c);
  cudaFree(c->d_words);
  cudaFree(c->d_off);
  cudaFree(c->d_len);
  cudaFree(c->d_net);
  cudaFree(c->d_cnt);
  cudaFree(c->d_codes);
  ngia::RunBufs &rb = c->rb;
  cudaFree(rb.st);
  cudaFree(rb.cluster);
  cudaFree(rb.ident);
  cudaFree(rb.alive);
  cudaFree(rb.rep_rec);
  cudaFree(rb.rep_list);
  cudaFree(rb.first_short);
  cudaFree(rb.scan_part);
  cudaFree(rb.long_list);
  cudaFree(rb.flags);
  cudaFree(rb.fstats);
  cudaFree(rb.scratch);
  for (int k = 0; k < ngia::kNumClasses; k++) cudaFree(rb.queue[k]);
  if (c->h_state) cudaFreeHost(c->h_state);
  cudaFree(c->d_flags);
  if (c->h_flags) cudaFreeHost(c->h_flags);
  for (int k = 0; k < ngia::kNumClasses; k++) {
    if (c->side[k]) cudaStreamDestroy(c->side[k]);
    if (c->join_ev[k]) cudaEventDestroy(c->join_ev[k]);
  }
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  for (cudaEvent_t ev : {c->ev_step0, c->ev_step1, c->ev_p0, c->ev_p1, c->ev_p2})
    if (ev) cudaEventDestroy(ev);
  for (cudaEvent_t ev : c->ev_cls)
    if (ev) cudaEventDestroy(ev);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return NGIA_OK;
}

extern "C" void *ngia_stream(ngia_ctx *c) { return c ? (void *)c->stream : nullptr; }

extern "C" int ngia_device_count(int32_t *count) {
  if (!count) return fail(NGIA_E_ARG, "ngia_device_count: null argument");
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess) n = 0;
  *count = n;
  return NGIA_OK;
}

extern "C" int ngia_cluster_begin(ngia_ctx *c, const ngia_params *p, int32_t mode) {
  return ngia::drv::begin_subset(c, p, mode, nullptr);
}

int ngia::drv::begin_subset(ngia_ctx *c, const ngia_params *p, int32_t mode, const uint32_t *d_alive) {
  ngia::clear_error();
  if (!c) return fail(NGIA_E_ARG, "ngia_cluster_begin: null context");
  if (c->db.n <= 0) return fail(NGIA_E_STATE, "ngia_cluster_begin: no database loaded");
  int rc = validate_params(c->db.type, p);
  if (rc) return rc;
  if (mode != NGIA_MODE_PLAIN && mode != NGIA_MODE_GRAPH && mode != NGIA_MODE_SPEC)
    return fail(NGIA_E_ARG, "unknown mode %d", mode);
  c->prm.s = p->similarity;
  c->prm.w = p->word_length;
  c->prm.precise = p->precise;
  c->prm.word_order = c->tuned_word_order;
  if (const char *wo = getenv("NGIA_WORD_ORDER")) c->prm.word_order = atoi(wo);
  c->prm.refill = c->tuned_refill;
  if (const char *rf = getenv("NGIA_REFILL")) c->prm.refill = std::max(1, std::min(32, atoi(rf)));
  if (!getenv("NGIA_WARP_PAIRS")) c->warp_pairs = c->tuned_warp_pairs >= 0 ? c->tuned_warp_pairs : c->warp_pairs_default;
  if (c->db.has_short && !c->prm.precise) c->prm.word_order = 1;  // exact path is word first
  // NGIA_WAIT_POLLS lowers the poll limit of the alignment kernels' staging
  // wait; at 0 every such wait gives up at once, which is how the tests make
  // the device-side error path (NGIA_E_DEVICE, context still usable) run
  c->prm.wait_polls = ngia::kWaitPolls;
  if (const char *wp = getenv("NGIA_WAIT_POLLS"))
    c->prm.wait_polls = (uint32_t)std::max<long long>(0, std::min<long long>(atoll(wp), ngia::kWaitPolls));
  c->mode = mode;
  c->ms_filter = c->ms_align = 0.0;
  for (double &m : c->ms_class) m = 0.0;
  c->last_step_ms = 0.f;
  c->begun = false;  // no steppable run until the new one is fully set up
  CK(ngia::launch_init_run(c));
  if (d_alive) CK(ngia::launch_subset_start(c, d_alive));
  rc = pull_state(c);
  if (rc) return rc;
  if (mode == NGIA_MODE_GRAPH) {
    rc = ensure_graph(c);
    if (rc) return rc;
  }
  if (mode == NGIA_MODE_SPEC) {
    rc = spec_prepare(c);
    if (rc) return rc;
  }
  c->begun = true;
  return NGIA_OK;
}

extern "C" int ngia_cluster_step(ngia_ctx *c, int64_t max_iters, int32_t *done) {
  if (!c) return fail(NGIA_E_ARG, "ngia_cluster_step: null context");
  if (!c->begun) return fail(NGIA_E_STATE, "ngia_cluster_step before ngia_cluster_begin");
  if (c->h_state->done) {
    if (done) *done = 1;
    return NGIA_OK;
  }
  if (c->mode == NGIA_MODE_GRAPH) {
    c->h_state->iter_limit = max_iters > 0 ? c->h_state->iter + max_iters : LLONG_MAX;
    CK(cudaMemcpyAsync(&c->rb.st->iter_limit, &c->h_state->iter_limit, sizeof(int64_t), cudaMemcpyHostToDevice,
                       c->stream));
    CK(cudaEventRecord(c->ev_step0, c->stream));
    CK(cudaGraphLaunch(c->graph_exec, c->stream));
    CK(cudaEventRecord(c->ev_step1, c->stream));
    int rc = pull_state(c);
    if (rc) return rc;
  } else if (c->mode == NGIA_MODE_SPEC) {
    CK(cudaEventRecord(c->ev_step0, c->stream));
    int rc = ngia::drv::spec_step(c, max_iters);
    if (rc) return rc;
    CK(cudaEventRecord(c->ev_step1, c->stream));
    CK(cudaEventSynchronize(c->ev_step1));
  } else {
    CK(cudaEventRecord(c->ev_step0, c->stream));
    for (int64_t it = 0; max_iters <= 0 || it < max_iters; it++) {
      if (it > (int64_t)c->db.n)  // every iteration retires one representative
        return fail(NGIA_E_STATE, "ngia_cluster_step: more iterations than sequences");
      int rc = enqueue_iteration(c, false, 0);
      if (rc) return rc;
      rc = pull_state(c);  // the per-representative host round trip of the plain form
      if (rc) return rc;
      if (c->profiling) account_stages(c);
      if (c->h_state->done) break;
    }
    CK(cudaEventRecord(c->ev_step1, c->stream));
    CK(cudaEventSynchronize(c->ev_step1));
  }
  CK(cudaEventElapsedTime(&c->last_step_ms, c->ev_step0, c->ev_step1));
  if (done) *done = c->h_state->done;
  return NGIA_OK;
}

extern "C" int ngia_step_device_ms(ngia_ctx *c, float *ms) {
  if (!c || !ms) return fail(NGIA_E_ARG, "ngia_step_device_ms: null argument");
  *ms = c->last_step_ms;
  return NGIA_OK;
}

extern "C" int ngia_set_profiling(ngia_ctx *c, int32_t on) {
  if (!c) return fail(NGIA_E_ARG, "ngia_set_profiling: null context");
  c->profiling = on != 0;
  return NGIA_OK;
}

extern "C" int ngia_cluster_stats(ngia_ctx *c, ngia_stats *stats) {
  if (!c || !stats) return fail(NGIA_E_ARG, "ngia_cluster_stats: null argument");
  if (!c->begun) return fail(NGIA_E_STATE, "ngia_cluster_stats before ngia_cluster_begin");
  int rc = pull_state(c);
  if (rc) return rc;
  fill_stats(c, stats);
  return NGIA_OK;
}

extern "C" int ngia_set_device(int32_t device) {
  cudaError_t e = cudaSetDevice(device);
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
  return NGIA_OK;
}

extern "C" int ngia_pin_host(void *ptr, size_t bytes) {
  if (!ptr || !bytes) return fail(NGIA_E_ARG, "ngia_pin_host: empty buffer");
  cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "cudaHostRegister: %s", cudaGetErrorString(e));
  return NGIA_OK;
}

extern "C" int ngia_unpin_host(void *ptr) {
  cudaError_t e = cudaHostUnregister(ptr);
  if (e != cudaSuccess) return fail(NGIA_E_CUDA, "cudaHostUnregister: %s", cudaGetErrorString(e));
  return NGIA_OK;
}

extern "C" int ngia_cluster_end(ngia_ctx *c, int32_t *cluster_out, int32_t *identity_out, ngia_stats *stats) {
  if (!c) return fail(NGIA_E_ARG, "ngia_cluster_end: null context");
  if (!c->begun) return fail(NGIA_E_STATE, "ngia_cluster_end before ngia_cluster_begin");
  const size_t n = (size_t)c->db.n;
  if (cluster_out) CK(cudaMemcpyAsync(cluster_out, c->rb.cluster, 4 * n, cudaMemcpyDeviceToHost, c->stream));
  if (identity_out) CK(cudaMemcpyAsync(identity_out, c->rb.ident, 4 * n, cudaMemcpyDeviceToHost, c->stream));
  int rc = pull_state(c);
  if (rc) return rc;
  if (stats) fill_stats(c, stats);
  return NGIA_OK;
}

extern "C" int ngia_cluster(ngia_ctx *c, const ngia_params *p, int32_t mode, int32_t *cluster_out,
                            int32_t *identity_out, ngia_stats *stats) {
  int rc = ngia_cluster_begin(c, p, mode);
  if (rc) return rc;
  int32_t done = 0;
  rc = ngia_cluster_step(c, 0, &done);
  if (rc) return rc;
  if (!done) return fail(NGIA_E_STATE, "clustering stopped before every sequence was assigned");
  return ngia_cluster_end(c, cluster_out, identity_out, stats);
}

extern "C" int ngia_pair_scores(ngia_ctx *c, const ngia_params *p, int32_t rep, const int32_t *cands, int32_t n,
                                int32_t *out) {
  ngia::clear_error();
  if (!c || !cands || !out || n < 0) return fail(NGIA_E_ARG, "ngia_pair_scores: bad argument");
  int rc = validate_params(c->db.type, p);
  if (rc) return rc;
  if (rep < 0 || rep >= c->db.n) return fail(NGIA_E_ARG, "ngia_pair_scores: rep %d out of range", rep);
  for (int32_t k = 0; k < n; k++)
    if (cands[k] < 0 || cands[k] >= c->db.n) return fail(NGIA_E_ARG, "ngia_pair_scores: candidate out of range");
  if (n == 0) return NGIA_OK;
  if (n > c->db.n) return fail(NGIA_E_LIMIT, "ngia_pair_scores: at most n pairs per call");
  c->prm.s = p->similarity;
  c->prm.w = p->word_length;
  c->prm.precise = p->precise;
  c->prm.refill = 32;
  c->prm.wait_polls = ngia::kWaitPolls;
  int32_t *d_c = nullptr, *d_o = nullptr;
  CK(dalloc(&d_c, (size_t)n));
  CK(dalloc(&d_o, 4 * (size_t)n));
  c->rb.score_cands = d_c;
  c->rb.score_out = d_o;
  CK(cudaMemcpyAsync(d_c, cands, 4 * (size_t)n, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemsetAsync(c->rb.st, 0, sizeof(ngia::RunState), c->stream));
  CK(ngia::launch_prep(c, rep));
  CK(ngia::launch_score_classify(c, n));
  for (int k = 0; k < ngia::num_classes(c->db.type); k++) CK(ngia::launch_align(c, k, c->stream, 1));
  CK(cudaMemcpyAsync(out, d_o, 16 * (size_t)n, cudaMemcpyDeviceToHost, c->stream));
  rc = pull_state(c);
  cudaFree(d_c);
  cudaFree(d_o);
  c->rb.score_cands = nullptr;
  c->rb.score_out = nullptr;
  c->begun = false;
  return rc;
}
