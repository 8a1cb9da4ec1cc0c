// batch.cu — many independent clustering jobs on one GPU.
//
// A batch owns one context per job (its database, run buffers and class
// queues, grids sized to the job).  In graph form every job's whole greedy
// loop is one launch of its CUDA graph (a conditional WHILE node re-running
// the job's iteration — prepare, filter into length classes, align, next
// representative — until the job is done); the batch enqueues the launches of
// all jobs on their own streams before waiting once, so jobs run side by side
// with no host round trip per representative anywhere in the batch.  The plain
// form runs the jobs one after the other with the host-loop driver (the
// reference's way of working, one job per run).  Every job's result is
// identical to clustering it alone.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <vector>

#include "../host/host_common.h"
#include "ctx.h"

using ngia::fail;

struct ngia_batch {
  std::vector<ngia_ctx *> jobs;
};

#define CKB(call)                                                                                 \
  do {                                                                                            \
    cudaError_t e_ = (call);                                                                      \
    if (e_ != cudaSuccess) return fail(NGIA_E_CUDA, "%s: %s", #call, cudaGetErrorString(e_));     \
  } while (0)

extern "C" int ngia_batch_open(const ngia_db_view *jobs, int32_t n_jobs, ngia_batch **out) {
  ngia::clear_error();
  if (!jobs || !out || n_jobs <= 0) return fail(NGIA_E_ARG, "ngia_batch_open: bad argument");
  ngia_batch *b = new (std::nothrow) ngia_batch();
  if (!b) return fail(NGIA_E_NOMEM, "ngia_batch_open: out of host memory");
  *out = nullptr;
  for (int32_t j = 0; j < n_jobs; j++) {
    ngia_ctx *c = nullptr;
    int rc = ngia::drv::open_ctx(&jobs[j], true, &c);
    if (rc) {
      ngia_batch_close(b);
      return rc;
    }
    b->jobs.push_back(c);
  }
  *out = b;
  return NGIA_OK;
}

extern "C" int ngia_batch_run(ngia_batch *b, const ngia_params *params, int32_t mode, int64_t max_iters,
                              int32_t **cluster_out, int32_t **identity_out, ngia_stats *stats) {
  ngia::clear_error();
  if (!b || !params) return fail(NGIA_E_ARG, "ngia_batch_run: bad argument");
  if (mode != NGIA_MODE_PLAIN && mode != NGIA_MODE_GRAPH) return fail(NGIA_E_ARG, "unknown mode %d", mode);
  const size_t nj = b->jobs.size();
  if (mode == NGIA_MODE_PLAIN) {
    // one job after the other, host loop per representative
    for (size_t j = 0; j < nj; j++) {
      ngia_ctx *c = b->jobs[j];
      c->tuned_warp_pairs = -1;
      int rc = ngia_cluster_begin(c, &params[j], NGIA_MODE_PLAIN);
      if (rc) return rc;
      int32_t done = 0;
      rc = ngia_cluster_step(c, max_iters, &done);
      if (rc) return rc;
    }
  } else {
    // every job's graph (built once per parameter set) is launched on the
    // job's own stream before any of them is waited for
    for (size_t j = 0; j < nj; j++) {
      ngia_ctx *c = b->jobs[j];
      // jobs running side by side fill the GPU: one thread per pair, the
      // form with the fewest instructions per cell (256-job batch on GB300:
      // 15.4M vs 13.0M candidate seqs/s with warp-per-pair classes)
      c->tuned_warp_pairs = 0;
      int rc = ngia_cluster_begin(c, &params[j], NGIA_MODE_GRAPH);
      if (rc) return rc;
      c->h_state->iter_limit = max_iters > 0 ? max_iters : INT64_MAX;
      CKB(cudaMemcpyAsync(&c->rb.st->iter_limit, &c->h_state->iter_limit, sizeof(int64_t),
                          cudaMemcpyHostToDevice, c->stream));
      CKB(cudaGraphLaunch(c->graph_exec, c->stream));
    }
  }
  ngia_stats sum;
  std::memset(&sum, 0, sizeof(sum));
  for (size_t j = 0; j < nj; j++) {
    ngia_ctx *c = b->jobs[j];
    int rc = ngia_cluster_end(c, cluster_out ? cluster_out[j] : nullptr, identity_out ? identity_out[j] : nullptr,
                              nullptr);
    if (rc) return rc;
    if (max_iters <= 0 && !c->h_state->done)
      return fail(NGIA_E_STATE, "ngia_batch_run: job %zu stopped before every sequence was assigned", j);
    ngia_stats s;
    ngia::drv::fill_stats(c, &s);
    sum.iterations += s.iterations;
    sum.candidates += s.candidates;
    sum.base_pass += s.base_pass;
    sum.align_pairs += s.align_pairs;
    sum.members += s.members;
    sum.band_cells += s.band_cells;
    sum.filter_bytes += s.filter_bytes;
    sum.word_checks += s.word_checks;
    sum.done_cells += s.done_cells;
  }
  if (stats) *stats = sum;
  return NGIA_OK;
}

extern "C" int ngia_batch_close(ngia_batch *b) {
  if (!b) return NGIA_OK;
  for (ngia_ctx *c : b->jobs) ngia_close(c);
  delete b;
  return NGIA_OK;
}
