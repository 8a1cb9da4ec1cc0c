// ctx.h — the library context behind the opaque ngia_ctx handle and the
// host-side launchers each kernel translation unit provides.
#pragma once
#include <cuda_runtime.h>

#include <vector>

#include "../../include/ngia.h"
#include "common.cuh"

struct ngia_spec;  // speculative-round driver state (spec.cu)
static_assert(ngia::kNumClasses == 7, "per-class initialisers of ngia_ctx");

struct ngia_ctx {
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  ngia::DevDB db{};
  // owned device allocations of the database
  uint32_t *d_words = nullptr;
  int64_t *d_off = nullptr;
  int32_t *d_len = nullptr, *d_net = nullptr;
  uint32_t *d_cnt = nullptr;
  uint32_t *d_codes = nullptr;  // protein residue-code streams (DevDB::codes)
  int64_t n_words = 0;
  int32_t longest = 0;
  // capacity of the allocations (a context can be reloaded with any database
  // within it: serving slots)
  int64_t cap_n = 0, cap_words = 0;
  int32_t cap_nb = 0;
  int32_t *d_flags = nullptr;  // loader results: max blocks, short record, bad record
  int32_t *h_flags = nullptr;  // pinned mirror
  // run buffers
  ngia::RunBufs rb{};
  ngia::RunState *h_state = nullptr;  // pinned mirror
  ngia::RunParams prm{};
  int mode = 0;
  bool begun = false;
  // launch shapes
  int grid_filter = 0;
  int grid_align[ngia::kNumClasses] = {0};
  int grid_warp = 0;    // CTAs of the warp-per-pair kernel
  int warp_pairs = -1;  // a class with at most this many pairs runs warp-per-pair
  int warp_pairs_default = -1;  // the above as sized for this context's grids
  // settings that change speed only (set by ngia_autotune / ngia_set_tuning):
  // test order (0 auto, 1 short words first, 2 alignment first), lockstep
  // refill threshold, warp-per-pair cut-off (-1: keep warp_pairs_default)
  int tuned_word_order = 0, tuned_refill = 32, tuned_warp_pairs = -1;
  // per length bucket (alignment class): warp-per-pair cut-off (-1: the
  // context's) and CTA divisor; the composition filter's words per warp
  int cls_warp_pairs[ngia::kNumClasses] = {-1, -1, -1, -1, -1, -1, -1};
  int cls_grid_div[ngia::kNumClasses] = {1, 1, 1, 1, 1, 1, 1};
  int filter_tile = 8;
  int tune_gen = 0;             // bumped by every change of the settings above
  int graph_tune_gen = -1;      // tune_gen the captured graph was built with
  int graph_warp_pairs = -1;    // warp_pairs the captured graph was built with
  // graph form of the greedy loop
  cudaGraphExec_t graph_exec = nullptr;
  cudaGraph_t graph = nullptr;
  bool graph_ready = false;
  ngia::RunParams graph_prm{};
  cudaStream_t side[ngia::kNumClasses] = {nullptr};
  cudaEvent_t fork_ev = nullptr, join_ev[ngia::kNumClasses] = {nullptr};
  // timing: whole steps, and (profiling, plain form) filter / align stages
  cudaEvent_t ev_step0 = nullptr, ev_step1 = nullptr, ev_p0 = nullptr, ev_p1 = nullptr, ev_p2 = nullptr;
  cudaEvent_t ev_cls[ngia::kNumClasses + 1] = {nullptr};
  bool profiling = false;
  bool batch_member = false;  // grids sized to the job; serial class launches
  double ms_filter = 0.0, ms_align = 0.0, ms_class[ngia::kNumClasses] = {0.0};
  float last_step_ms = 0.f;
  ngia_spec *spec = nullptr;  // NGIA_MODE_SPEC buffers, allocated on first use
};

namespace ngia {
// api.cu: driver internals shared with batch.cu / serve.cu
namespace drv {
int open_ctx(const ngia_db_view *v, bool batch_member, ngia_ctx **out);
// A context with room for cap_n records, cap_words record words and records
// of up to cap_nb plane blocks, holding no database until reload_ctx.
int open_ctx_capacity(int type, int64_t cap_n, int64_t cap_words, int cap_nb, ngia_ctx **out);
// Loads a database within the capacity (stream-ordered copies on the
// context's stream; waits for that stream only).
int reload_ctx(ngia_ctx *c, const ngia_db_view *v);
// begin a run whose unclustered set is the given device bitmap (bit i =
// sequence i takes part), instead of every sequence.
int begin_subset(ngia_ctx *c, const ngia_params *p, int32_t mode, const uint32_t *d_alive);
// graph form of the greedy loop (captured once per parameter set)
int build_graph(ngia_ctx *c);
int ensure_graph(ngia_ctx *c);  // build_graph unless the captured one is current
void destroy_graph(ngia_ctx *c);
int pull_state(ngia_ctx *c);
int enqueue_iteration(ngia_ctx *c, bool graph, cudaGraphConditionalHandle cond);
void fill_stats(const ngia_ctx *c, ngia_stats *stats);
int validate_params(int type, const ngia_params *p);
// spec.cu: speculative rounds (NGIA_MODE_SPEC)
int spec_prepare(ngia_ctx *c);                 // buffers for the context's capacity; zeroed masks
int spec_step(ngia_ctx *c, int64_t max_iters);  // up to max_iters representatives (<= 0: all)
void spec_free(ngia_ctx *c);
bool spec_exact(const ngia_ctx *c);            // rounds reproduce the greedy loop exactly
void spec_stats(const ngia_ctx *c, int64_t *pairs, int64_t *cells);
}  // namespace drv
// loader.cu / filter.cu
cudaError_t launch_loader(ngia_ctx *c, int32_t *d_maxnb, int32_t *d_short, int32_t *d_bad);
cudaError_t launch_init_run(ngia_ctx *c);
cudaError_t launch_prep(ngia_ctx *c, int score_rep);
cudaError_t launch_filter(ngia_ctx *c);
cudaError_t launch_next(ngia_ctx *c, unsigned long long cond_handle, int use_cond);
cudaError_t launch_subset_start(ngia_ctx *c, const uint32_t *d_alive);
cudaError_t launch_score_classify(ngia_ctx *c, int n);
// align.cu
cudaError_t launch_align(ngia_ctx *c, int cls, cudaStream_t s, int score_mode);
int align_occupancy(int type, int cls, int max_nb);
int align_threads();
cudaError_t align_configure(int type, int max_nb);
cudaError_t filter_configure();
// pool.cu: the pooled batch form (NGIA_MODE_POOL), one pool per record type
namespace pool {
struct Group;
int group_open(const std::vector<ngia_ctx *> &jobs, Group **out);  // jobs of one type
int group_fill(Group *g, cudaStream_t s);  // the jobs' current run buffers and parameters
int group_enqueue_round(Group *g, cudaStream_t s, cudaGraphConditionalHandle cond);
int group_size(const Group *g);
void group_close(Group *g);
}  // namespace pool
}  // namespace ngia
