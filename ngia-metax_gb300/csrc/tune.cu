// tune.cu — run-time tuning of the settings that change the speed of a run
// but never its result: the order of the two cheap tests, the lockstep
// refill threshold of the tiled alignment and the warp-per-pair cut-off.
// Each candidate is timed (device time, graph driver) on the first greedy
// iterations of a fresh run of the context's database; the fastest is kept
// for the context's later runs.  The candidates: the default; each test
// order; refill 24 and 28; the warp cut-off at a quarter, half and twice the
// default.  Coordinate-wise: the best test order is kept while the refill
// and the cut-off are tried.
#include <cstring>
#include <vector>

#include "../host/host_common.h"
#include "ctx.h"

using ngia::fail;

namespace {

// Device time per iteration of `iters` fresh iterations with these settings
// (one untimed run first: graph capture and warm caches).
int time_setting(ngia_ctx *c, const ngia_params *p, int32_t iters, int word_order, int refill, int warp_pairs,
                 double *ms_per_iter) {
  c->tuned_word_order = word_order;
  c->tuned_refill = refill;
  c->tuned_warp_pairs = warp_pairs;
  float total = 0.f;
  int64_t done_iters = 0;
  for (int rep = 0; rep < 2; rep++) {
    int rc = ngia_cluster_begin(c, p, NGIA_MODE_GRAPH);
    if (rc) return rc;
    int32_t done = 0;
    rc = ngia_cluster_step(c, iters, &done);
    if (rc) return rc;
    if (rep == 1) {
      rc = ngia_step_device_ms(c, &total);
      if (rc) return rc;
      done_iters = c->h_state->iter;
    }
  }
  *ms_per_iter = done_iters > 0 ? total / (double)done_iters : 0.0;
  return NGIA_OK;
}

}  // namespace

extern "C" int ngia_autotune(ngia_ctx *c, const ngia_params *p, int32_t iters, ngia_tuning *out) {
  ngia::clear_error();
  if (!c || !p || iters <= 0) return fail(NGIA_E_ARG, "ngia_autotune: bad argument");
  int rc = ngia::drv::validate_params(c->db.type, p);
  if (rc) return rc;
  const int def_wp = c->warp_pairs_default;
  int best_wo = 0, best_rf = 32, best_wp = -1, count = 0;
  double best = 0.0, base = 0.0;
  auto trial = [&](int wo, int rf, int wp) -> int {
    double ms = 0.0;
    const int r = time_setting(c, p, iters, wo, rf, wp, &ms);
    if (r) return r;
    count++;
    if (count == 1) base = ms;
    if (count == 1 || ms < best) {
      best = ms;
      best_wo = wo;
      best_rf = rf;
      best_wp = wp;
    }
    return NGIA_OK;
  };
  rc = trial(0, 32, -1);  // the default
  for (int wo : {1, 2})
    if (!rc && !(c->db.has_short && !p->precise && wo == 2)) rc = trial(wo, 32, -1);  // short records: word first
  const int wo = best_wo;
  for (int rf : {24, 28})
    if (!rc) rc = trial(wo, rf, best_wp);
  const int rf = best_rf;
  for (int wp : {def_wp / 4, def_wp / 2, def_wp * 2})
    if (!rc) rc = trial(wo, rf, wp);
  if (rc) {
    c->tuned_word_order = 0;
    c->tuned_refill = 32;
    c->tuned_warp_pairs = -1;
    return rc;
  }
  c->tuned_word_order = best_wo;
  c->tuned_refill = best_rf;
  c->tuned_warp_pairs = best_wp;
  c->warp_pairs = best_wp >= 0 ? best_wp : def_wp;
  c->begun = false;
  if (out) {
    out->word_order = best_wo;
    out->refill = best_rf;
    out->warp_pairs = best_wp;
    out->candidates = count;
    out->ms_per_iter = best;
    out->default_ms_per_iter = base;
  }
  return NGIA_OK;
}

extern "C" int ngia_set_tuning(ngia_ctx *c, const ngia_tuning *t) {
  ngia::clear_error();
  if (!c || !t) return fail(NGIA_E_ARG, "ngia_set_tuning: null argument");
  if (t->word_order < 0 || t->word_order > 2 || t->refill < 1 || t->refill > 32 || t->warp_pairs < -1)
    return fail(NGIA_E_ARG, "ngia_set_tuning: setting out of range");
  c->tuned_word_order = t->word_order;
  c->tuned_refill = t->refill;
  c->tuned_warp_pairs = t->warp_pairs;
  c->warp_pairs = t->warp_pairs >= 0 ? t->warp_pairs : c->warp_pairs_default;
  return NGIA_OK;
}
