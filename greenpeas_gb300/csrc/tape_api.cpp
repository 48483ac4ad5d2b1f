// tape_api.cpp -- host-only C ABI that exposes the lowered tape (include/gpc.h).
#include <memory>
#include <new>
#include <string>
#include <vector>

#include "../../include/gpc.h"
#include "host_pool.hpp"
#include "lower.hpp"

struct gpc_tape {
  gpc::Tape t;
};

struct gpc_lowerer {
  gpc::LowerOptions lo;
  gpc::LowerScratch scratch;
};

namespace {
thread_local std::string g_tape_error;

template <typename F>
gpc_status tape_guarded(F &&f) {
  try {
    f();
    return GPC_OK;
  } catch (const gpc::Error &e) {
    g_tape_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    g_tape_error = "host allocation failed";
    return GPC_ERR_OOM;
  } catch (const std::exception &e) {
    g_tape_error = e.what();
    return GPC_ERR_INVALID;
  }
}

// A lowering as a compile does it: a large text is parsed in pieces on a pool.
void lower_like_compile(const char *text, size_t len, const gpc::LowerOptions &lo, gpc::Tape &T,
                        gpc::LowerScratch &scratch) {
  if (len >= 64 * 1024) {
    gpc::HostPool pool(3);
    gpc::lower_text(text, len, lo, T, scratch, &pool);
  } else {
    gpc::lower_text(text, len, lo, T, scratch);
  }
}
}  // namespace

extern "C" {

gpc_status gpc_tape_lower(const char *stim_text, size_t len, int32_t correlation_level, gpc_tape **out) {
  if (!out || !stim_text) return GPC_ERR_INVALID;
  *out = nullptr;
  return tape_guarded([&] {
    gpc::LowerOptions lo;
    lo.level = correlation_level;
    lo.segment_occ = 8192;  // as a compile lowers it
    std::unique_ptr<gpc_tape> t(new gpc_tape{});
    gpc::LowerScratch scratch;
    lower_like_compile(stim_text, len, lo, t->t, scratch);
    *out = t.release();
  });
}

gpc_status gpc_tape_lower_cuts(const char *stim_text, size_t len, int32_t correlation_level, const uint64_t *cuts,
                               uint32_t ncuts, gpc_tape **out) {
  if (!out || !stim_text || (ncuts && !cuts)) return GPC_ERR_INVALID;
  *out = nullptr;
  return tape_guarded([&] {
    std::vector<size_t> c(cuts, cuts + ncuts);
    gpc::LowerOptions lo;
    lo.level = correlation_level;
    lo.segment_occ = 8192;
    lo.cuts = &c;
    std::unique_ptr<gpc_tape> t(new gpc_tape{});
    gpc::LowerScratch scratch;
    gpc::lower_text(stim_text, len, lo, t->t, scratch);
    *out = t.release();
  });
}

gpc_status gpc_lowerer_create(int32_t correlation_level, int32_t incremental, gpc_lowerer **out) {
  if (!out) return GPC_ERR_INVALID;
  *out = nullptr;
  if (correlation_level < 0 || correlation_level > 2) {
    g_tape_error = "correlation level must be 0, 1 or 2";
    return GPC_ERR_INVALID;
  }
  return tape_guarded([&] {
    std::unique_ptr<gpc_lowerer> lw(new gpc_lowerer{});
    lw->lo.level = correlation_level;
    lw->lo.segment_occ = 8192;  // as a compile lowers it
    lw->lo.incremental = incremental != 0;
    *out = lw.release();
  });
}

gpc_status gpc_lowerer_lower(gpc_lowerer *lowerer, const char *stim_text, size_t len, gpc_tape **out) {
  if (!lowerer || !out || !stim_text) return GPC_ERR_INVALID;
  *out = nullptr;
  return tape_guarded([&] {
    std::unique_ptr<gpc_tape> t(new gpc_tape{});
    gpc::lower_text(stim_text, len, lowerer->lo, t->t, lowerer->scratch);  // on this thread, as a batch's
    *out = t.release();
  });
}

gpc_status gpc_lowerer_stats(const gpc_lowerer *lowerer, gpc_lower_stats *stats, uint64_t *cuts, uint32_t cap,
                             uint32_t *ncuts) {
  if (!lowerer || (cap && !cuts)) return GPC_ERR_INVALID;
  const gpc::LowerScratch &S = lowerer->scratch;
  if (stats) {
    stats->incremental = S.stats.incremental ? 1u : 0u;
    stats->segments = S.stats.segments;
    stats->reused = S.stats.reused;
    stats->reserved = 0;
    stats->parsed_bytes = S.stats.parsed_bytes;
  }
  const std::vector<size_t> &c = S.last_cuts();
  if (ncuts) *ncuts = (uint32_t)c.size();
  if (c.size() > cap) return cap ? GPC_ERR_CAPACITY : GPC_OK;
  for (size_t i = 0; i < c.size(); ++i) cuts[i] = c[i];
  return GPC_OK;
}

void gpc_lowerer_free(gpc_lowerer *lowerer) { delete lowerer; }

const char *gpc_tape_last_error(void) { return g_tape_error.c_str(); }

gpc_status gpc_tape_get_view(const gpc_tape *tape, gpc_tape_view *v) {
  if (!tape || !v) return GPC_ERR_INVALID;
  const gpc::Tape &T = tape->t;
  v->num_qubits = T.nq;
  v->qpad = T.qpad;
  v->num_measurements = T.nmeas;
  v->num_detectors = T.ndet;
  v->num_observables = T.nobs;
  v->words = T.w;
  v->num_epochs = T.n_epochs;
  v->kmax = T.kmax;
  v->num_points = T.npoints;
  v->num_mechanisms = T.M;
  v->num_records = (uint32_t)T.rec.size();
  v->num_ops = T.ops.size();
  v->ops = T.ops.data();
  v->ep_opoff = T.ep_opoff.data();
  v->ep_k = T.ep_k.data();
  v->ep_ptoff = T.ep_ptoff.data();
  v->inj_lo = T.inj_lo.data();
  v->inj_hi = T.inj_hi.data();
  v->rec = T.rec.data();
  v->rec_p = T.rec_p.data();
  v->rec_moff = T.rec_moff.data();
  v->rec_src = T.rec_src.data();
  v->num_ticks = T.n_ticks;
  return GPC_OK;
}

gpc_status gpc_tape_walk_segments(const gpc_tape *tape, uint32_t target, uint32_t *bounds, uint32_t cap,
                                  uint32_t *n) {
  if (!tape || !n || (cap && !bounds)) return GPC_ERR_INVALID;
  std::vector<uint32_t> b;
  gpc::walk_segment_bounds(tape->t, target, b);
  *n = (uint32_t)b.size();
  if (b.size() > cap) return GPC_ERR_CAPACITY;
  for (size_t i = 0; i < b.size(); ++i) bounds[i] = b[i];
  return GPC_OK;
}

void gpc_tape_free(gpc_tape *tape) { delete tape; }
}
