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

namespace {
thread_local std::string g_tape_error;
}

extern "C" {

gpc_status gpc_tape_lower(const char *stim_text, size_t len, int32_t correlation_level, gpc_tape **out) {
  if (!out || !stim_text) return GPC_ERR_INVALID;
  *out = nullptr;
  try {
    gpc::LowerOptions lo;
    lo.level = correlation_level;
    lo.segment_occ = 8192;  // as a compile lowers it
    std::unique_ptr<gpc_tape> t(new gpc_tape{});
    gpc::LowerScratch scratch;
    if (len >= 64 * 1024) {  // a large text is parsed in pieces, as the compile path does
      gpc::HostPool pool(3);
      gpc::lower_text(stim_text, len, lo, t->t, scratch, &pool);
    } else {
      gpc::lower_text(stim_text, len, lo, t->t, scratch);
    }
    *out = t.release();
    return GPC_OK;
  } catch (const gpc::Error &e) {
    g_tape_error = e.what();
    return e.code;
  } catch (const std::bad_alloc &) {
    return GPC_ERR_OOM;
  } catch (const std::exception &e) {
    g_tape_error = e.what();
    return GPC_ERR_INVALID;
  }
}

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
