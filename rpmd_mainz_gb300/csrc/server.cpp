// server.cpp -- a request loop over the batch: continuous batching of
// independent RPMD trajectories with resident state.
//
// A request names a system (na, nb, its own gb_params, masses, charges, box),
// its starting state in host arrays owned by the caller, a number of evolve_pi
// steps, dt, beta and an optional Andersen test.  Requests wait in arrival
// order; at each tick the server admits from the head of the queue while a slot
// is free and the request's estimated device footprint
// (gbrpmd_estimate_device_bytes) fits in the memory budget next to the
// trajectories already resident, creates the request's context, uploads its
// state and adds it to the running batch.  The tick then advances the batch
// (one CUDA-graph launch per step for all resident trajectories), retires the
// trajectories that reached their step count -- final r, p, dvdr, dvdr2 copied
// into the caller's arrays, energies recorded, context freed -- and so makes
// room for the next requests.  Times (submit, admission, completion) come from
// the host's steady clock.
#include <cuda_runtime.h>

#include <chrono>
#include <cstring>
#include <deque>
#include <vector>

#include "gb_common.h"
#include "gb_context.h"

int ctx_set_error(int code, const std::string &msg);

struct gb_request {
  int64_t id = 0;
  int na = 0, nb = 0, nsteps = 0, done = 0, irun = 0, forces_given = 1;
  gb_params P{};
  double dt = 0, beta = 0, thresh = 0, box[3] = {0, 0, 0};
  const double *mass = nullptr, *z = nullptr;
  double *r = nullptr, *p = nullptr, *dvdr = nullptr, *dvdr2 = nullptr;
  gb_context *ctx = nullptr;
  size_t bytes = 0;
  double t_submit = 0, t_admit = 0, t_finish = 0;
  double energies[5] = {0, 0, 0, 0, 0};
  int status = GB_OK;
};

struct gb_server {
  size_t budget = 0, in_use = 0;
  int max_slots = 0;
  gb_batch *batch = nullptr;
  std::deque<gb_request *> queue;
  std::vector<gb_request *> active, finished;
  int64_t next_id = 1;
  std::chrono::steady_clock::time_point t0;
  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

extern "C" {
int gbrpmd_batch_create(gb_batch **batch);
int gbrpmd_batch_destroy(gb_batch *batch);
int gbrpmd_batch_add(gb_batch *batch, gb_context *ctx, double dt, double beta, double thresh, int irun);
int gbrpmd_batch_remove(gb_batch *batch, gb_context *ctx);
int gbrpmd_batch_step(gb_batch *batch, int nsteps);
int gbrpmd_batch_sync(gb_batch *batch);
int gbrpmd_ctx_create(gb_context **ctx, int na, int nb, const double *mass, const double *z);
int gbrpmd_ctx_destroy(gb_context *ctx);
int gbrpmd_ctx_set_params(gb_context *ctx, const gb_params *params);
int gbrpmd_ctx_upload(gb_context *c, const double *r, const double *p, const double *dvdr, const double *dvdr2,
                      const double *boxlxyz);
int gbrpmd_ctx_download(gb_context *c, double *r, double *p, double *dvdr, double *dvdr2);
int gbrpmd_ctx_full_forces(gb_context *c, double *v, double *vew, double *voo, double *vint, double *vir);
int gbrpmd_ctx_sync(gb_context *c);
int gbrpmd_ctx_energies(gb_context *c, double *out5, double *vir, double *vir_lf);
}

namespace {

// creates the request's context, uploads its state (forces from full_forces
// when the request brings none) and adds it to the batch
int admit(gb_server *s, gb_request *q) {
  int st = gbrpmd_ctx_create(&q->ctx, q->na, q->nb, q->mass, q->z);
  if (st) return st;
  if ((st = gbrpmd_ctx_set_params(q->ctx, &q->P))) return st;
  if ((st = gbrpmd_ctx_upload(q->ctx, q->r, q->p, q->forces_given ? q->dvdr : nullptr,
                               q->forces_given ? q->dvdr2 : nullptr, q->box)))
    return st;
  if (!q->forces_given) {
    double v, vew, voo, vint, vir[9];
    if ((st = gbrpmd_ctx_full_forces(q->ctx, &v, &vew, &voo, &vint, vir))) return st;
  }
  if ((st = gbrpmd_ctx_sync(q->ctx))) return st;
  return gbrpmd_batch_add(s->batch, q->ctx, q->dt, q->beta, q->thresh, q->irun);
}

int retire(gb_server *s, gb_request *q) {
  int st = gbrpmd_batch_remove(s->batch, q->ctx);  // synchronises the batch stream
  if (!st) st = gbrpmd_ctx_sync(q->ctx);
  if (!st) st = gbrpmd_ctx_energies(q->ctx, q->energies, nullptr, nullptr);
  if (!st) st = gbrpmd_ctx_download(q->ctx, q->r, q->p, q->dvdr, q->dvdr2);
  gbrpmd_ctx_destroy(q->ctx);
  q->ctx = nullptr;
  s->in_use -= q->bytes;
  q->status = st;
  q->t_finish = s->now();
  return st;
}

}  // namespace

extern "C" {

int gbrpmd_server_create(gb_server **out, size_t budget_bytes, int max_slots) {
  if (!out || max_slots <= 0) return ctx_set_error(GB_E_ARG, "server: null handle or no slots");
  gb_server *s = new gb_server();
  s->budget = budget_bytes;
  s->max_slots = max_slots;
  s->t0 = std::chrono::steady_clock::now();
  int st = gbrpmd_batch_create(&s->batch);
  if (st) {
    delete s;
    return st;
  }
  *out = s;
  return GB_OK;
}

int gbrpmd_server_destroy(gb_server *s) {
  if (!s) return GB_OK;
  gbrpmd_batch_sync(s->batch);
  for (gb_request *q : s->active) {
    gbrpmd_batch_remove(s->batch, q->ctx);
    gbrpmd_ctx_destroy(q->ctx);
    delete q;
  }
  for (gb_request *q : s->queue) delete q;
  for (gb_request *q : s->finished) delete q;
  gbrpmd_batch_destroy(s->batch);
  delete s;
  return GB_OK;
}

int gbrpmd_server_submit(gb_server *s, int na, int nb, const gb_params *params, const double *mass,
                         const double *z, const double *boxlxyz, double *r, double *p, double *dvdr,
                         double *dvdr2, int forces_given, int nsteps, double dt, double beta, double thresh,
                         int irun, int64_t *id) {
  if (!s || !params || !mass || !z || !boxlxyz || !r || !p || !dvdr || !dvdr2 || nsteps < 0)
    return ctx_set_error(GB_E_ARG, "server: incomplete request");
  gb_request *q = new gb_request();
  q->id = s->next_id++;
  q->na = na;
  q->nb = nb;
  q->P = *params;
  q->mass = mass;
  q->z = z;
  std::memcpy(q->box, boxlxyz, sizeof(q->box));
  q->r = r;
  q->p = p;
  q->dvdr = dvdr;
  q->dvdr2 = dvdr2;
  q->forces_given = forces_given ? 1 : 0;
  q->nsteps = nsteps;
  q->dt = dt;
  q->beta = beta;
  q->thresh = thresh;
  q->irun = irun;
  q->bytes = dev_estimate_bytes(na, nb, q->P);
  q->t_submit = s->now();
  if (q->bytes > s->budget) {
    delete q;
    return ctx_set_error(GB_E_NOMEM, "server: request larger than the whole memory budget");
  }
  s->queue.push_back(q);
  if (id) *id = q->id;
  return GB_OK;
}

// admits what fits, advances every resident trajectory by up to `steps` steps
// (fewer when one of them finishes earlier) and retires the finished ones
int gbrpmd_server_tick(gb_server *s, int steps) {
  if (!s || steps <= 0) return ctx_set_error(GB_E_ARG, "server: bad tick");
  while (!s->queue.empty() && (int)s->active.size() < s->max_slots &&
         s->in_use + s->queue.front()->bytes <= s->budget) {
    gb_request *q = s->queue.front();
    s->queue.pop_front();
    q->t_admit = s->now();
    int st = admit(s, q);
    if (st) {
      if (q->ctx) gbrpmd_ctx_destroy(q->ctx);
      q->ctx = nullptr;
      q->status = st;
      q->t_finish = s->now();
      s->finished.push_back(q);
      continue;
    }
    s->in_use += q->bytes;
    s->active.push_back(q);
  }
  if (s->active.empty()) return GB_OK;
  int k = steps;
  for (gb_request *q : s->active) k = std::min(k, q->nsteps - q->done);
  if (k > 0) {
    int st = gbrpmd_batch_step(s->batch, k);
    if (st) return st;
    for (gb_request *q : s->active) q->done += k;
  }
  for (size_t i = 0; i < s->active.size();) {
    gb_request *q = s->active[i];
    if (q->done >= q->nsteps) {
      retire(s, q);
      s->finished.push_back(q);
      s->active.erase(s->active.begin() + i);
    } else {
      ++i;
    }
  }
  return GB_OK;
}

int gbrpmd_server_counts(gb_server *s, int *queued, int *active, int *finished, size_t *bytes_in_use) {
  if (!s) return ctx_set_error(GB_E_ARG, "null server");
  if (queued) *queued = (int)s->queue.size();
  if (active) *active = (int)s->active.size();
  if (finished) *finished = (int)s->finished.size();
  if (bytes_in_use) *bytes_in_use = s->in_use;
  return GB_OK;
}

// hands out finished requests: id, status, seconds from submit to admission
// and to completion, energies (v, vew, vlj, vint, tv of the last step)
int gbrpmd_server_poll(gb_server *s, int max, int64_t *ids, int *status, double *t_admit, double *t_done,
                       double *energies5, int *n) {
  if (!s || !n) return ctx_set_error(GB_E_ARG, "null argument");
  int m = 0;
  while (m < max && !s->finished.empty()) {
    gb_request *q = s->finished.front();
    s->finished.erase(s->finished.begin());
    if (ids) ids[m] = q->id;
    if (status) status[m] = q->status;
    if (t_admit) t_admit[m] = q->t_admit - q->t_submit;
    if (t_done) t_done[m] = q->t_finish - q->t_submit;
    if (energies5)
      for (int e = 0; e < 5; ++e) energies5[5 * m + e] = q->energies[e];
    delete q;
    ++m;
  }
  *n = m;
  return GB_OK;
}

}  // extern "C"
