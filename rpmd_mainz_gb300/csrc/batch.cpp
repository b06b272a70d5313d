// batch.cpp -- independent ring-polymer trajectories advanced together.
//
// The reference runs one trajectory per process (md_eq.f90:182-323).  A batch
// holds resident contexts of any molecule and bead counts, each with its own
// parameters (gbrpmd_ctx_set_params), time step, temperature and Andersen
// random stream, and advances all of them by one evolve_pi step per graph
// launch: the replicas' steps are captured into one CUDA graph, one branch per
// replica forked from and joined back to the batch stream, so that their
// kernels overlap on the device.  The first step after a change of membership
// runs the branches as ordinary launches on the replicas' streams (it also
// performs any lazy set-up); the next one is captured; later steps replay.
//
// The Andersen test of md_eq (md_eq.f90:311-315) stays on the host: after each
// step, every replica with thresh > 0 draws ran2 from its own stream (its own
// saved generator state, so that it is the stream the replica would draw
// alone) and, on a collision, momenta from sample_rpmd are copied in on the
// batch stream.  Neither the draws nor the new momenta depend on the device
// state, so the host does this work while the step it follows still runs:
// the momenta go into a pinned staging buffer that is copied on the batch
// stream behind that step, and a buffer is reused only once its copy is done
// (an event per buffer).  No step waits for the host.
//
// Work runs on the batch stream: call gbrpmd_batch_sync before using a
// replica's context directly (gbrpmd_ctx_sync, gbrpmd_ctx_download), and do
// not queue work on a replica's context while it is in a batch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "gb_common.h"
#include "gb_context.h"
#include "gb_rng.h"

int ctx_set_error(int code, const std::string &msg);
int ctx_check_cuda(cudaError_t e, const char *what);

struct gb_batch {
  struct Rep {
    gb_context *c = nullptr;
    double dt = 0, beta = 0, thresh = 0;
    int irun = 0;
    std::vector<double> hmass;
    RngState rng;  // this replica's ran2 / gaussian state
    cudaEvent_t join = nullptr;
    int64_t launches = 0;  // this replica's kernels in the captured step
    EnergyPlan plan;       // and its accumulator plan
  };
  cudaStream_t s0 = nullptr;
  cudaEvent_t fork = nullptr;
  std::vector<Rep> reps;
  // pinned staging buffers of resampled momenta, each free again once the
  // copy recorded in its event has run
  struct Stage {
    double *h = nullptr;
    size_t cap = 0;
    cudaEvent_t done = nullptr;
  };
  std::vector<Stage> stages;
  cudaGraphExec_t exec = nullptr;
  bool valid = false;
  int seen = 0;
  int64_t steps = 0;
  bool graphs = true;  // GBRPMD_BATCH_GRAPHS=0: every step as ordinary launches
};

namespace {

#define BCK(x)                                                  \
  do {                                                          \
    cudaError_t e_ = (x);                                       \
    if (e_ != cudaSuccess) return ctx_check_cuda(e_, #x);       \
  } while (0)

void drop_graph(gb_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  b->exec = nullptr;
  b->valid = false;
  b->seen = 0;
}

// every replica's step on its own stream, forked from and joined to s0
int run_branches(gb_batch *b) {
  BCK(cudaEventRecord(b->fork, b->s0));
  for (auto &r : b->reps) {
    BCK(cudaStreamWaitEvent(r.c->stream, b->fork, 0));
    int st = dev_evolve_step(r.c, r.dt, r.beta);  // evolve_pi, or evolve_rig_pi for rigid water
    if (st) return st;
    BCK(cudaEventRecord(r.join, r.c->stream));
    BCK(cudaStreamWaitEvent(b->s0, r.join, 0));
  }
  return GB_OK;
}

// a staging buffer of at least n doubles whose last copy has run
int stage_for(gb_batch *b, size_t n, gb_batch::Stage **out) {
  for (auto &st : b->stages) {
    if (st.cap < n) continue;
    const cudaError_t q = cudaEventQuery(st.done);
    if (q == cudaSuccess) {
      *out = &st;
      return GB_OK;
    }
    if (q != cudaErrorNotReady) return ctx_check_cuda(q, "cudaEventQuery (batch staging)");
  }
  gb_batch::Stage st;
  BCK(cudaHostAlloc((void **)&st.h, sizeof(double) * n, cudaHostAllocDefault));
  st.cap = n;
  BCK(cudaEventCreateWithFlags(&st.done, cudaEventDisableTiming));
  b->stages.push_back(st);
  *out = &b->stages.back();
  return GB_OK;
}

int andersen(gb_batch *b) {
  for (auto &r : b->reps) {
    if (!(r.thresh > 0.0)) continue;
    if (rng_ran2(r.rng, &r.irun, 0.0, 1.0) < r.thresh) {
      const size_t n = 3 * (size_t)r.c->na * r.c->nb;
      gb_batch::Stage *st = nullptr;
      int e = stage_for(b, n, &st);
      if (e) return e;
      rng_sample_rpmd(r.rng, st->h, r.c->na, r.c->nb, r.hmass.data(), r.beta, &r.irun);
      BCK(cudaMemcpyAsync(r.c->p, st->h, sizeof(double) * n, cudaMemcpyHostToDevice, b->s0));
      BCK(cudaEventRecord(st->done, b->s0));
    }
  }
  return GB_OK;
}

}  // namespace

extern "C" {

int gbrpmd_batch_create(gb_batch **out) {
  if (!out) return ctx_set_error(GB_E_ARG, "null argument");
  gb_batch *b = new gb_batch();
  if (cudaStreamCreateWithFlags(&b->s0, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess) {
    delete b;
    return ctx_set_error(GB_E_CUDA, "batch stream or event creation failed");
  }
  if (const char *e = std::getenv("GBRPMD_BATCH_GRAPHS")) b->graphs = e[0] != '0';
  *out = b;
  return GB_OK;
}

int gbrpmd_batch_destroy(gb_batch *b) {
  if (!b) return GB_OK;
  cudaStreamSynchronize(b->s0);
  drop_graph(b);
  for (auto &r : b->reps)
    if (r.join) cudaEventDestroy(r.join);
  for (auto &st : b->stages) {
    cudaEventDestroy(st.done);
    cudaFreeHost(st.h);
  }
  cudaEventDestroy(b->fork);
  cudaStreamDestroy(b->s0);
  delete b;
  return GB_OK;
}

int gbrpmd_batch_add(gb_batch *b, gb_context *c, double dt, double beta, double thresh, int irun) {
  if (!b || !c) return ctx_set_error(GB_E_ARG, "null argument");
  if (!c->own_params) return ctx_set_error(GB_E_ARG, "a batch replica needs its own parameters (gbrpmd_ctx_set_params)");
  if (c->nbaro) return ctx_set_error(GB_E_UNSUPPORTED, "a batch replica cannot run a barostat (it synchronises each step)");
  if ((c->P.therm == GB_THERM_PRG || c->P.therm == GB_THERM_PRL) && c->rng_mode != GB_RNG_DEVICE)
    return ctx_set_error(GB_E_UNSUPPORTED,
                         "a batch replica with PRG/PRL kicks needs the device random stream (gbrpmd_ctx_set_rng_mode)");
  for (auto &r : b->reps)
    if (r.c == c) return ctx_set_error(GB_E_ARG, "context already in the batch");
  BCK(cudaStreamSynchronize(b->s0));
  BCK(cudaStreamSynchronize(c->stream));  // work queued on the context's own stream is done
  gb_batch::Rep r;
  r.c = c;
  r.dt = dt;
  r.beta = beta;
  r.thresh = thresh;
  r.irun = irun;
  if (thresh > 0.0) {
    r.hmass.resize(c->na);
    BCK(cudaMemcpyAsync(r.hmass.data(), c->mass, sizeof(double) * c->na, cudaMemcpyDeviceToHost, c->stream));
    BCK(cudaStreamSynchronize(c->stream));
  }
  BCK(cudaEventCreateWithFlags(&r.join, cudaEventDisableTiming));
  b->reps.push_back(std::move(r));
  drop_graph(b);
  return GB_OK;
}

int gbrpmd_batch_remove(gb_batch *b, gb_context *c) {
  if (!b || !c) return ctx_set_error(GB_E_ARG, "null argument");
  BCK(cudaStreamSynchronize(b->s0));
  for (size_t i = 0; i < b->reps.size(); ++i) {
    if (b->reps[i].c == c) {
      cudaEventDestroy(b->reps[i].join);
      b->reps.erase(b->reps.begin() + i);
      drop_graph(b);
      return GB_OK;
    }
  }
  return ctx_set_error(GB_E_ARG, "context not in the batch");
}

int gbrpmd_batch_size(gb_batch *b) { return b ? (int)b->reps.size() : 0; }

int gbrpmd_batch_step(gb_batch *b, int nsteps) {
  if (!b) return ctx_set_error(GB_E_ARG, "null batch");
  if (b->reps.empty()) return GB_OK;
  for (int s = 0; s < nsteps; ++s) {
    for (auto &r : b->reps) {
      if (r.c->prof) drop_graph(b);  // profiled steps run as ordinary launches
      r.c->last_beta = r.beta;
    }
    if (b->valid) {
      BCK(cudaGraphLaunch(b->exec, b->s0));
      for (auto &r : b->reps) {
        r.c->launches += r.launches;
        r.c->plan = r.plan;
      }
    } else if (b->seen < 1 || !b->graphs) {
      int st = run_branches(b);
      if (st) return st;
      b->seen += 1;
    } else {
      std::vector<int64_t> l0;
      for (auto &r : b->reps) {
        int sp = dev_prepare(r.c, r.dt, r.beta);  // set-up copies synchronise: never inside the capture
        if (sp) return sp;
        dev_graph_reset(r.c);  // nor a graph destruction
        l0.push_back(r.c->launches);
      }
      BCK(cudaStreamBeginCapture(b->s0, cudaStreamCaptureModeThreadLocal));
      int st = run_branches(b);
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamEndCapture(b->s0, &g);
      if (st) {
        if (g) cudaGraphDestroy(g);
        return st;
      }
      if (e != cudaSuccess) return ctx_check_cuda(e, "cudaStreamEndCapture (batch)");
      e = cudaGraphInstantiate(&b->exec, g, cudaGraphInstantiateFlagUseNodePriority);
      cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        b->exec = nullptr;
        return ctx_check_cuda(e, "cudaGraphInstantiate (batch)");
      }
      b->valid = true;
      for (size_t i = 0; i < b->reps.size(); ++i) {
        b->reps[i].launches = b->reps[i].c->launches - l0[i];
        b->reps[i].plan = b->reps[i].c->plan;
        dev_graph_reset(b->reps[i].c);  // the context's own step graph would not know about the batch
      }
      BCK(cudaGraphLaunch(b->exec, b->s0));  // the captured step has not run yet
    }
    int st = andersen(b);
    if (st) return st;
    b->steps += 1;
  }
  return GB_OK;
}

int gbrpmd_ctx_autotune(gb_context *c, double dt, double beta, int steps, double *out6);  // tune.cpp

// launch shapes of every replica (gbrpmd_ctx_autotune; shapes seen before
// come from the process-wide cache), then a fresh capture at the next step
int gbrpmd_batch_autotune(gb_batch *b, int steps) {
  if (!b) return ctx_set_error(GB_E_ARG, "null batch");
  BCK(cudaStreamSynchronize(b->s0));
  for (auto &r : b->reps) {
    int st = gbrpmd_ctx_autotune(r.c, r.dt, r.beta, steps, nullptr);
    if (st) return st;
  }
  drop_graph(b);
  return GB_OK;
}

int gbrpmd_batch_sync(gb_batch *b) {
  if (!b) return ctx_set_error(GB_E_ARG, "null batch");
  BCK(cudaStreamSynchronize(b->s0));
  return GB_OK;
}

void *gbrpmd_batch_stream(gb_batch *b) { return b ? (void *)b->s0 : nullptr; }

}  // extern "C"
