// tune.cpp -- the library's autotuner for the launch shapes of one context.
//
// The reference has no counterpart (it runs one serial code path).  On the
// device the fastest launch shape of several kernels depends on the system:
// the lanes that share one site's pair list in the FP32 real-space Ewald and
// LJ kernels (more lanes give more warps for small systems, fewer lanes less
// reduction work for large ones), the molecules per block of the fused MTS
// kernel (occupancy against the one-wave grid), and the pair-list skin (larger
// lists against fewer rebuilds), the warps that share a block's sites in the
// FP32 k-space force kernel and the sites each of its lanes carries (more
// sites share each table load, fewer blocks fill the SMs).
// gbrpmd_ctx_autotune runs evolve_pi steps of the context itself with
// candidate shapes, one parameter at a time from the defaults (coordinate
// descent), restores the trajectory state after every trial and keeps the
// fastest shape.  A kernel's launch shape is judged on the median CUDA-event
// time of that kernel alone (list-rebuild steps do not decide); the skin, which
// trades pair count against rebuild frequency, on the mean time of whole steps
// over a longer trial.  Results are cached for the process per
// shape key (atoms, beads, precision, MTS, contraction, box kind, model), so a
// batch of many replicas tunes each distinct shape once.  The shapes change
// results only through the order of floating-point sums.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "gb_common.h"
#include "gb_context.h"

int ctx_set_error(int code, const std::string &msg);
int ctx_check_cuda(cudaError_t e, const char *what);
bool recip_force_tc_on(const gb_context *c);  // k_mixed.cu

namespace {

#define TCK(x)                                            \
  do {                                                    \
    cudaError_t e_ = (x);                                 \
    if (e_ != cudaSuccess) return ctx_check_cuda(e_, #x); \
  } while (0)

struct Shape {
  gb_context::Tune tune;
  double skin = 0.1;
};

using Key = std::tuple<int, int, int, int, int, int, int, int>;
std::map<Key, Shape> g_cache;

Key key_of(const gb_context *c) {
  const gb_params &P = c->P;
  return Key(c->na, c->nb, P.precision, P.mts, P.nbdf1, P.nbdf2, P.iamcub, P.intra_model);
}

// the trajectory arrays and host energies a trial must not disturb
struct Saved {
  double *dev = nullptr;
  size_t n = 0;
  double e[5], vir[9], vir_lf[9], vir_hf[9], vir_lf_in[9], box[3];
  unsigned long long ctr = 0;  // the device random stream's kick counter
};

int save(gb_context *c, Saved &S) {
  S.n = 3 * (size_t)c->na * c->nb;
  TCK(cudaMalloc(&S.dev, sizeof(double) * 4 * S.n));
  double *src[4] = {c->r, c->p, c->dvdr, c->dvdr2};
  for (int i = 0; i < 4; ++i)
    TCK(cudaMemcpyAsync(S.dev + i * S.n, src[i], sizeof(double) * S.n, cudaMemcpyDeviceToDevice, c->stream));
  S.e[0] = c->e_v, S.e[1] = c->e_vew, S.e[2] = c->e_vlj, S.e[3] = c->e_vint, S.e[4] = c->e_tv;
  std::memcpy(S.vir, c->e_vir, sizeof S.vir);
  std::memcpy(S.vir_lf, c->e_vir_lf, sizeof S.vir_lf);
  std::memcpy(S.vir_hf, c->e_vir_hf, sizeof S.vir_hf);
  std::memcpy(S.vir_lf_in, c->vir_lf_in, sizeof S.vir_lf_in);
  std::memcpy(S.box, c->box, sizeof S.box);
  if (c->d_rngctr) {
    TCK(cudaMemcpyAsync(&S.ctr, c->d_rngctr, sizeof S.ctr, cudaMemcpyDeviceToHost, c->stream));
    TCK(cudaStreamSynchronize(c->stream));
  }
  return GB_OK;
}

int restore(gb_context *c, const Saved &S) {
  double *dst[4] = {c->r, c->p, c->dvdr, c->dvdr2};
  for (int i = 0; i < 4; ++i)
    TCK(cudaMemcpyAsync(dst[i], S.dev + i * S.n, sizeof(double) * S.n, cudaMemcpyDeviceToDevice, c->stream));
  if (c->d_rngctr) TCK(cudaMemcpyAsync(c->d_rngctr, &S.ctr, sizeof S.ctr, cudaMemcpyHostToDevice, c->stream));
  TCK(cudaStreamSynchronize(c->stream));
  c->e_v = S.e[0], c->e_vew = S.e[1], c->e_vlj = S.e[2], c->e_vint = S.e[3], c->e_tv = S.e[4];
  std::memcpy(c->e_vir, S.vir, sizeof S.vir);
  std::memcpy(c->e_vir_lf, S.vir_lf, sizeof S.vir_lf);
  std::memcpy(c->e_vir_hf, S.vir_hf, sizeof S.vir_hf);
  std::memcpy(c->vir_lf_in, S.vir_lf_in, sizeof S.vir_lf_in);
  std::memcpy(c->box, S.box, sizeof S.box);
  for (SkinList &L : c->sl) L.valid = false;  // rebuilt from the restored positions
  dev_graph_reset(c);
  return GB_OK;
}

void apply(gb_context *c, const Shape &s) {
  c->tune = s.tune;
  if (c->list_skin != s.skin) {
    c->list_skin = s.skin;
    for (SkinList &L : c->sl) L.valid = false;
  }
  dev_graph_reset(c);
}

// milliseconds per step after three warm-up steps (plain, captured,
// replayed), from the restored state.  region < 0: the mean over `steps` whole
// steps; else the median CUDA-event time of that profiled region (its kernel
// alone; steps run uncaptured with per-region events), which keeps the rare
// pair-list rebuild steps out of the comparison.
int trial(gb_context *c, const Saved &S, const Shape &shape, double dt, double beta, int steps, int region,
          std::vector<cudaEvent_t> &ev, double *ms) {
  int st;
  if ((st = restore(c, S))) return st;
  apply(c, shape);
  for (int i = 0; i < 3; ++i)
    if ((st = dev_step(c, dt, beta))) return st;
  std::vector<double> t;
  if (region < 0) {  // mean over whole steps (rebuilds included)
    TCK(cudaEventRecord(ev[0], c->stream));
    for (int i = 0; i < steps; ++i)
      if ((st = dev_step(c, dt, beta))) return st;
    TCK(cudaEventRecord(ev[1], c->stream));
    TCK(cudaEventSynchronize(ev[1]));
    float x = 0.f;
    TCK(cudaEventElapsedTime(&x, ev[0], ev[1]));
    *ms = (double)x / steps;
    return GB_OK;
  } else {
    TCK(cudaStreamSynchronize(c->stream));
    c->prof = 1;
    c->marks.clear();
    c->ev_next = 0;
    for (int i = 0; i < steps && !st; ++i) st = dev_step(c, dt, beta);
    cudaError_t e = cudaStreamSynchronize(c->stream);
    for (const gb_context::Mark &m : c->marks) {
      float x = 0.f;
      if (m.region == region && cudaEventElapsedTime(&x, m.a, m.b) == cudaSuccess) t.push_back(x);
    }
    c->prof = 0;
    c->marks.clear();
    c->ev_next = 0;
    dev_graph_reset(c);
    if (st) return st;
    TCK(e);
    if (t.empty()) return ctx_set_error(GB_E_ARG, "autotune: the timed region did not run");
  }
  std::sort(t.begin(), t.end());
  const size_t n = t.size();
  *ms = n % 2 ? t[n / 2] : 0.5 * (t[n / 2 - 1] + t[n / 2]);
  return GB_OK;
}

}  // namespace

// the cached shape of c's key, if one was tuned (drop-in contexts take it)
void tune_apply_cached(gb_context *c) {
  if (c->tune.done || g_cache.empty()) return;
  auto it = g_cache.find(key_of(c));
  if (it == g_cache.end()) return;
  apply(c, it->second);
  c->tune.done = 1;
}

extern "C" {

// Chooses the launch shapes of `ctx` for steps of (dt, beta) by timing
// `steps` evolve_pi steps per candidate; the trajectory state is the same
// afterwards.  out6 (optional): lanes per site (Ewald), lanes per oxygen (LJ),
// molecules per MTS block (0: one wave over the SMs), skin fraction, warps per
// k-space force block, sites per lane of the k-space force kernel.
int gbrpmd_ctx_autotune(gb_context *c, double dt, double beta, int steps, double *out6) {
  if (!c) return ctx_set_error(GB_E_ARG, "null context");
  if (steps < 1) return ctx_set_error(GB_E_ARG, "steps must be >= 1");
  const gb_params &P = c->P;
  const bool tunable = !ctx_rigid(c) && !c->nbaro &&
                       (c->rng_mode == GB_RNG_DEVICE || (P.therm != GB_THERM_PRG && P.therm != GB_THERM_PRL));
  auto report = [&]() {
    if (out6) {
      out6[0] = c->tune.ew_np;
      out6[1] = c->tune.lj_np;
      out6[2] = c->tune.mts_mpb;
      out6[3] = c->list_skin;
      out6[4] = c->tune.rf_g;
      out6[5] = c->tune.rf_ns;
    }
    return GB_OK;
  };
  if (!tunable) return report();  // host-side steps or no tunable kernel: defaults
  const Key key = key_of(c);
  auto it = g_cache.find(key);
  if (it != g_cache.end()) {
    apply(c, it->second);
    c->tune.done = 1;
    return report();
  }
  int st;
  TCK(cudaStreamSynchronize(c->stream));
  Saved S;
  if ((st = save(c, S))) return st;
  std::vector<cudaEvent_t> ev(2, nullptr);
  for (cudaEvent_t &e : ev) TCK(cudaEventCreate(&e));
  const bool mixed = P.precision == GB_PREC_MIXED;
  Shape best;
  best.skin = c->list_skin;  // 0 (lists rebuilt at every use) stays 0
  double best_ms = 0.0;
  // each parameter is compared on the time of the kernel it shapes (the
  // region), the list skin on whole steps
  int region = -1, nstep = steps;
  auto baseline = [&](int reg) {
    region = reg;
    nstep = reg < 0 ? 4 * steps : steps;  // rebuilds are rare: whole-step means need longer trials
    if (!st) st = trial(c, S, best, dt, beta, nstep, region, ev, &best_ms);
  };
  auto probe = [&](Shape cand) {
    if (st) return;
    double ms = 0.0;
    st = trial(c, S, cand, dt, beta, nstep, region, ev, &ms);
    // a clear gain only: 2 % on a kernel's own median time, 3 % on whole steps
    if (!st && ms < (region < 0 ? 0.97 : 0.98) * best_ms) {
      best = cand;
      best_ms = ms;
    }
  };
  if (mixed) {
    baseline(PR_EW_REAL);
    for (int np : {8, 32}) {
      Shape cand = best;
      cand.tune.ew_np = np;
      probe(cand);
    }
    baseline(PR_LJ);
    for (int np : {2, 8}) {
      Shape cand = best;
      cand.tune.lj_np = np;
      probe(cand);
    }
    baseline(PR_RECIP_F);
    if (!recip_force_tc_on(c)) {  // the CUDA-core pass's shapes (the tensor-core pass has none to tune)
      for (int g : {8, 16})
        for (int ns : {1, 2}) {
          if (g == best.tune.rf_g && ns == best.tune.rf_ns) continue;
          Shape cand = best;
          cand.tune.rf_g = g;
          cand.tune.rf_ns = ns;
          probe(cand);
        }
      for (int ks : {2, 3, 4, 6}) {
        Shape cand = best;
        cand.tune.rf_ks = ks;
        probe(cand);
      }
    }
  }
  baseline(PR_MTS);
  for (int mpb : {4, 8, 14, 28}) {
    if (mpb >= c->nm) continue;
    Shape cand = best;
    cand.tune.mts_mpb = mpb;
    probe(cand);
  }
  if (best.skin > 0.0) {
    baseline(-1);
    for (double skin : {0.05, 0.15, 0.2}) {
      Shape cand = best;
      cand.skin = skin;
      probe(cand);
    }
  }
  for (cudaEvent_t e : ev) cudaEventDestroy(e);
  int st2 = restore(c, S);
  cudaFree(S.dev);
  if (st) return st;
  if (st2) return st2;
  best.tune.done = 1;
  apply(c, best);
  g_cache[key] = best;
  return report();
}

// forgets the cached shapes (the next autotune of every shape times again)
void gbrpmd_autotune_reset(void) { g_cache.clear(); }

}  // extern "C"
