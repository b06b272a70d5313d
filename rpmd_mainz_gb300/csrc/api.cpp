// api.cpp -- C ABI of the library (include/gbrpmd.h): parameter store,
// device contexts, drop-in entry points and the serial random stream.
#include <cstddef>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <utility>

#include "gb_common.h"
#include "gb_context.h"
#include "gb_rng.h"
#include "gb_kernels.h"

RngState g_rng;  // the process-wide random stream (random.f90's saved state)

namespace {

gb_params g_params;
bool g_init = false;
thread_local std::string g_err = "no error";
std::map<std::pair<int, int>, gb_context *> g_dropin;  // drop-in contexts by (na, nb)

#define CK(x)                                             \
  do {                                                    \
    cudaError_t e_ = (x);                                 \
    if (e_ != cudaSuccess) return ctx_check_cuda(e_, #x); \
  } while (0)

template <typename T>
int dalloc(gb_context *c, T **p, size_t n) {
  CK(cudaMalloc((void **)p, sizeof(T) * (n ? n : 1)));
  c->allocs.push_back((void *)*p);
  c->alloc_bytes += sizeof(T) * (n ? n : 1);
  return GB_OK;
}

// drop-in calls keep one device context per (na, nb)
int dropin_ctx(int na, int nb, gb_context **out) {
  if (!g_init) return ctx_set_error(GB_E_NOINIT, "gbrpmd_init has not been called");
  auto key = std::make_pair(na, nb);
  auto it = g_dropin.find(key);
  if (it != g_dropin.end()) {
    *out = it->second;
    (*out)->P = g_params;
    return GB_OK;
  }
  gb_context *c = new gb_context();
  int st = ctx_alloc(c, na, nb);
  if (st) {
    ctx_free(c);
    delete c;
    return st;
  }
  c->P = g_params;
  g_dropin[key] = c;
  *out = c;
  return GB_OK;
}

int upload(gb_context *c, double *dst, const double *src, size_t n) {
  if (!src) return GB_OK;
  CK(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyHostToDevice, c->stream));
  return GB_OK;
}

int download(gb_context *c, double *dst, const double *src, size_t n) {
  if (!dst) return GB_OK;
  CK(cudaMemcpyAsync(dst, src, sizeof(double) * n, cudaMemcpyDeviceToHost, c->stream));
  return GB_OK;
}

// masses to the device; a change of the O, H, H masses marks the monodromy
// table stale (dev_prepare rebuilds it before the next step, never inside a
// captured one)
int set_masses(gb_context *c, const double *mass) {
  if (!mass) return GB_OK;
  const size_t bytes = sizeof(double) * (size_t)c->na;
  if (c->h_mass_all.size() == (size_t)c->na && std::memcmp(c->h_mass_all.data(), mass, bytes) == 0) return GB_OK;
  c->h_mass_all.assign(mass, mass + c->na);
  const int n = std::min(3, c->na);
  bool same = true;
  for (int i = 0; i < n; ++i) same = same && c->h_mass3[i] == mass[i];
  if (!same) {
    for (int i = 0; i < n; ++i) c->h_mass3[i] = mass[i];
    c->mass_version += 1;
  }
  return upload(c, c->mass, mass, (size_t)c->na);
}

int set_charges(gb_context *c, const double *z) {
  if (!z) return GB_OK;
  const size_t bytes = sizeof(double) * (size_t)c->na;
  if (c->h_z_all.size() == (size_t)c->na && std::memcmp(c->h_z_all.data(), z, bytes) == 0) return GB_OK;
  c->h_z_all.assign(z, z + c->na);
  double qq = 0.0;
  for (int i = 0; i < c->na; ++i) qq = qq + z[i] * z[i];
  c->qq = qq;
  return upload(c, c->z, z, (size_t)c->na);
}

int check_sizes(int na, int nb) {
  if (na <= 0 || na % 3 != 0) return ctx_set_error(GB_E_ARG, "potenl 1: na is not 3*nm");
  if (nb <= 0 || nb > 256) return ctx_set_error(GB_E_ARG, "nb must be 1..256 (fourier.f90 nmax)");
  return GB_OK;
}

}  // namespace

const gb_params &current_params() { return g_params; }

int ctx_set_error(int code, const std::string &msg) {
  g_err = msg;
  return code;
}

int ctx_check_cuda(cudaError_t e, const char *what) {
  g_err = std::string("CUDA error ") + cudaGetErrorString(e) + " at " + what;
  return e == cudaErrorMemoryAllocation ? GB_E_NOMEM : GB_E_CUDA;
}

void prof_begin(gb_context *c, int region) {
  if (!c->prof) return;
  (void)region;
  if (c->ev_next + 2 > c->ev_pool.size()) {
    for (int i = 0; i < 64; ++i) {
      cudaEvent_t e;
      cudaEventCreate(&e);
      c->ev_pool.push_back(e);
    }
  }
  cudaEventRecord(c->ev_pool[c->ev_next], c->stream);
}

void prof_end(gb_context *c, int region, double units) {
  if (!c->prof) return;
  cudaEvent_t a = c->ev_pool[c->ev_next], b = c->ev_pool[c->ev_next + 1];
  cudaEventRecord(b, c->stream);
  c->marks.push_back({region, a, b, units});
  c->ev_next += 2;
}

int watch_mark(gb_context *c, int region, cudaStream_t s, int which) {
  if (c->watch != region || !c->watch_ev[which]) return GB_OK;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(s, &cap));
  if (cap == cudaStreamCaptureStatusActive) CK(cudaEventRecordWithFlags(c->watch_ev[which], s, cudaEventRecordExternal));
  else CK(cudaEventRecord(c->watch_ev[which], s));
  if (which == 1) c->watch_seen = true;
  return GB_OK;
}

int ctx_alloc(gb_context *c, int na, int nb) {
  int st = check_sizes(na, nb);
  if (st) return st;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
    return ctx_set_error(GB_E_CUDA, "no CUDA device");
  CK(cudaGetDevice(&c->device));
  c->na = na;
  c->nb = nb;
  c->nm = na / 3;
  const char *gen = std::getenv("GBRPMD_GENERIC_MTS");
  c->generic_mts = gen && gen[0] == '1';
  if (const char *sk = std::getenv("GBRPMD_LIST_SKIN")) c->list_skin = std::max(0.0, std::atof(sk));
  if (const char *gr = std::getenv("GBRPMD_GRAPHS")) c->use_graphs = gr[0] != '0';
  if (const char *ce = std::getenv("GBRPMD_LIST_CELLS")) c->list_cells = ce[0] != '0';
  if (const char *br = std::getenv("GBRPMD_BRANCHES")) c->use_branches = br[0] != '0';
  if (const char *es = std::getenv("GBRPMD_EW_SHARED")) c->ew_share = es[0] != '0';
  CK(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&c->aux_stream, cudaStreamNonBlocking));
  CK(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming));
  {  // the k-space chain (three dependent launches with few blocks each) goes
     // first when SMs free up; the real-space and LJ kernels fill the rest
    int least = 0, greatest = 0;
    CK(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CK(cudaStreamCreateWithPriority(&c->aux2_stream, cudaStreamNonBlocking, greatest));
  }
  CK(cudaEventCreateWithFlags(&c->fork2_ev, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&c->join2_ev, cudaEventDisableTiming));
  const size_t N = 3 * (size_t)na * nb, S = 3 * (size_t)na;
  if ((st = dalloc(c, &c->p, N)) || (st = dalloc(c, &c->r, N)) || (st = dalloc(c, &c->dvdr, N)) ||
      (st = dalloc(c, &c->dvdr2, N)) || (st = dalloc(c, &c->rst, N)) || (st = dalloc(c, &c->rnm, N)) ||
      (st = dalloc(c, &c->mass, (size_t)na)) || (st = dalloc(c, &c->z, (size_t)na)) ||
      (st = dalloc(c, &c->f_a, N)) || (st = dalloc(c, &c->f_b, N)) || (st = dalloc(c, &c->f_c, N)) ||
      (st = dalloc(c, &c->rb1, N)) || (st = dalloc(c, &c->fb1, N)) || (st = dalloc(c, &c->rb2, N)) ||
      (st = dalloc(c, &c->fb2, N)) || (st = dalloc(c, &c->g, N)) || (st = dalloc(c, &c->rs, N)) ||
      (st = dalloc(c, &c->rs32, (size_t)na * nb)) || (st = dalloc(c, &c->lo32, (size_t)na * nb)) ||
      (st = dalloc(c, &c->fx32, (size_t)na * nb)) || (st = dalloc(c, &c->fxs_b, (size_t)na * nb)) ||
      (st = dalloc(c, &c->rcen, S)) || (st = dalloc(c, &c->spread, 4)) ||
      (st = dalloc(c, &c->hi32, (size_t)na * nb / 3)) || (st = dalloc(c, &c->olo32, (size_t)na * nb / 3)) ||
      (st = dalloc(c, &c->rs32_lj, (size_t)na * nb / 3)) || (st = dalloc(c, &c->g2, N)) ||
      (st = dalloc(c, &c->rc, S)) ||
      (st = dalloc(c, &c->monod, 12 * (size_t)nb)) ||
      (st = dalloc(c, &c->acc, (size_t)ACC_NSLOT * ACC_STRIDE)) || (st = dalloc(c, &c->status, 1)))
    return st;
  CK(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
  CK(cudaMemsetAsync(c->spread, 0, 4 * sizeof(float), c->stream));
  CK(cudaMemsetAsync(c->dvdr, 0, sizeof(double) * N, c->stream));
  CK(cudaMemsetAsync(c->dvdr2, 0, sizeof(double) * N, c->stream));
  CK(cudaMemsetAsync(c->p, 0, sizeof(double) * N, c->stream));
  CK(cudaMallocHost(&c->h_acc, sizeof(double) * ACC_NSLOT * ACC_STRIDE));
  CK(cudaMallocHost(&c->h_status, sizeof(unsigned)));
  CK(cudaStreamSynchronize(c->stream));
  return GB_OK;
}

void ctx_free(gb_context *c) {
  if (c->stream) cudaStreamSynchronize(c->stream);
  dev_graph_reset(c);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  c->ev_pool.clear();
  if (c->d_count) cudaFree(c->d_count);
  if (c->d_npair) cudaFree(c->d_npair);
  for (void *p : c->allocs) cudaFree(p);
  c->allocs.clear();
  for (void *p : {(void *)c->pl.idx, (void *)c->pl.count, (void *)c->pl_lj.idx, (void *)c->pl_lj.count, (void *)c->kcol,
                  (void *)c->kgrp,
                  (void *)c->kpair, (void *)c->kw, (void *)c->kvir, (void *)c->ktab, (void *)c->sk_part, (void *)c->sk,
                  (void *)c->tw_nb, (void *)c->tw_c1, (void *)c->tw_c2})
    if (p) cudaFree(p);
  for (SkinList &L : c->sl)  // the cell offsets and per-point cell arrays live in ccount and spos
    for (void *p : {(void *)L.pl.idx, (void *)L.pl.count, (void *)L.ref, (void *)L.flag, (void *)L.rebuilds,
                    (void *)L.cells.ccount, (void *)L.cells.spos, (void *)L.cells.ticket})
      if (p) cudaFree(p);
  if (c->h_acc) cudaFreeHost(c->h_acc);
  if (c->h_status) cudaFreeHost(c->h_status);
  if (c->h_gauss) cudaFreeHost(c->h_gauss);
  if (c->d_gauss) cudaFree(c->d_gauss);
  if (c->d_therm) cudaFree(c->d_therm);
  if (c->d_rngctr) cudaFree(c->d_rngctr);
  if (c->gauss_ev) cudaEventDestroy(c->gauss_ev);
  if (c->mid_ev) cudaEventDestroy(c->mid_ev);
  for (cudaEvent_t e : c->watch_ev)
    if (e) cudaEventDestroy(e);
  if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
  if (c->fork_ev) cudaEventDestroy(c->fork_ev);
  if (c->join_ev) cudaEventDestroy(c->join_ev);
  if (c->aux_stream) cudaStreamDestroy(c->aux_stream);
  if (c->fork2_ev) cudaEventDestroy(c->fork2_ev);
  if (c->join2_ev) cudaEventDestroy(c->join2_ev);
  if (c->aux2_stream) cudaStreamDestroy(c->aux2_stream);
  if (c->stream) cudaStreamDestroy(c->stream);
  c->stream = nullptr;
}

extern "C" {

int gbrpmd_init(const gb_params *params) {
  if (!params) return ctx_set_error(GB_E_ARG, "null params");
  if (params->mts < 1) return ctx_set_error(GB_E_ARG, "mts must be >= 1");
  if (params->precision != GB_PREC_FP64 && params->precision != GB_PREC_MIXED)
    return ctx_set_error(GB_E_ARG, "precision must be GB_PREC_FP64 or GB_PREC_MIXED");
  g_params = *params;
  g_init = true;
  return GB_OK;
}

int gbrpmd_get_params(gb_params *params) {
  if (!g_init) return ctx_set_error(GB_E_NOINIT, "gbrpmd_init has not been called");
  *params = g_params;
  return GB_OK;
}

int gbrpmd_params_layout(int64_t *offsets, int nfield) {
  static const int64_t off[] = {
      offsetof(gb_params, oo_eps), offsetof(gb_params, oo_sig), offsetof(gb_params, oo_gam),
      offsetof(gb_params, rcut), offsetof(gb_params, alpha), offsetof(gb_params, ecut), offsetof(gb_params, wm),
      offsetof(gb_params, wh), offsetof(gb_params, wrcut), offsetof(gb_params, walpha), offsetof(gb_params, rkmax),
      offsetof(gb_params, kmax), offsetof(gb_params, nbdf1), offsetof(gb_params, nbdf2), offsetof(gb_params, apot),
      offsetof(gb_params, bpot), offsetof(gb_params, alp), offsetof(gb_params, alpb), offsetof(gb_params, theta),
      offsetof(gb_params, reoh), offsetof(gb_params, sig), offsetof(gb_params, mts), offsetof(gb_params, iamcub),
      offsetof(gb_params, nctot), offsetof(gb_params, nbond), offsetof(gb_params, therm), offsetof(gb_params, ttau),
      offsetof(gb_params, taub), offsetof(gb_params, patm), offsetof(gb_params, intra_model),
      offsetof(gb_params, precision), offsetof(gb_params, baro)};
  constexpr int n = (int)(sizeof(off) / sizeof(off[0]));
  static_assert(n == 32, "gb_params has 32 fields");
  for (int i = 0; offsets && i < nfield && i < n; ++i) offsets[i] = off[i];
  return (int)sizeof(gb_params);
}

const char *gbrpmd_last_error(void) { return g_err.c_str(); }

int gbrpmd_finalize(void) {
  for (auto &kv : g_dropin) {
    ctx_free(kv.second);
    delete kv.second;
  }
  g_dropin.clear();
  return GB_OK;
}

// ---- drop-in entry points ----

int gbrpmd_forces(double *r, double *v, double *dvdr, const int *nb, const int *na,
                  const double *boxlxyz, const double *z, double *virial, const int *iopt) {
  gb_context *c;
  int st = dropin_ctx(*na, *nb, &c);
  if (st) return st;
  const size_t N = 3 * (size_t)(*na) * (*nb);
  std::memcpy(c->box, boxlxyz, sizeof(double) * 3);
  if ((st = upload(c, c->r, r, N)) || (st = set_charges(c, z))) return st;
  if ((st = dev_forces(c, c->r, *nb, c->dvdr, *iopt))) return st;
  if ((st = download(c, dvdr, c->dvdr, N))) return st;
  if ((st = dev_collect(c, 0, 0.0, 1.0))) return st;
  *v = c->e_v;
  for (int i = 0; i < 9; ++i) virial[i] = c->e_vir[i];
  return GB_OK;
}

int gbrpmd_full_forces(double *r, const int *na, const int *nb, double *v, double *vew,
                       double *voo, double *vint, double *vir, const double *z,
                       const double *boxlxyz, double *dvdr, double *dvdr2) {
  gb_context *c;
  int st = dropin_ctx(*na, *nb, &c);
  if (st) return st;
  const size_t N = 3 * (size_t)(*na) * (*nb);
  std::memcpy(c->box, boxlxyz, sizeof(double) * 3);
  if ((st = upload(c, c->r, r, N)) || (st = set_charges(c, z))) return st;
  if ((st = dev_full_forces(c))) return st;
  if ((st = download(c, dvdr, c->dvdr, N)) || (st = download(c, dvdr2, c->dvdr2, N))) return st;
  if ((st = dev_collect(c, 0, 0.0, 1.0))) return st;
  *v = c->e_v;
  *vew = c->e_vew;
  *voo = c->e_vlj;
  *vint = c->e_vint;
  for (int i = 0; i < 9; ++i) vir[i] = c->e_vir[i];
  return GB_OK;
}

int gbrpmd_evolve_pi(double *p, double *r, double *v, double *vew, double *vlj, double *vint,
                     double *dvdr, double *dvdr2, const double *dt, const double *mass,
                     const int *na, const int *nb, double *boxlxyz, const double *z,
                     const double *beta, double *vir, double *vir_lf, int *irun,
                     const int *nbaro) {
  gb_context *c;
  int st = dropin_ctx(*na, *nb, &c);
  if (st) return st;
  const size_t N = 3 * (size_t)(*na) * (*nb);
  std::memcpy(c->box, boxlxyz, sizeof(double) * 3);
  std::memcpy(c->vir_lf_in, vir_lf, sizeof(double) * 9);  // the barostat reads the previous call's vir_lf
  c->nbaro = *nbaro;
  tune_apply_cached(c);  // launch shapes of an autotuned context of the same shape
  if (!c->mid_ev) {
    CK(cudaEventCreateWithFlags(&c->mid_ev, cudaEventDisableTiming));
    CK(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
  }
  c->want_mid = 1;
  c->th_rng = &g_rng;  // thermostat kicks draw the process-wide stream with the caller's irun
  c->th_idum = irun;
  if ((st = upload(c, c->p, p, N)) || (st = upload(c, c->r, r, N)) || (st = upload(c, c->dvdr, dvdr, N)) ||
      (st = upload(c, c->dvdr2, dvdr2, N)) || (st = set_masses(c, mass)) || (st = set_charges(c, z)))
    return st;
  c->mid_recorded = false;
  st = dev_step(c, *dt, *beta);
  c->th_rng = nullptr;
  c->th_idum = nullptr;
  if (st) return st;
  std::memcpy(boxlxyz, c->box, sizeof(double) * 3);  // scaled by the barostat
  if (c->mid_recorded) {  // r and dvdr2 leave while the low-frequency forces compute
    CK(cudaStreamWaitEvent(c->copy_stream, c->mid_ev, 0));
    CK(cudaMemcpyAsync(r, c->r, sizeof(double) * N, cudaMemcpyDeviceToHost, c->copy_stream));
    CK(cudaMemcpyAsync(dvdr2, c->dvdr2, sizeof(double) * N, cudaMemcpyDeviceToHost, c->copy_stream));
    if ((st = download(c, p, c->p, N)) || (st = download(c, dvdr, c->dvdr, N))) return st;
  } else if ((st = download(c, p, c->p, N)) || (st = download(c, r, c->r, N)) ||
             (st = download(c, dvdr, c->dvdr, N)) || (st = download(c, dvdr2, c->dvdr2, N))) {
    return st;
  }
  st = dev_collect(c, 1, *dt, *beta);
  if (c->mid_recorded) CK(cudaStreamSynchronize(c->copy_stream));
  if (st) return st;
  *v = c->e_v;
  *vew = c->e_vew;
  *vlj = c->e_vlj;
  *vint = c->e_vint;
  for (int i = 0; i < 9; ++i) {
    vir[i] = c->e_vir[i];
    vir_lf[i] = c->e_vir_lf[i];
  }
  return GB_OK;
}

// ---- resident interface ----

int gbrpmd_ctx_create(gb_context **ctx, int na, int nb, const double *mass, const double *z) {
  if (!g_init) return ctx_set_error(GB_E_NOINIT, "gbrpmd_init has not been called");
  gb_context *c = new gb_context();
  int st = ctx_alloc(c, na, nb);
  if (st) {
    ctx_free(c);
    delete c;
    return st;
  }
  c->P = g_params;
  if ((st = set_masses(c, mass)) || (st = set_charges(c, z))) {
    ctx_free(c);
    delete c;
    return st;
  }
  cudaStreamSynchronize(c->stream);
  *ctx = c;
  return GB_OK;
}

int gbrpmd_ctx_destroy(gb_context *ctx) {
  if (!ctx) return GB_OK;
  ctx_free(ctx);
  delete ctx;
  return GB_OK;
}

int gbrpmd_ctx_upload(gb_context *c, const double *r, const double *p, const double *dvdr,
                      const double *dvdr2, const double *boxlxyz) {
  const size_t N = 3 * (size_t)c->na * c->nb;
  int st;
  if (boxlxyz) std::memcpy(c->box, boxlxyz, sizeof(double) * 3);
  if ((st = upload(c, c->r, r, N)) || (st = upload(c, c->p, p, N)) || (st = upload(c, c->dvdr, dvdr, N)) ||
      (st = upload(c, c->dvdr2, dvdr2, N)))
    return st;
  return GB_OK;
}

int gbrpmd_ctx_download(gb_context *c, double *r, double *p, double *dvdr, double *dvdr2) {
  const size_t N = 3 * (size_t)c->na * c->nb;
  int st;
  if ((st = download(c, r, c->r, N)) || (st = download(c, p, c->p, N)) || (st = download(c, dvdr, c->dvdr, N)) ||
      (st = download(c, dvdr2, c->dvdr2, N)))
    return st;
  CK(cudaStreamSynchronize(c->stream));
  return GB_OK;
}

int gbrpmd_ctx_full_forces(gb_context *c, double *v, double *vew, double *voo, double *vint,
                           double *vir) {
  if (!c->own_params) c->P = g_params;
  int st = dev_full_forces(c);
  if (st) return st;
  if ((st = dev_collect(c, 0, 0.0, 1.0))) return st;
  if (v) *v = c->e_v;
  if (vew) *vew = c->e_vew;
  if (voo) *voo = c->e_vlj;
  if (vint) *vint = c->e_vint;
  if (vir)
    for (int i = 0; i < 9; ++i) vir[i] = c->e_vir[i];
  return GB_OK;
}

int gbrpmd_ctx_evolve(gb_context *c, int nsteps, double dt, double beta) {
  if (!c->own_params) c->P = g_params;
  if (c->has_own_rng) {
    c->th_rng = &c->own_rng;
    c->th_idum = &c->own_idum;
  }
  int st = GB_OK;
  for (int s = 0; s < nsteps && !st; ++s) {
    st = dev_step(c, dt, beta);
    // with a barostat each step needs the last one's vir_lf on the host
    if (!st && c->nbaro) st = dev_collect(c, 1, dt, beta);
  }
  c->th_rng = nullptr;
  c->th_idum = nullptr;
  return st;
}

int gbrpmd_ctx_set_rng(gb_context *c, int idum) {
  if (!c) return ctx_set_error(GB_E_ARG, "null context");
  c->own_rng = RngState();
  c->own_idum = idum;
  c->has_own_rng = true;
  return GB_OK;
}

int gbrpmd_ctx_set_rng_mode(gb_context *c, int mode, uint64_t seed) {
  if (!c) return ctx_set_error(GB_E_ARG, "null context");
  if (mode != GB_RNG_REFERENCE && mode != GB_RNG_DEVICE) return ctx_set_error(GB_E_ARG, "unknown random-stream mode");
  CK(cudaStreamSynchronize(c->stream));
  if (mode == GB_RNG_DEVICE) {
    if (!c->d_rngctr) CK(cudaMalloc(&c->d_rngctr, sizeof(unsigned long long)));
    if (!c->d_therm) CK(cudaMalloc(&c->d_therm, sizeof(double) * 4));
    CK(cudaMemsetAsync(c->d_rngctr, 0, sizeof(unsigned long long), c->stream));
    CK(cudaStreamSynchronize(c->stream));
  }
  c->rng_mode = mode;
  c->rng_seed = seed;
  dev_graph_reset(c);
  return GB_OK;
}

int gbrpmd_ctx_set_nbaro(gb_context *c, int nbaro) {
  if (!c) return ctx_set_error(GB_E_ARG, "null context");
  if (nbaro != 0 && nbaro != 1) return ctx_set_error(GB_E_ARG, "nbaro must be 0 or 1");
  c->nbaro = nbaro;
  dev_graph_reset(c);
  return GB_OK;
}

int gbrpmd_ctx_box(gb_context *c, double *box3) {
  if (!c || !box3) return ctx_set_error(GB_E_ARG, "null argument");
  for (int d = 0; d < 3; ++d) box3[d] = c->box[d];
  return GB_OK;
}

void gbrpmd_rng_reset(void) { g_rng = RngState(); }

int gbrpmd_ctx_sync(gb_context *c) { return dev_collect(c, 1, 0.0, c->last_beta); }

int gbrpmd_ctx_energies(gb_context *c, double *out5, double *vir, double *vir_lf) {
  if (out5) {
    out5[0] = c->e_v;
    out5[1] = c->e_vew;
    out5[2] = c->e_vlj;
    out5[3] = c->e_vint;
    out5[4] = c->e_tv;
  }
  if (vir)
    for (int i = 0; i < 9; ++i) vir[i] = c->e_vir[i];
  if (vir_lf)
    for (int i = 0; i < 9; ++i) vir_lf[i] = c->e_vir_lf[i];
  return GB_OK;
}

void *gbrpmd_ctx_stream(gb_context *c) { return (void *)c->stream; }

// md_eq's output block (md_eq.f90:190-299) on the resident state; see gbrpmd.h
int gbrpmd_ctx_estimators(gb_context *c, double beta, double *out, double *rcm, double *mdip) {
  if (!c || !out) return ctx_set_error(GB_E_ARG, "null argument");
  if (!(beta > 0.0)) return ctx_set_error(GB_E_ARG, "beta must be positive");
  if (!c->own_params) c->P = g_params;
  const int na = c->na, nb = c->nb, nm = na / 3;
  int st;
  if (!c->est && (st = dalloc(c, &c->est, 16 + 6 * (size_t)nm))) return st;
  double *d_rcm = rcm ? c->est + 16 : nullptr, *d_mdip = mdip ? c->est + 16 + 3 * (size_t)nm : nullptr;
  CK(cudaMemsetAsync(c->est, 0, sizeof(double) * 16, c->stream));
  launch_estimators(c->stream, c->r, c->p, c->dvdr, c->dvdr2, c->mass, c->z, na, nb, c->P.alpha, c->est, d_rcm,
                    d_mdip);
  ++c->launches;
  CK(cudaGetLastError());
  double a[16];
  CK(cudaMemcpyAsync(a, c->est, sizeof(double) * 16, cudaMemcpyDeviceToHost, c->stream));
  if (rcm) CK(cudaMemcpyAsync(rcm, d_rcm, sizeof(double) * 3 * nm, cudaMemcpyDeviceToHost, c->stream));
  if (mdip) CK(cudaMemcpyAsync(mdip, d_mdip, sizeof(double) * 3 * nm, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const gb_params &P = c->P;
  const double tk = a[0];                                      // kinetic_rpmd
  const double omegan = (double)nb / (beta * GB_HBAR);         // md_eq.f90:254
  const double vrp = 0.5 * omegan * omegan * a[1];
  const double temp = GB_TO_K * (2.0 * tk / ((double)(3 * na - P.nctot - 3) * (double)nb)) / (double)nb;
  const double tc = 0.5 * (double)(3 * na - 3 - P.nctot) / beta;  // virial_ke: nc = 3 (kinetic.f90:42-47)
  const double tv = tc + 0.5 * a[2] / nb + 0.5 * a[3] / nb;
  const double vol = c->box[0] * c->box[1] * c->box[2];
  // pressure (md_pressure.f90:1-30) from the virial of the last evaluation and pres_lj_tail (32-56)
  const double w = -(c->e_vir[0] + c->e_vir[4] + c->e_vir[8]) / 3.0;
  double pres = (2.0 * tv / 3.0 + w) / vol;
  if (P.oo_gam == 0.0) {
    const double rho = (double)nm / vol, sr = P.oo_sig / P.rcut;
    const double pi = std::acos(-1.0);
    const double prefac = (16.0 * pi * (rho * rho) * P.oo_eps * (P.oo_sig * P.oo_sig * P.oo_sig)) / 3.0;
    pres += prefac * ((2.0 / 3.0) * std::pow(sr, 9) - std::pow(sr, 3));
  }
  const double dip[3] = {a[10] / nb, a[11] / nb, a[12] / nb};
  out[0] = tk;
  out[1] = vrp;
  out[2] = nb * c->e_v + tk + vrp;  // md_eq.f90:274 (times na)
  out[3] = temp;
  out[4] = tv;
  for (int x = 0; x < 3; ++x) out[5 + x] = tc / 3.0 + 0.5 * a[4 + x] / nb + 0.5 * a[7 + x] / nb;
  out[8] = pres;
  for (int x = 0; x < 3; ++x) out[9 + x] = dip[x];
  out[12] = dip[0] * dip[0] + dip[1] * dip[1] + dip[2] * dip[2];
  out[13] = a[13] / ((double)nb * nm);
  out[14] = GB_TO_KGCM3 * ((c->h_mass3[0] + c->h_mass3[1] + c->h_mass3[2]) * (double)nm / vol);  // md_eq.f90:196-198
  out[15] = c->e_v;
  return GB_OK;
}

int gbrpmd_ctx_set_profiling(gb_context *c, int on) {
  CK(cudaStreamSynchronize(c->stream));
  dev_graph_reset(c);
  c->prof = on;
  c->marks.clear();
  c->ev_next = 0;
  return GB_OK;
}

int gbrpmd_ctx_watch_region(gb_context *c, int region) {
  if (!c) return ctx_set_error(GB_E_ARG, "null context");
  if (region != -1 && region != PR_MTS && region != PR_EW_REAL && region != PR_RECIP_F && region != PR_LJ)
    return ctx_set_error(GB_E_ARG, "watched region must be -1, 0, 2, 5 or 6");
  CK(cudaStreamSynchronize(c->stream));
  for (cudaEvent_t &e : c->watch_ev)
    if (!e) CK(cudaEventCreate(&e));
  dev_graph_reset(c);
  c->watch = region;
  c->watch_seen = false;
  return GB_OK;
}

int gbrpmd_ctx_watch_ms(gb_context *c, float *ms) {
  if (!c || !ms) return ctx_set_error(GB_E_ARG, "null argument");
  if (c->watch < 0 || !c->watch_seen) return ctx_set_error(GB_E_ARG, "no watched launch recorded");
  CK(cudaEventSynchronize(c->watch_ev[1]));
  CK(cudaEventElapsedTime(ms, c->watch_ev[0], c->watch_ev[1]));
  return GB_OK;
}

int gbrpmd_ctx_set_list_skin(gb_context *c, double fraction) {
  if (!c) return ctx_set_error(GB_E_ARG, "null context");
  if (!(fraction >= 0.0) || fraction > 1.0) return ctx_set_error(GB_E_ARG, "list skin fraction must be in [0, 1]");
  c->list_skin = fraction;
  for (SkinList &L : c->sl) L.valid = false;
  dev_graph_reset(c);
  return GB_OK;
}

int gbrpmd_ctx_set_params(gb_context *c, const gb_params *params) {
  if (!c || !params) return ctx_set_error(GB_E_ARG, "null argument");
  if (params->mts < 1) return ctx_set_error(GB_E_ARG, "mts must be >= 1");
  if (params->precision != GB_PREC_FP64 && params->precision != GB_PREC_MIXED)
    return ctx_set_error(GB_E_ARG, "precision must be GB_PREC_FP64 or GB_PREC_MIXED");
  CK(cudaStreamSynchronize(c->stream));
  c->P = *params;
  c->own_params = 1;
  return GB_OK;
}

size_t gbrpmd_ctx_device_bytes(gb_context *c) { return c ? ctx_device_bytes(c) : 0; }

size_t gbrpmd_estimate_device_bytes(int na, int nb, const gb_params *params) {
  return params ? dev_estimate_bytes(na, nb, *params) : 0;
}

int gbrpmd_ctx_list_occupancy(gb_context *c, int *out8) {
  if (!c || !out8) return ctx_set_error(GB_E_ARG, "null argument");
  CK(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < LIST_N; ++i) {
    out8[2 * i] = list_max(c->stream, c->sl[i].pl);
    out8[2 * i + 1] = c->sl[i].pl.cap;
  }
  out8[6] = list_max(c->stream, c->pl);
  out8[7] = c->pl.cap;
  return GB_OK;
}

int gbrpmd_ctx_set_graphs(gb_context *c, int on) {
  if (!c) return ctx_set_error(GB_E_ARG, "null context");
  CK(cudaStreamSynchronize(c->stream));
  dev_graph_reset(c);
  c->use_graphs = on ? 1 : 0;
  return GB_OK;
}

int gbrpmd_ctx_list_rebuilds(gb_context *c, unsigned *counts3) {
  if (!c || !counts3) return ctx_set_error(GB_E_ARG, "null argument");
  CK(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < LIST_N; ++i) {
    counts3[i] = 0;
    if (c->sl[i].rebuilds) {
      CK(cudaMemcpyAsync(&counts3[i], c->sl[i].rebuilds, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
    }
  }
  return GB_OK;
}

int gbrpmd_ctx_region_times(gb_context *c, double *ms, double *units, int *counts, int nregion) {
  CK(cudaStreamSynchronize(c->stream));
  for (int i = 0; i < nregion; ++i) {
    ms[i] = 0.0;
    units[i] = 0.0;
    counts[i] = 0;
  }
  for (const auto &m : c->marks) {
    if (m.region < 0 || m.region >= nregion) continue;
    float t = 0.f;
    CK(cudaEventElapsedTime(&t, m.a, m.b));
    ms[m.region] += t;
    units[m.region] += m.units;
    counts[m.region] += 1;
  }
  c->marks.clear();
  c->ev_next = 0;
  return GB_OK;
}

int64_t gbrpmd_ctx_launch_count(gb_context *c) { return c->launches; }

// ---- serial random stream (random.f90:1-72), one process-wide state ----

double gbrpmd_ran2(int *idum, const double *rmin, const double *rmax) { return rng_ran2(g_rng, idum, *rmin, *rmax); }

double gbrpmd_gaussian(int *idum, const double *sigma) { return rng_gaussian(g_rng, idum, *sigma); }

}  // extern "C"

// ---- rigid path entry points (device implementation in rattle.cpp) ----
int dev_rattle_setup(int nm, const gb_params &P);
int dev_rattle_set_itmax(int itmax);
int dev_rattle_s1(double *r, const double *rold, double *p, int nm, const double *mass, double dt,
                  double *dvdr, double *vir, int na);
int dev_rattle_s2(double *r, double *p, int nm, const double *mass, double dt, double *dvdr,
                  double *vir, int na);

extern "C" {

int gbrpmd_rattle_setup(const int *nm) {
  if (!g_init) return ctx_set_error(GB_E_NOINIT, "gbrpmd_init has not been called");
  if (*nm <= 0) return ctx_set_error(GB_E_ARG, "nm must be positive");
  g_params.nctot = 3 * (*nm);
  g_params.nbond = 3;
  return dev_rattle_setup(*nm, g_params);
}

int gbrpmd_rattle_set_itmax(const int *itmax) {
  if (!itmax) return ctx_set_error(GB_E_ARG, "null argument");
  return dev_rattle_set_itmax(*itmax);
}

int gbrpmd_rattle_s1(double *r, const double *rold, double *p, const int *nm, const double *mass,
                     const double *dt, double *dvdr, double *vir, const int *na) {
  if (!g_init) return ctx_set_error(GB_E_NOINIT, "gbrpmd_init has not been called");
  return dev_rattle_s1(r, rold, p, *nm, mass, *dt, dvdr, vir, *na);
}

int gbrpmd_rattle_s2(double *r, double *p, const int *nm, const double *mass, const double *dt,
                     double *dvdr, double *vir, const int *na) {
  if (!g_init) return ctx_set_error(GB_E_NOINIT, "gbrpmd_init has not been called");
  return dev_rattle_s2(r, p, *nm, mass, *dt, dvdr, vir, *na);
}

int gbrpmd_evolve_rig_pi(double *p, double *r, double *v, double *v_lf, double *v_hf, double *dvdr,
                         double *dvdr2, const double *dt, const double *mass, const int *na,
                         const int *nb, double *boxlxyz, const double *z, const double *beta,
                         double *vir, double *vir_lf, int *irun, const int *nbaro) {
  gb_context *c;
  int st = dropin_ctx(*na, *nb, &c);
  if (st) return st;
  const size_t N = 3 * (size_t)(*na) * (*nb);
  std::memcpy(c->box, boxlxyz, sizeof(double) * 3);
  c->nbaro = *nbaro;
  if ((st = upload(c, c->p, p, N)) || (st = upload(c, c->r, r, N)) || (st = upload(c, c->dvdr, dvdr, N)) ||
      (st = upload(c, c->dvdr2, dvdr2, N)) || (st = set_masses(c, mass)) ||
      (st = set_charges(c, z)))
    return st;
  c->th_rng = &g_rng;
  c->th_idum = irun;
  st = dev_evolve_rig_pi(c, *dt, *beta, vir);
  c->th_rng = nullptr;
  c->th_idum = nullptr;
  if (st) return st;
  std::memcpy(boxlxyz, c->box, sizeof(double) * 3);  // scaled by the barostat
  if ((st = download(c, p, c->p, N)) || (st = download(c, r, c->r, N)) ||
      (st = download(c, dvdr, c->dvdr, N)) || (st = download(c, dvdr2, c->dvdr2, N)))
    return st;
  if ((st = dev_collect(c, 2, *dt, *beta))) return st;
  *v = c->e_v;
  *v_lf = c->e_v;
  *v_hf = 0.0;
  for (int i = 0; i < 9; ++i) {
    vir_lf[i] = c->e_vir_lf[i];
    vir[i] = c->e_vir_lf[i] + c->e_vir_hf[i] + vir[i];
  }
  return GB_OK;
}

}  // extern "C"
