// noalloc.cu -- the Ewald force entry point that allocates no device memory.
//
// gbrpmd_forces_ewald_static computes what gbrpmd_forces computes for
// iopt = 2 in FP64 (M-site substitution, real-space and reciprocal Ewald sums,
// chain rule; bead-averaged energy and virial), whatever gb_params.precision
// says, but every device buffer it needs -- positions, pair lists, structure
// factors, accumulators -- lives in one file-scope __device__ array of
// STATIC_SCRATCH_BYTES (16 MiB).  It is meant for callers that may not call
// cudaMalloc themselves or through us: hosts that run under a fixed
// device-memory budget handed out by another framework's pool, or codes that
// must not trigger allocation (and the implicit synchronisation a cudaFree
// brings) in the middle of their own stream work.
//
// The array is part of the module image: every GPU that loads the library
// reserves the 16 MiB until the process exits.  Host code only knows a
// host-side stand-in for the array's name, so the device address is fetched
// once per device with cudaGetSymbolAddress, with that device current, on the
// first call made on that device; make that first call before any stream
// capture.  The work runs on the calling thread's per-thread default stream
// (cudaStreamPerThread), which creates nothing and does not synchronise with
// the caller's other streams.  The array keeps the last call's contents and is
// shared by all calls, as are the host-side k tables below: each call clears
// what must start at zero, and since two calls in flight at once would race on
// both, a process-wide lock serialises the calls from the start of a call until
// its device work has finished.
//
// Limits (rejected with GB_E_NOMEM and a message): na * nb <= 8192 sites,
// nb <= 64, at most 2048 k vectors in 512 (kx, ky) columns, and every buffer
// together within 16 MiB -- mostly the pair list, 4 bytes per site and partner
// slot, with slots for 1.1 times the partners a uniform liquid has within the
// real-space cut-off, plus 48.  A configuration denser than that somewhere
// returns GB_E_LIST.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>

#include "gb_common.cuh"
#include "gb_context.h"
#include "gb_kernels.h"

const gb_params &current_params();
int ctx_set_error(int code, const std::string &msg);

namespace {

constexpr size_t STATIC_SCRATCH_BYTES = 16u << 20;
constexpr int MAX_SITES = 8192;
constexpr int MAX_NB = 64;
constexpr int MAX_NK = 2048;
constexpr int MAX_NKXY = 512;
constexpr int MAX_DEVICES = 64;

__device__ __align__(256) unsigned char g_static_scratch[STATIC_SCRATCH_BYTES];

unsigned char *g_scratch_ptr[MAX_DEVICES] = {nullptr};

// serialises calls: the device array and the host tables below are shared
std::mutex g_static_lock;

// host-side k tables (fixed size: no heap allocation)
KCol h_col[MAX_NKXY];
int4 h_kp[MAX_NK], h_grp[MAX_NK];
double h_kw[MAX_NK], h_kvir[GB_KVIR * MAX_NK];

const double PI = 3.141592653589793238462643383279502884;

size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

int cuda_fail(cudaError_t e, const char *what) {
  return ctx_set_error(e == cudaErrorMemoryAllocation ? GB_E_NOMEM : GB_E_CUDA,
                       std::string("CUDA error ") + cudaGetErrorString(e) + " at " + what);
}

#define SCK(x)                                         \
  do {                                                 \
    cudaError_t e_ = (x);                              \
    if (e_ != cudaSuccess) return cuda_fail(e_, #x);   \
  } while (0)

}  // namespace

extern "C" int gbrpmd_forces_ewald_static(double *r, double *v, double *dvdr, const int *nb,
                                          const int *na, const double *boxlxyz, const double *z,
                                          double *virial) {
  std::lock_guard<std::mutex> hold(g_static_lock);
  cudaStream_t s = cudaStreamPerThread;  // per-thread default stream: no stream object is created
  struct Drain {  // an error return still waits for the call's device work before the lock opens
    cudaStream_t s;
    ~Drain() { cudaStreamSynchronize(s); }
  } drain{s};
  const gb_params &P = current_params();
  const int B = *nb, n = *na;
  if (n <= 0 || n % 3 != 0) return ctx_set_error(GB_E_ARG, "potenl 1: na is not 3*nm");
  if (B <= 0 || B > MAX_NB) return ctx_set_error(GB_E_NOMEM, "static Ewald: nb must be 1..64");
  if ((long long)n * B > MAX_SITES) return ctx_set_error(GB_E_NOMEM, "static Ewald: na*nb exceeds 8192 sites");
  if (!P.iamcub) return ctx_set_error(GB_E_UNSUPPORTED, "non-cubic Ewald (ewald_nc) is not on the device path");
  if (P.wm > 0.0 || P.wh > 0.0) return ctx_set_error(GB_E_UNSUPPORTED, "smeared-charge Ewald is not on the device path");
  int dev = 0;
  SCK(cudaGetDevice(&dev));
  if (dev < 0 || dev >= MAX_DEVICES) return ctx_set_error(GB_E_ARG, "static Ewald: device index out of range");
  if (!g_scratch_ptr[dev]) {  // once per device, with that device current
    void *p = nullptr;
    SCK(cudaGetSymbolAddress(&p, g_static_scratch));
    g_scratch_ptr[dev] = (unsigned char *)p;
  }
  if (P.kmax < 0 || recip_sk_smem(P.kmax) > 227 * 1024 || recip_force_smem(P.kmax) > 227 * 1024)
    return ctx_set_error(GB_E_NOMEM, "static Ewald: kmax too large for the reciprocal-space kernels");
  KTables kt;
  if (gb_build_ktables(P, recip_group_len(), h_col, MAX_NKXY, h_kp, h_kw, MAX_NK, h_grp, MAX_NK, &kt) ||
      kt.nk > MAX_NK)
    return ctx_set_error(GB_E_NOMEM, "static Ewald: more than 2048 k vectors or 512 (kx, ky) columns");
  const int nchunk = (n + recip_sk_chunk() - 1) / recip_sk_chunk();
  const size_t N = 3 * (size_t)n * B;
  // partner slots per site: 1.1 times a uniform liquid's partners within the
  // cut-off (unit box), plus 48, at most every other site
  double onepivol = (4.0 / 3.0) * PI * P.wrcut * P.wrcut * P.wrcut;
  int cap = std::min((int)(1.1 * n * onepivol) + 48, n);
  // carve the buffer
  unsigned char *base = g_scratch_ptr[dev];
  size_t off = 0;
  auto take = [&](size_t bytes) {
    unsigned char *q = base + off;
    off = align256(off + bytes);
    return q;
  };
  double *d_r = (double *)take(sizeof(double) * N);
  double *d_rs = (double *)take(sizeof(double) * N);
  double *d_g = (double *)take(sizeof(double) * N);
  double *d_out = (double *)take(sizeof(double) * N);
  double *d_z = (double *)take(sizeof(double) * n);
  float4 *d_frac = (float4 *)take(sizeof(float4) * (size_t)n * B);
  int *d_cnt = (int *)take(sizeof(int) * (size_t)n * B);
  int *d_idx = (int *)take(sizeof(int) * (size_t)n * B * cap);
  KCol *d_col = (KCol *)take(sizeof(KCol) * kt.ncol);
  int4 *d_grp = (int4 *)take(sizeof(int4) * kt.ngrp);
  int4 *d_kp = (int4 *)take(sizeof(int4) * kt.nkp);
  double *d_kw = (double *)take(sizeof(double) * kt.nkp);
  double *d_kvir = (double *)take(sizeof(double) * GB_KVIR * kt.nkp);
  double2 *d_tab = (double2 *)take(sizeof(double2) * 3 * (size_t)(P.kmax + 1) * n * B);
  double *d_skp = (double *)take(sizeof(double) * 4 * (size_t)kt.nkp * nchunk * B);
  double *d_sk = (double *)take(sizeof(double) * 8 * (size_t)kt.nkp * B);
  double *d_acc = (double *)take(sizeof(double) * ACC_STRIDE);
  unsigned *d_status = (unsigned *)take(sizeof(unsigned));
  if (off > STATIC_SCRATCH_BYTES)
    return ctx_set_error(GB_E_NOMEM, "static Ewald: working set (" + std::to_string(off >> 10) + " KiB, " +
                                         std::to_string(cap) + " list slots per site) exceeds the 16 MiB buffer");

  SCK(cudaMemcpyAsync(d_r, r, sizeof(double) * N, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(d_z, z, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(d_col, h_col, sizeof(KCol) * kt.ncol, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(d_grp, h_grp, sizeof(int4) * kt.ngrp, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(d_kp, h_kp, sizeof(int4) * kt.nkp, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(d_kw, h_kw, sizeof(double) * kt.nkp, cudaMemcpyHostToDevice, s));
  gb_kvir_table(h_kp, kt.nkp, P.walpha, h_kvir);
  SCK(cudaMemcpyAsync(d_kvir, h_kvir, sizeof(double) * GB_KVIR * kt.nkp, cudaMemcpyHostToDevice, s));
  // cleared every call: gradient accumulator, energy/virial sums, status word
  SCK(cudaMemsetAsync(d_g, 0, sizeof(double) * N, s));
  SCK(cudaMemsetAsync(d_acc, 0, sizeof(double) * ACC_STRIDE, s));
  SCK(cudaMemsetAsync(d_status, 0, sizeof(unsigned), s));

  gb_context view;  // pointer view for the reciprocal launchers; owns nothing
  view.na = n;
  view.nb = B;
  view.nm = n / 3;
  view.P = P;
  view.ncol = kt.ncol;
  view.nkp = kt.nkp;
  view.ngrp = kt.ngrp;
  view.nk = kt.nk;
  view.kcol = d_col;
  view.kgrp = d_grp;
  view.kpair = d_kp;
  view.kw = d_kw;
  view.kvir = d_kvir;
  view.ktab = d_tab;
  view.sk_part = d_skp;
  view.sk = d_sk;
  recip_set_attributes();

  const double L = boxlxyz[0], onboxl = 1.0 / L;
  launch_msite(s, d_r, d_rs, n, B, P.alpha, onboxl);
  PairGeom g{};
  g.pos = d_rs;
  g.cstride = 3LL * n;
  g.pstride = 3;
  g.npt = n;
  g.unit = 1;
  g.box[0] = g.box[1] = g.box[2] = 1.0;
  g.onbox[0] = g.onbox[1] = g.onbox[2] = 1.0;
  g.rcutsq = P.wrcut * P.wrcut;
  g.excl_mol = 0;
  PairList pl;
  pl.nconf = B;
  pl.npt = n;
  pl.cap = cap;
  pl.count = d_cnt;
  pl.idx = d_idx;
  launch_frac32(s, g, B, d_frac);
  launch_build_list(s, g, B, d_frac, pl, d_status);
  launch_ewald_real(s, d_rs, d_z, n, B, pl, P.walpha, nullptr, d_g, d_acc);
  launch_recip_sk(s, &view, d_rs, d_z, B);
  launch_recip_weights(s, &view, B, d_acc);
  launch_recip_force(s, &view, d_rs, d_z, B, d_g);
  launch_msite_chain(s, d_g, d_out, n, B, P.alpha, onboxl * onboxl, 1.0, 0);
  SCK(cudaGetLastError());
  double acc[ACC_STRIDE];
  unsigned status = 0;
  SCK(cudaMemcpyAsync(dvdr, d_out, sizeof(double) * N, cudaMemcpyDeviceToHost, s));
  SCK(cudaMemcpyAsync(acc, d_acc, sizeof(double) * ACC_STRIDE, cudaMemcpyDeviceToHost, s));
  SCK(cudaMemcpyAsync(&status, d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  SCK(cudaStreamSynchronize(s));
  if (status & ST_LIST_OVERFLOW)
    return ctx_set_error(GB_E_LIST, "static Ewald: a site has more than " + std::to_string(cap) + " partners");
  double qq = 0.0;
  for (int i = 0; i < n; ++i) qq = qq + z[i] * z[i];
  const double vself = P.walpha / std::sqrt(PI) * qq;
  *v = (acc[0] - B * vself) / L / B;
  for (int i = 0; i < 9; ++i) virial[i] = acc[1 + i] / L / B;
  return GB_OK;
}
