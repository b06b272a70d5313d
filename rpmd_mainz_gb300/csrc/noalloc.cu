// noalloc.cu -- the Ewald force entry point that allocates no device memory.
//
// gbrpmd_forces_ewald_static computes what gbrpmd_forces computes for
// iopt = 2 (M-site substitution, real-space and reciprocal Ewald sums, chain
// rule; bead-averaged energy and virial), but every device buffer it needs --
// positions, pair lists, structure factors, accumulators -- lives in one
// file-scope __device__ array of STATIC_SCRATCH_BYTES (16 MiB).  It is meant for
// callers that may not call cudaMalloc themselves or through us: hosts that run
// under a fixed device-memory budget handed out by another framework's pool, or
// codes that must not trigger allocation (and the implicit synchronisation a
// cudaFree brings) in the middle of their own stream work.
//
// The array is part of the module image: every GPU that loads the library
// reserves the 16 MiB until the process exits.  Host code only knows a
// host-side stand-in for the array's name, so the device address is fetched
// once per device with cudaGetSymbolAddress, with that device current, on the
// first call made on that device; make that first call before any stream
// capture.  The buffer is shared by all calls: each call clears the parts that
// must start at zero, and calls that overlap on the GPU (from several host
// threads) race on it.
//
// Limits (rejected with GB_E_NOMEM and a message): na * nb <= 8192 sites,
// nb <= 64, at most 2048 k vectors in 512 (kx, ky) columns, and every buffer
// together within 16 MiB; pair lists hold at most 192 partners per site
// (overflow is reported as GB_E_LIST).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "gb_common.cuh"
#include "gb_context.h"
#include "gb_kernels.h"

size_t recip_sk_smem(int kmax, int nkxy);
size_t recip_force_smem(int kmax);
int recip_sk_chunk();
void recip_set_attributes(size_t sk_smem, size_t f_smem);
const gb_params &current_params();
int ctx_set_error(int code, const std::string &msg);

namespace {

constexpr size_t STATIC_SCRATCH_BYTES = 16u << 20;
constexpr int MAX_SITES = 8192;
constexpr int MAX_NB = 64;
constexpr int MAX_NK = 2048;
constexpr int MAX_NKXY = 512;
constexpr int MAX_CAP = 192;
constexpr int MAX_DEVICES = 64;

__device__ __align__(256) unsigned char g_static_scratch[STATIC_SCRATCH_BYTES];

unsigned char *g_scratch_ptr[MAX_DEVICES] = {nullptr};

// host-side k tables (fixed size: no heap allocation)
int h_kxy[4 * MAX_NKXY], h_koff[MAX_NKXY], h_klist[4 * MAX_NK];
double h_kw[MAX_NK];

const double PI = 3.141592653589793238462643383279502884;

// the reference's half-space k vectors (ewald_cubic.f90:292-520), grouped in
// (kx, ky) columns sorted by kz range; returns GB_OK or an error
int kvectors(const gb_params &P, int *nkxy, int *nk) {
  const int kmax = P.kmax;
  const double rlat = 2.0 * PI, rkmax2 = P.rkmax * P.rkmax, b = 0.25 / (P.walpha * P.walpha);
  int cols[4 * MAX_NKXY];
  int nc = 0;
  auto push = [&](int kx, int ky, int lo, int hi) {
    if (nc >= MAX_NKXY) return false;
    cols[4 * nc] = kx; cols[4 * nc + 1] = ky; cols[4 * nc + 2] = lo; cols[4 * nc + 3] = hi;
    ++nc;
    return true;
  };
  for (int kx = 0; kx <= kmax; ++kx) {
    const double rkx = rlat * kx;
    int kz0 = 0;
    for (int kz = 1; kz <= kmax; ++kz) {
      double rkz = rlat * kz;
      if (rkx * rkx + rkz * rkz > rkmax2) break;
      kz0 = kz;
    }
    bool ok = true;
    if (kx > 0) ok = push(kx, 0, -kz0, kz0);
    else if (kz0 > 0) ok = push(0, 0, 1, kz0);
    if (!ok) return ctx_set_error(GB_E_NOMEM, "static Ewald: more than 512 (kx, ky) columns");
    for (int ky = 1; ky <= kmax; ++ky) {
      const double rky = rlat * ky;
      if (rkx * rkx + rky * rky > rkmax2) break;
      int kzm = 0;
      for (int kz = 1; kz <= kmax; ++kz) {
        double rkz = rlat * kz;
        if (rkx * rkx + rky * rky + rkz * rkz > rkmax2) break;
        kzm = kz;
      }
      if (!push(kx, ky, -kzm, kzm) || (kx > 0 && !push(kx, -ky, -kzm, kzm)))
        return ctx_set_error(GB_E_NOMEM, "static Ewald: more than 512 (kx, ky) columns");
    }
  }
  // insertion sort by descending kz range (stable)
  for (int i = 1; i < nc; ++i) {
    int t[4] = {cols[4 * i], cols[4 * i + 1], cols[4 * i + 2], cols[4 * i + 3]};
    int j = i - 1;
    while (j >= 0 && (cols[4 * j + 3] - cols[4 * j + 2]) < (t[3] - t[2])) {
      for (int d = 0; d < 4; ++d) cols[4 * (j + 1) + d] = cols[4 * j + d];
      --j;
    }
    for (int d = 0; d < 4; ++d) cols[4 * (j + 1) + d] = t[d];
  }
  int n = 0;
  for (int p = 0; p < nc; ++p) {
    for (int d = 0; d < 4; ++d) h_kxy[4 * p + d] = cols[4 * p + d];
    h_koff[p] = n;
    for (int kz = cols[4 * p + 2]; kz <= cols[4 * p + 3]; ++kz) {
      if (n >= MAX_NK) return ctx_set_error(GB_E_NOMEM, "static Ewald: more than 2048 k vectors");
      h_klist[4 * n] = cols[4 * p]; h_klist[4 * n + 1] = cols[4 * p + 1];
      h_klist[4 * n + 2] = kz; h_klist[4 * n + 3] = p;
      double rkx = rlat * cols[4 * p], rky = rlat * cols[4 * p + 1], rkz = rlat * kz;
      double rk2 = rkx * rkx + rky * rky + rkz * rkz;
      h_kw[n] = (2.0 * rlat / rk2) * std::exp(-b * rk2);
      ++n;
    }
  }
  *nkxy = nc;
  *nk = n;
  return GB_OK;
}

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
  int nkxy = 0, nk = 0;
  int st = kvectors(P, &nkxy, &nk);
  if (st) return st;
  if (recip_sk_smem(P.kmax, nkxy) > 227 * 1024 || recip_force_smem(P.kmax) > 227 * 1024)
    return ctx_set_error(GB_E_NOMEM, "static Ewald: kmax too large for the reciprocal-space kernels");
  const int nchunk = (n + recip_sk_chunk() - 1) / recip_sk_chunk();
  const size_t N = 3 * (size_t)n * B;
  double onepivol = (4.0 / 3.0) * PI * P.wrcut * P.wrcut * P.wrcut;
  int cap = std::min(std::min((int)(1.1 * n * onepivol) + 48, n), MAX_CAP);
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
  int *d_kxy = (int *)take(sizeof(int) * 4 * nkxy);
  int *d_koff = (int *)take(sizeof(int) * nkxy);
  int4 *d_klist = (int4 *)take(sizeof(int4) * nk);
  double *d_kw = (double *)take(sizeof(double) * nk);
  double *d_skp = (double *)take(sizeof(double) * 2 * (size_t)nk * nchunk * B);
  double *d_sk = (double *)take(sizeof(double) * 2 * (size_t)nk * B);
  double *d_acc = (double *)take(sizeof(double) * ACC_STRIDE);
  unsigned *d_status = (unsigned *)take(sizeof(unsigned));
  if (off > STATIC_SCRATCH_BYTES) return ctx_set_error(GB_E_NOMEM, "static Ewald: working set exceeds the 16 MiB buffer");

  cudaStream_t s = 0;  // legacy default stream: no stream object is created
  SCK(cudaMemcpyAsync(d_r, r, sizeof(double) * N, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(d_z, z, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(d_kxy, h_kxy, sizeof(int) * 4 * nkxy, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(d_koff, h_koff, sizeof(int) * nkxy, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(d_klist, h_klist, sizeof(int) * 4 * nk, cudaMemcpyHostToDevice, s));
  SCK(cudaMemcpyAsync(d_kw, h_kw, sizeof(double) * nk, cudaMemcpyHostToDevice, s));
  // cleared every call: gradient accumulator, energy/virial sums, status word
  SCK(cudaMemsetAsync(d_g, 0, sizeof(double) * N, s));
  SCK(cudaMemsetAsync(d_acc, 0, sizeof(double) * ACC_STRIDE, s));
  SCK(cudaMemsetAsync(d_status, 0, sizeof(unsigned), s));

  gb_context view;  // pointer view for the reciprocal launchers; owns nothing
  view.na = n;
  view.nb = B;
  view.nm = n / 3;
  view.P = P;
  view.nkxy = nkxy;
  view.nk = nk;
  view.kxy = d_kxy;
  view.kxy_koff = d_koff;
  view.klist = d_klist;
  view.kw = d_kw;
  view.sk_part = d_skp;
  view.sk = d_sk;
  recip_set_attributes(recip_sk_smem(P.kmax, nkxy), recip_force_smem(P.kmax));

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
  launch_ewald_real(s, d_rs, d_z, n, B, pl, P.walpha, d_g, d_acc);
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
  if (status & ST_LIST_OVERFLOW) return ctx_set_error(GB_E_LIST, "static Ewald: more than 192 partners per site");
  double qq = 0.0;
  for (int i = 0; i < n; ++i) qq = qq + z[i] * z[i];
  const double vself = P.walpha / std::sqrt(PI) * qq;
  *v = (acc[0] - B * vself) / L / B;
  for (int i = 0; i < 9; ++i) virial[i] = acc[1 + i] / L / B;
  return GB_OK;
}
