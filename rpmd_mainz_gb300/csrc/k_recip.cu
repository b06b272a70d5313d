// k_recip.cu -- reciprocal-space Ewald sum in the unit box (FP64).
//
// Restates kwald (ewald_cubic.f90:235-533).  The reference walks the half
// space kx >= 0 with incremental cos/sin tables per site and combines the
// (+-ky, +-kz) partners into 4 or 8 real sums; here every k vector of the half
// space {kx > 0} u {kx = 0, ky > 0} u {kx = ky = 0, kz > 0} is kept once with
// weight (4 pi / k^2) exp(-k^2 / (4 alpha^2)), which equals the reference's
// 2 pi weight on both k and -k.  Membership follows the reference's loop exits
// (|k|^2 <= rkmax^2, decided on the host with the reference's rounding).
//
// Pass 1 (structure factors): one block per (configuration, chunk of sites),
// one thread per (kx, ky) column; the column's kz values accumulate in shared
// memory, e^{i k.r} = cx[kx] cy[ky] cz[kz] from per-site power tables built by
// the reference's recurrence.  Pass 2 sums the chunk partials in fixed order
// and forms energy, virial and the force weights 2 A_k S_k.  Pass 3: one
// thread per site sums sum_k (2 A_k) k Im(S_k conj(q e^{i k.r})).
#include "gb_common.cuh"
#include "gb_kernels.h"

namespace {

constexpr int SK_CHUNK = 64;

// per-site power tables exp(i 2 pi m x), m = 0..kmax, by the reference's
// recurrence (ewald_cubic.f90:254-286); the x table carries the charge
GB_D void site_tables(double x, double q0, int kmax, double *tr, double *ti, int stride) {
  const double arg = 2.0 * acos(-1.0) * x;
  double s, c;
  sincos(arg, &s, &c);
  double pr = q0, pi = 0.0;
  tr[0] = pr;
  ti[0] = pi;
  for (int k = 1; k <= kmax; ++k) {
    const double nr = c * pr - s * pi;
    const double ni = s * pr + c * pi;
    pr = nr;
    pi = ni;
    tr[k * stride] = pr;
    ti[k * stride] = pi;
  }
}

__global__ void k_recip_sk(const double *rs, const double *q, int na, int kmax, int nkxy,
                           const int4 *kxy, const int *koff, int nk, int nchunk, double *sk_part) {
  extern __shared__ double sm[];
  const int K1 = kmax + 1, T = blockDim.x;
  double *cxr = sm, *cxi = cxr + SK_CHUNK * K1;
  double *cyr = cxi + SK_CHUNK * K1, *cyi = cyr + SK_CHUNK * K1;
  double *czr = cyi + SK_CHUNK * K1, *czi = czr + SK_CHUNK * K1;
  double *accr = czi + SK_CHUNK * K1, *acci = accr + (2 * kmax + 1) * T;
  const int c = blockIdx.y, chunk = blockIdx.x;
  const int s0 = chunk * SK_CHUNK, ns = min(SK_CHUNK, na - s0);
  const double *R = rs + ((long long)c * na + s0) * 3;
  for (int w = threadIdx.x; w < ns * 3; w += T) {
    const int s = w / 3, ax = w % 3;
    double *tr = ax == 0 ? cxr : (ax == 1 ? cyr : czr);
    double *ti = ax == 0 ? cxi : (ax == 1 ? cyi : czi);
    site_tables(R[3 * s + ax], ax == 0 ? q[s0 + s] : 1.0, kmax, tr + s * K1, ti + s * K1, 1);
  }
  for (int w = threadIdx.x; w < (2 * kmax + 1) * T; w += T) {
    accr[w] = 0.0;
    acci[w] = 0.0;
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t < nkxy) {
    const int4 kk = kxy[t];
    const int kx = kk.x, aky = abs(kk.y), lo = kk.z, hi = kk.w;
    const double sy = kk.y < 0 ? -1.0 : 1.0;
    for (int s = 0; s < ns; ++s) {
      const double ar = cxr[s * K1 + kx], ai = cxi[s * K1 + kx];
      const double br = cyr[s * K1 + aky], bi = sy * cyi[s * K1 + aky];
      const double cr = ar * br - ai * bi, ci = ar * bi + ai * br;
      for (int kz = lo; kz <= hi; ++kz) {
        const int akz = abs(kz);
        const double dr = czr[s * K1 + akz], di = kz < 0 ? -czi[s * K1 + akz] : czi[s * K1 + akz];
        const int slot = (kz + kmax) * T + t;
        accr[slot] += cr * dr - ci * di;
        acci[slot] += cr * di + ci * dr;
      }
    }
    double *out = sk_part + ((long long)(c * nchunk + chunk) * nk + koff[t]) * 2;
    for (int kz = lo; kz <= hi; ++kz) {
      const int slot = (kz + kmax) * T + t;
      out[2 * (kz - lo)] = accr[slot];
      out[2 * (kz - lo) + 1] = acci[slot];
    }
  }
}

// sums the chunk partials; energy, virial, force weights (ewald_cubic.f90:308-328 etc.)
__global__ void k_recip_weights(const double *sk_part, int nchunk, int nk, int B, const int4 *klist,
                                const double *kw, double bfac, double *sk, double *acc) {
  __shared__ double sh[32 * 10];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double vals[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (t < (long long)nk * B) {
    const int c = (int)(t / nk), k = (int)(t % nk);
    double sr = 0.0, si = 0.0;
    for (int ch = 0; ch < nchunk; ++ch) {
      const double *p = sk_part + ((long long)(c * nchunk + ch) * nk + k) * 2;
      sr += p[0];
      si += p[1];
    }
    const int4 kv = klist[k];
    const double rlat = 2.0 * acos(-1.0);
    const double rk[3] = {rlat * kv.x, rlat * kv.y, rlat * kv.z};
    const double rk2 = rk[0] * rk[0] + rk[1] * rk[1] + rk[2] * rk[2];
    const double w = kw[k];
    const double et = w * (sr * sr + si * si);
    const double term = 2.0 * (1.0 / rk2 + bfac);
    vals[0] = et;
    // the reference combines the (+-ky, +-kz) partners into one energy and
    // multiplies it by term * rk_a * rk_b with rk_y, rk_z >= 0, so its
    // off-diagonal virial uses |k_a| |k_b| (ewald_cubic.f90:488-503)
#pragma unroll
    for (int b = 0; b < 3; ++b)
#pragma unroll
      for (int a = 0; a < 3; ++a)
        vals[1 + a + 3 * b] = et * (term * fabs(rk[a]) * fabs(rk[b]) - (a == b ? 1.0 : 0.0));
    double *o = sk + ((long long)c * nk + k) * 2;
    o[0] = 2.0 * w * sr;
    o[1] = 2.0 * w * si;
  }
  block_sum_atomic<10>(vals, sh, acc);
}

// g[i] += sum_k (2 A_k) (2 pi k) Im(S_k conj(q_i e^{i 2 pi k.r_i}))
__global__ void k_recip_force(const double *rs, const double *q, int na, int kmax, int nkxy,
                              const int4 *kxy, const int *koff, int nk, const double *sk, double *g) {
  extern __shared__ double sm[];
  const int K1 = kmax + 1, T = blockDim.x;
  double *cxr = sm, *cxi = cxr + K1 * T, *cyr = cxi + K1 * T, *cyi = cyr + K1 * T;
  double *czr = cyi + K1 * T, *czi = czr + K1 * T;
  const int c = blockIdx.y;
  const int i = blockIdx.x * T + threadIdx.x;
  const bool valid = i < na;
  const int t = threadIdx.x;
  if (valid) {
    const double *R = rs + ((long long)c * na + i) * 3;
    site_tables(R[0], q[i], kmax, cxr + t, cxi + t, T);
    site_tables(R[1], 1.0, kmax, cyr + t, cyi + t, T);
    site_tables(R[2], 1.0, kmax, czr + t, czi + t, T);
  }
  __syncthreads();
  if (!valid) return;
  const double *S = sk + (long long)c * nk * 2;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int pr = 0; pr < nkxy; ++pr) {
    const int4 kk = __ldg(kxy + pr);
    const int kx = kk.x, aky = abs(kk.y), lo = kk.z, hi = kk.w;
    const double ar = cxr[kx * T + t], ai = cxi[kx * T + t];
    const double br = cyr[aky * T + t], bi = kk.y < 0 ? -cyi[aky * T + t] : cyi[aky * T + t];
    const double cr = ar * br - ai * bi, ci = ar * bi + ai * br;
    const double *Sp = S + 2LL * __ldg(koff + pr);
    double ur_s = 0.0, ui_s = 0.0, vr_s = 0.0, vi_s = 0.0;
    for (int kz = lo; kz <= hi; ++kz) {
      const int akz = abs(kz);
      const double dr = czr[akz * T + t], di = kz < 0 ? -czi[akz * T + t] : czi[akz * T + t];
      const double sr = __ldg(Sp + 2 * (kz - lo)), si = __ldg(Sp + 2 * (kz - lo) + 1);
      const double ur = sr * dr + si * di, ui = sr * di - si * dr;
      ur_s += ur;
      ui_s += ui;
      vr_s += (double)kz * ur;
      vi_s += (double)kz * ui;
    }
    // t = S_i e_r - S_r e_i (ewald_cubic.f90:325) = -Im(cxy * sum conj(S) cz)
    const double ts = -(cr * ui_s + ci * ur_s);
    const double tz = -(cr * vi_s + ci * vr_s);
    fx += (double)kx * ts;
    fy += (double)kk.y * ts;
    fz += tz;
  }
  const double rlat = 2.0 * acos(-1.0);
  double *G = g + ((long long)c * na + i) * 3;
  G[0] += rlat * fx;
  G[1] += rlat * fy;
  G[2] += rlat * fz;
}

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

void launch_recip_sk(cudaStream_t s, gb_context *c, const double *rs, const double *q, int B) {
  const int kmax = c->P.kmax;
  const int T = ((c->nkxy + 31) / 32) * 32;
  const int nchunk = (c->na + SK_CHUNK - 1) / SK_CHUNK;
  const size_t smem = sizeof(double) * (6 * SK_CHUNK * (kmax + 1) + 2 * (2 * kmax + 1) * T);
  dim3 grid(nchunk, B);
  k_recip_sk<<<grid, T, smem, s>>>(rs, q, c->na, kmax, c->nkxy, (const int4 *)c->kxy, c->kxy_koff,
                                   c->nk, nchunk, c->sk_part);
}

void launch_recip_weights(cudaStream_t s, gb_context *c, int B, double *acc) {
  const int nchunk = (c->na + SK_CHUNK - 1) / SK_CHUNK;
  const double bfac = 0.25 / (c->P.walpha * c->P.walpha);
  long long n = (long long)c->nk * B;
  k_recip_weights<<<nblk(n, 128), 128, 0, s>>>(c->sk_part, nchunk, c->nk, B, c->klist, c->kw, bfac,
                                               c->sk, acc);
}

void launch_recip_force(cudaStream_t s, gb_context *c, const double *rs, const double *q, int B,
                        double *g) {
  const int kmax = c->P.kmax;
  const int T = 128;
  const size_t smem = sizeof(double) * 6 * (kmax + 1) * T;
  dim3 grid(nblk(c->na, T), B);
  k_recip_force<<<grid, T, smem, s>>>(rs, q, c->na, kmax, c->nkxy, (const int4 *)c->kxy, c->kxy_koff,
                                      c->nk, c->sk, g);
}

// shared-memory need of the structure-factor pass (for the attribute set-up)
size_t recip_sk_smem(int kmax, int nkxy) {
  const int T = ((nkxy + 31) / 32) * 32;
  return sizeof(double) * (6 * SK_CHUNK * (kmax + 1) + 2 * (2 * kmax + 1) * T);
}
size_t recip_force_smem(int kmax) { return sizeof(double) * 6 * (kmax + 1) * 128; }
int recip_sk_chunk() { return SK_CHUNK; }
// The dynamic shared-memory limit is a per-kernel property of the process, so
// it is raised once to the largest size any context may request (227 KB).
void recip_set_attributes(size_t sk_smem, size_t f_smem) {
  (void)sk_smem;
  (void)f_smem;
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_recip_sk, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  cudaFuncSetAttribute(k_recip_force, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  done = true;
}
