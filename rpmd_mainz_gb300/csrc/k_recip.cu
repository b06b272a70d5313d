// k_recip.cu -- reciprocal-space Ewald sum in the unit box (FP64).
//
// Restates kwald (ewald_cubic.f90:235-533).  The reference walks the half
// space kx >= 0 with incremental cos/sin tables per site and combines the
// (+-ky, +-kz) partners into real sums; here the half space is cut into
// (kx, ky) columns, and within a column kz and -kz are taken together:
//   S(kx, ky, +-m) = P_m +- i Q_m,
//   P_m = sum_i q_i e^{i 2 pi (kx x_i + ky y_i)} cos(2 pi m z_i),  Q_m: sin,
// so a "k pair" costs two complex-times-real FMAs per site for both vectors
// (gb_kvec.h lists the pairs and their kinds).  Each k vector counts once with
// weight A_k = (4 pi / k^2) exp(-k^2 / (4 alpha^2)), the reference's 2 pi
// weight on k and -k.
//
// Per site the powers e^{i 2 pi m x}, m = 0..kmax, of the three coordinates are
// built once per evaluation by the reference's recurrence (x carries the
// charge): table [conf][site][axis][m] of double2.
//
// Pass 1 (k_recip_sk): a thread owns up to G consecutive m of one column, a
// block one chunk of sites; per site it forms c_xy = cx[kx] cy[ky] once and
// accumulates P and Q.  Chunk partials go to memory.
// Pass 2 (k_recip_weights): sums the partials in a fixed order, forms energy
// and virial, and stores per pair the force table built from
// A = S~(+m) + S~(-m), D = S~(+m) - S~(-m), S~ = 2 A_k S_k.
// Pass 3 (k_recip_force): per site and column, U = sum_kz conj(S~) cz and
// V = sum_kz kz conj(S~) cz are
//   U = c conj(A) + i d conj(D),   V = m (c conj(D) + i d conj(A)),
// (cz = c + i d), eight FMAs per pair; then t = -Im(c_xy U) gives the force
// 2 pi (kx t, ky t, -Im(c_xy V)) (ewald_cubic.f90:325-328).
#include "gb_common.cuh"
#include "gb_kernels.h"

namespace {

constexpr int SK_CHUNK = 32;  // sites per structure-factor block
constexpr int SK_G = 8;       // m values per structure-factor thread
constexpr int SK_T = 128;     // threads per structure-factor block
constexpr int F_T = 64;       // sites per force block
constexpr long long SIGN = (long long)0x8000000000000000ULL;

// flips the sign of v when mask is the sign bit (integer pipe, no FP64 op)
GB_D double flip(double v, long long mask) { return __longlong_as_double(__double_as_longlong(v) ^ mask); }

// per (conf, site, axis): powers e^{i lat m x}, m = 0..kmax, by the
// reference's recurrence (ewald_cubic.f90:254-286, ewald_noncubic.f90:296-336);
// lat = 2 pi in the unit box, 2 pi / L_axis for positions in bohr (non-cubic);
// the x table carries the charge
__global__ void k_recip_tables(const double *rs, const double *q, int na, int B, int kmax, double3 lat,
                               double2 *tab) {
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= 3LL * na * B) return;
  const int ax = (int)(w % 3);
  const int s = (int)((w / 3) % na);
  const double arg = (ax == 0 ? lat.x : ax == 1 ? lat.y : lat.z) * rs[w];
  double sn, cs;
  sincos(arg, &sn, &cs);
  double pr = ax == 0 ? q[s] : 1.0, pi = 0.0;
  double2 *t = tab + w * (kmax + 1);
  t[0] = make_double2(pr, pi);
  for (int k = 1; k <= kmax; ++k) {
    const double nr = cs * pr - sn * pi;
    const double ni = sn * pr + cs * pi;
    pr = nr;
    pi = ni;
    t[k] = make_double2(pr, pi);
  }
}

// item: x = kx | (len << 16), y = ky, z = first m, w = first k pair
__global__ void __launch_bounds__(SK_T) k_recip_sk(const double2 *tab, int na, int kmax, int ngrp,
                                                   const int4 *grp, int nkp, int nchunk, double4_32a *sk_part) {
  extern __shared__ double2 st[];  // [SK_CHUNK][3][K1]
  const int K1 = kmax + 1, K3 = 3 * K1;
  const int c = blockIdx.z, chunk = blockIdx.y;
  const int s0 = chunk * SK_CHUNK, ns = min(SK_CHUNK, na - s0);
  const double2 *src = tab + ((long long)c * na + s0) * K3;
  for (int w = threadIdx.x; w < ns * K3; w += SK_T) st[w] = src[w];
  __syncthreads();
  const int gi = blockIdx.x * SK_T + threadIdx.x;
  if (gi >= ngrp) return;
  const int4 gr = __ldg(grp + gi);
  const int kx = gr.x & 0xffff, len = gr.x >> 16, ky = gr.y, m0 = gr.z;
  const int aky = abs(ky);
  const long long ymask = ky < 0 ? SIGN : 0;  // cy(-ky) = conj(cy(ky))
  double pr[SK_G], pi[SK_G], qr[SK_G], qi[SK_G];
#pragma unroll
  for (int g = 0; g < SK_G; ++g) pr[g] = pi[g] = qr[g] = qi[g] = 0.0;
  for (int s = 0; s < ns; ++s) {
    const double2 *S = st + s * K3;
    const double2 X = S[kx], Y = S[K1 + aky];
    const double yi = flip(Y.y, ymask);
    const double cr = fma(X.x, Y.x, -X.y * yi);
    const double ci = fma(X.x, yi, X.y * Y.x);
    const double2 *Z = S + 2 * K1 + m0;
#pragma unroll
    for (int g = 0; g < SK_G; ++g) {
      if (g < len) {
        const double2 z = Z[g];
        pr[g] = fma(cr, z.x, pr[g]);
        pi[g] = fma(ci, z.x, pi[g]);
        qr[g] = fma(cr, z.y, qr[g]);
        qi[g] = fma(ci, z.y, qi[g]);
      }
    }
  }
  double4_32a *out = sk_part + ((long long)c * nchunk + chunk) * nkp + gr.w;
#pragma unroll
  for (int g = 0; g < SK_G; ++g)
    if (g < len) out[g] = make_double4_32a(pr[g], pi[g], qr[g], qi[g]);
}

// one block: 32 k pairs x 8 chunk slices; energy, virial and force tables
// (ewald_cubic.f90:308-328, 355-380, 408-440, 482-517)
__global__ void __launch_bounds__(256) k_recip_weights(const double4_32a *sk_part, int nchunk, int nkp,
                                                       const int4 *kpair, const double *kw, const double *kvir,
                                                       double4_32a *sk, double *acc) {
  __shared__ double4_32a part[8][32];
  __shared__ double sh[8 * 10];
  const int lane = threadIdx.x & 31, slice = threadIdx.x >> 5;
  const int c = blockIdx.y;
  const int k = blockIdx.x * 32 + lane;
  double4_32a a = make_double4_32a(0, 0, 0, 0);
  if (k < nkp) {
    for (int ch = slice; ch < nchunk; ch += 8) {
      const double4_32a p = sk_part[((long long)c * nchunk + ch) * nkp + k];
      a.x += p.x;
      a.y += p.y;
      a.z += p.z;
      a.w += p.w;
    }
  }
  part[slice][lane] = a;
  __syncthreads();
  double vals[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (slice == 0 && k < nkp) {
    double Pr = 0, Pi = 0, Qr = 0, Qi = 0;
    for (int j = 0; j < 8; ++j) {
      Pr += part[j][lane].x;
      Pi += part[j][lane].y;
      Qr += part[j][lane].z;
      Qi += part[j][lane].w;
    }
    const int4 kv = kpair[k];
    const double w = kw[k];
    double et, ed = 0.0, Ar, Ai, Dr, Di;  // ed: et(+m) - et(-m)
    if (kv.w == 1) {  // S(+-m) = P +- iQ
      et = 2.0 * w * (Pr * Pr + Pi * Pi + Qr * Qr + Qi * Qi);
      ed = 4.0 * w * (Pi * Qr - Pr * Qi);
      Ar = 4.0 * w * Pr;
      Ai = 4.0 * w * Pi;
      Dr = -4.0 * w * Qi;
      Di = 4.0 * w * Qr;
    } else if (kv.w == 2) {  // +m only: S = P + iQ, A = D = S~
      const double sr = Pr - Qi, si = Pi + Qr;
      et = w * (sr * sr + si * si);
      Ar = Dr = 2.0 * w * sr;
      Ai = Di = 2.0 * w * si;
    } else {  // m = 0: S = P
      et = w * (Pr * Pr + Pi * Pi);
      Ar = 2.0 * w * Pr;
      Ai = 2.0 * w * Pi;
      Dr = Di = 0.0;
    }
    vals[0] = et;
    // virial factors (gb_kvec.h): [0..8] on the summed energy, [9], [10] on the
    // difference for xz, yz (non-cubic sum; zero in the cubic one, whose
    // reference virial uses |k_a| |k_b|, ewald_cubic.f90:488-503)
    const double *kf = kvir + (long long)GB_KVIR * k;
#pragma unroll
    for (int e = 0; e < 9; ++e) vals[1 + e] = et * kf[e];
    vals[1 + 6] += ed * kf[9];
    vals[1 + 2] += ed * kf[9];
    vals[1 + 7] += ed * kf[10];
    vals[1 + 5] += ed * kf[10];
    const double m = (double)kv.z;
    double4_32a *o = sk + ((long long)c * nkp + k) * 2;
    o[0] = make_double4_32a(Ar, -Ai, Dr, Di);
    o[1] = make_double4_32a(m * Dr, m * Ai, -m * Di, m * Ar);
  }
  block_sum_atomic<10>(vals, sh, acc);
}

// g[i] += 2 pi sum_k k Im(S~_k conj(q_i e^{i 2 pi k.r_i})) over the columns
// whose first k pair lies in this block's share [seg nkp / nseg, (seg+1) nkp / nseg)
__global__ void __launch_bounds__(F_T) k_recip_force(const double2 *__restrict__ tab, int na, int kmax,
                                                     int ncol, const KCol *__restrict__ cols, int nkp,
                                                     const double4_32a *__restrict__ sk, double3 lat, double *g) {
  extern __shared__ double2 st[];  // [3][K1][F_T]
  const int K1 = kmax + 1, K3 = 3 * K1;
  const int c = blockIdx.z, t = threadIdx.x;
  const int i0 = blockIdx.x * F_T, i = i0 + t;
  for (int w = t; w < K3 * F_T; w += F_T) {
    const int e = w / F_T, sl = w % F_T;
    const int si = min(i0 + sl, na - 1);
    st[w] = tab[((long long)c * na + si) * K3 + e];
  }
  // the block's column range
  const long long kp_lo = (long long)blockIdx.y * nkp / gridDim.y;
  const long long kp_hi = (long long)(blockIdx.y + 1) * nkp / gridDim.y;
  auto first_col = [&](long long kp) {  // first column with koff >= kp
    int lo = 0, hi = ncol;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (__ldg(&cols[mid].koff) < kp) lo = mid + 1;
      else hi = mid;
    }
    return lo;
  };
  const int col0 = first_col(kp_lo), col1 = first_col(kp_hi);
  __syncthreads();
  const double4_32a *T = sk + (long long)c * nkp * 2;
  double fx = 0.0, fy = 0.0, fz = 0.0;
  for (int col = col0; col < col1; ++col) {
    const int4 ci4 = __ldg(reinterpret_cast<const int4 *>(cols + col));
    const double2 kd = __ldg(reinterpret_cast<const double2 *>(cols + col) + 1);
    const int kx = ci4.x, ky = ci4.y, koff = ci4.z, mlo = ci4.w & 0xffff, mhi = ci4.w >> 16;
    const double2 X = st[kx * F_T + t], Y = st[(K1 + abs(ky)) * F_T + t];
    const double yi = flip(Y.y, ky < 0 ? SIGN : 0);
    const double cr = fma(X.x, Y.x, -X.y * yi);
    const double ci = fma(X.x, yi, X.y * Y.x);
    const double4_32a *Tp = T + 2LL * (koff - mlo);
    const double2 *Z = st + 2 * K1 * F_T + t;
    double ur = 0.0, ui = 0.0, vr = 0.0, vi = 0.0;
    for (int m = mlo; m <= mhi; ++m) {
      const double2 z = Z[m * F_T];
      const double4_32a t0 = Tp[2 * m], t1 = Tp[2 * m + 1];
      ur = fma(z.x, t0.x, fma(z.y, t0.w, ur));
      ui = fma(z.x, t0.y, fma(z.y, t0.z, ui));
      vr = fma(z.x, t1.x, fma(z.y, t1.y, vr));
      vi = fma(z.x, t1.z, fma(z.y, t1.w, vi));
    }
    const double ts = -fma(cr, ui, ci * ur);
    fx = fma(kd.x, ts, fx);
    fy = fma(kd.y, ts, fy);
    fz = fz - fma(cr, vi, ci * vr);
  }
  if (i < na && col1 > col0) {
    double *G = g + ((long long)c * na + i) * 3;
    atomicAdd(G, lat.x * fx);
    atomicAdd(G + 1, lat.y * fy);
    atomicAdd(G + 2, lat.z * fz);
  }
}

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

int sm_count() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 1;
  return n;
}

}  // namespace

// 2 pi per axis for unit-box positions (cubic sum), 2 pi / L_axis for bohr (non-cubic)
double3 recip_lat(const gb_context *c) {
  const double twopi = 2.0 * acos(-1.0);
  if (c->P.iamcub) return make_double3(twopi, twopi, twopi);
  return make_double3(twopi / c->box[0], twopi / c->box[1], twopi / c->box[2]);
}

int recip_sk_chunk() { return SK_CHUNK; }
int recip_group_len() { return SK_G; }
size_t recip_sk_smem(int kmax) { return sizeof(double2) * SK_CHUNK * 3 * (kmax + 1); }
size_t recip_force_smem(int kmax) { return sizeof(double2) * 3 * (kmax + 1) * F_T; }

void launch_recip_sk(cudaStream_t s, gb_context *c, const double *rs, const double *q, int B) {
  if (c->nkp == 0) return;  // no k vector inside rkmax
  const int kmax = c->P.kmax;
  const long long nw = 3LL * c->na * B;
  k_recip_tables<<<nblk(nw, 128), 128, 0, s>>>(rs, q, c->na, B, kmax, recip_lat(c), c->ktab);
  const int nchunk = (c->na + SK_CHUNK - 1) / SK_CHUNK;
  dim3 grid(nblk(c->ngrp, SK_T), nchunk, B);
  k_recip_sk<<<grid, SK_T, recip_sk_smem(kmax), s>>>(c->ktab, c->na, kmax, c->ngrp, c->kgrp, c->nkp, nchunk,
                                                     (double4_32a *)c->sk_part);
}

void launch_recip_weights(cudaStream_t s, gb_context *c, int B, double *acc) {
  if (c->nkp == 0) return;
  const int nchunk = (c->na + SK_CHUNK - 1) / SK_CHUNK;
  dim3 grid(nblk(c->nkp, 32), B);
  k_recip_weights<<<grid, 256, 0, s>>>((const double4_32a *)c->sk_part, nchunk, c->nkp, c->kpair, c->kw, c->kvir,
                                       (double4_32a *)c->sk, acc);
}

void launch_recip_force(cudaStream_t s, gb_context *c, const double *rs, const double *q, int B,
                        double *g) {
  (void)rs;
  (void)q;
  if (c->nkp == 0) return;
  const int kmax = c->P.kmax;
  const unsigned bx = nblk(c->na, F_T);
  // about eight blocks per SM over all configurations, at most 16 column shares
  const long long want = 8LL * sm_count();
  int nseg = (int)((want + (long long)bx * B - 1) / ((long long)bx * B));
  nseg = std::max(1, std::min(16, std::min(nseg, c->ncol)));
  dim3 grid(bx, nseg, B);
  k_recip_force<<<grid, F_T, recip_force_smem(kmax), s>>>(c->ktab, c->na, kmax, c->ncol, c->kcol, c->nkp,
                                                          (const double4_32a *)c->sk, recip_lat(c), g);
}

// The dynamic shared-memory limit is a per-kernel property of the process, so
// it is raised once to the largest size any context may request (227 KB).
void recip_set_attributes() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_recip_sk, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  cudaFuncSetAttribute(k_recip_force, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
  done = true;
}
