// k_modes.cu -- normal-mode transforms, free ring-polymer propagation,
// ring-polymer contraction, intramolecular forces and the virial kinetic
// energy estimator (FP64), one thread per coordinate row or per molecule.
#include <cmath>
#include <type_traits>

#include "gb_common.cuh"
#include "gb_df.cuh"
#include "gb_fft.cuh"
#include "gb_intra.cuh"
#include "gb_kernels.h"

namespace {

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// realft on rows: data(m, n) column-major, row k = data[k + m*j] (fourier.f90:47-61)
template <int N>
__global__ void k_realft_pow2(const double *in, double *out, int m, int mode, const double *tw,
                              double scale) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= m) return;
  double x[N], y[N];
#pragma unroll
  for (int j = 0; j < N; ++j) x[j] = in[row + (long long)m * j];
  if (mode == 1) gb_r2hc<N>(x, y, tw); else gb_hc2r<N>(x, y, tw);
#pragma unroll
  for (int j = 0; j < N; ++j) out[row + (long long)m * j] = scale * y[j];
}

constexpr int NMAX_DIRECT = 256;  // longest generic transform (fourier.f90:19, nmax)
constexpr int NMAXC = 64;         // longest contracted ring on the device (nbdf1, nbdf2)

__global__ void k_realft_direct(const double *in, double *out, int m, int n, int mode,
                                const double *tw, double scale) {
  const int row = blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= m) return;
  double x[NMAX_DIRECT], y[NMAX_DIRECT];
  for (int j = 0; j < n; ++j) x[j] = in[row + (long long)m * j];
  if (mode == 1) gb_r2hc_direct(x, y, n, tw); else gb_hc2r_direct(x, y, n, tw);
  for (int j = 0; j < n; ++j) out[row + (long long)m * j] = scale * y[j];
}

// free ring-polymer step in normal modes (evolve_pi.f90:109-125):
// p' = p m1 + r m2, r' = p m3 + r m4 with the atom type's monodromy of mode k
__global__ void k_rotate(double *p, double *r, const double *monod, int na, int nb) {
  const long long S = 3LL * na;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= S * nb) return;
  const int k = (int)(t / S);
  const int row = (int)(t % S);
  const int ic = (row / 3) % 3;
  const double *m = monod + ic + 12 * k;  // monod(ic, c, k) at ic + 3*(c + 4*k)
  const double pv = p[t], rv = r[t];
  const double pprime = pv * m[0] + rv * m[3];
  r[t] = pv * m[6] + rv * m[9];
  p[t] = pprime;
}

__global__ void k_axpy(double *y, const double *x, double a, long long n) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) y[t] = y[t] + a * x[t];
}

__global__ void k_copy(double *dst, const double *src, long long n) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) dst[t] = src[t];
}

// ring_contract (evolve_pi.f90:405-431): keep modes 0, 1..h, nb-h..nb-1 of
// rnm, HC2R of length nbc, scale 1/sqrt(nbc) then sqrt(nbc/nb)
__global__ void k_ring_contract(const double *rnm, double *rb, int na, int nb, int nbc,
                                const double *tw_c, double s1, double s2) {
  const long long S = 3LL * na;
  const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= S) return;
  double x[NMAXC], y[NMAXC];
  const int h = (nbc - 1) / 2;
  x[0] = rnm[row];
  for (int k = 1; k <= h; ++k) {
    x[k] = rnm[row + S * k];
    x[nbc - k] = rnm[row + S * (nb - k)];
  }
  gb_hc2r_direct(x, y, nbc, tw_c);
  for (int j = 0; j < nbc; ++j) rb[row + S * j] = s2 * (s1 * y[j]);
}

// force_contract (evolve_pi.f90:377-403) of up to two contracted terms, sum in
// normal modes, HC2R of length nb (evolve_pi.f90:238-247), bead-rep extras
// added, optional kick p -= halfdt * dvdr (evolve_pi.f90:279)
__global__ void k_expand_forces(double *dvdr, const double *fb1, int nbc1, const double *tw_c1,
                                const double *fb2, int nbc2, const double *tw_c2, const double *e1,
                                const double *e2, const double *e3, double *p, double halfdt,
                                int na, int nb, const double *tw_nb, unsigned *status) {
  const long long S = 3LL * na;
  const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (row >= S) return;
  double xr[NMAXC / 2 + 1], xi[NMAXC / 2 + 1];  // X_k, k = 0..hmax
  int hmax = 0;
  double tmp[NMAXC], hc[NMAXC];
  const double *fbs[2] = {fb1, fb2};
  const int nbcs[2] = {nbc1, nbc2};
  const double *tws[2] = {tw_c1, tw_c2};
  for (int k = 0; k <= NMAXC / 2; ++k) xr[k] = xi[k] = 0.0;
  for (int t = 0; t < 2; ++t) {
    if (!fbs[t]) continue;
    const int nbc = nbcs[t], h = (nbc - 1) / 2;
    for (int j = 0; j < nbc; ++j) tmp[j] = fbs[t][row + S * j];
    gb_r2hc_direct(tmp, hc, nbc, tws[t]);
    const double s1 = sqrt(1.0 / (double)nbc), s2 = sqrt((double)nb / (double)nbc);
    xr[0] += s2 * (s1 * hc[0]);
    for (int k = 1; k <= h; ++k) {
      xr[k] += s2 * (s1 * hc[k]);
      xi[k] += s2 * (s1 * hc[nbc - k]);
    }
    hmax = max(hmax, h);
  }
  const double sc = sqrt(1.0 / (double)nb);
  bool bad = false;
  for (int j = 0; j < nb; ++j) {
    double s = xr[0];
    int m = 0;
    for (int k = 1; k <= hmax; ++k) {
      m += j;
      if (m >= nb) m -= nb;
      s += 2.0 * (xr[k] * tw_nb[m] - xi[k] * tw_nb[nb + m]);
    }
    double v = (fb1 || fb2) ? sc * s : 0.0;
    const long long o = row + S * j;
    if (e1) v += e1[o];
    if (e2) v += e2[o];
    if (e3) v += e3[o];
    dvdr[o] = v;
    bad |= gb_nonfinite(v);
    if (p) p[o] = p[o] - halfdt * v;
  }
  gb_flag_nonfinite(status, bad);
}

// The same expansion for contracted rings of at most 2*HM+1 beads: the
// contracted forces of a row are reduced to NQ = 2*HM+1 mode coefficients
// (force_contract, evolve_pi.f90:377-403), and each bead's value is the dot
// product with a per-bead table E[j] = sqrt(1/nb) (1, 2 cos(2 pi jk/nb),
// -2 sin(2 pi jk/nb), k = 1..HM) held in shared memory.  R = float runs the
// contraction and the dot product in FP32 (mixed precision; FP64 loads and
// stores through the integer conversions of gb_df.cuh); the kick stays FP64.
// A block takes XR coordinate rows: XR threads reduce the rows' contracted
// forces to coefficients (shared memory), then all XT threads expand them, four
// threads per row each over a quarter of the beads, consecutive rows in
// consecutive lanes so that every bead plane is written coalesced.
// sc[t] = (sqrt(1/nbc_t), sqrt(nb/nbc_t)) of the two contracted terms, sc =
// sqrt(1/nb) (from the host: no per-thread FP64 square roots).
constexpr int XR = 32;
constexpr int XT = 4 * XR;
constexpr int XPJ = 8;  // momenta per thread staged in shared memory (rings of nb <= 4 XPJ)

// 8-byte asynchronous copy global -> shared (cp.async, sm_80 and later): no
// register holds the value, so the copy runs while the thread computes
GB_D void cp_async8(double *smem, const double *gmem) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gmem) : "memory");
}
GB_D void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

template <int HM, typename R>
__global__ void __launch_bounds__(XT) k_expand_table(double *dvdr, const double *fb1, int nbc1, const double *tw_c1,
                                                     const double *fb2, int nbc2, const double *tw_c2,
                                                     const double *e1, const double *e2, const double *e3, double *p,
                                                     double halfdt, int na, int nb, const double *tw_nb,
                                                     double2 sc1, double2 sc2, double sc, unsigned *status) {
  constexpr int NQ = 2 * HM + 1;
  constexpr bool F32 = std::is_same<R, float>::value;
  extern __shared__ double smx[];
  R *E = reinterpret_cast<R *>(smx);  // [nb][NQ]
  R *CF = E + nb * NQ;                // [XR][NQ]
  const long long S = 3LL * na;
  const bool any = fb1 || fb2;
  const int lr = threadIdx.x % XR, grp = threadIdx.x / XR;
  const long long row = (long long)blockIdx.x * XR + lr;
  const int j0 = grp * nb / 4, j1 = (grp + 1) * nb / 4;
  // the momenta this thread kicks, copied to shared memory asynchronously
  // first: their loads are all in flight at once and overlap the
  // coefficients' computation, instead of one load round trip per bead in
  // the bead loop (rings of at most 4 XPJ beads; longer ones load them there,
  // and the launch leaves the staging area out of their shared memory)
  double *PS = smx + (size_t)(nb + XR) * NQ;  // [XPJ][XT], after E and CF
  const bool pre = p != nullptr && row < S && nb <= 4 * XPJ;
  if (pre) {
#pragma unroll 1
    for (int u = 0; u < j1 - j0; ++u) cp_async8(PS + u * XT + threadIdx.x, p + row + S * (j0 + u));
  }
  if (grp == 0 && row < S) {
    R cf[NQ];
#pragma unroll
    for (int q = 0; q < NQ; ++q) cf[q] = (R)0;
    const double *fbs[2] = {fb1, fb2};
    const int nbcs[2] = {nbc1, nbc2};
    const double *tws[2] = {tw_c1, tw_c2};
    const double2 scs[2] = {sc1, sc2};
    for (int t = 0; t < 2; ++t) {
      if (!fbs[t]) continue;
      const int nbc = nbcs[t], h = (nbc - 1) / 2;
      R hc[NQ + 1];  // nbc <= 2 HM + 2
      if constexpr (F32) {  // r2hc of the contracted forces in FP32 (gb_r2hc_direct's sums)
        float tmp[NQ + 1];
        for (int j = 0; j < nbc; ++j) tmp[j] = d2f(fbs[t][row + S * j]);
        const double *tw = tws[t];
        for (int k = 0; k <= h; ++k) {
          float re = 0.f, im = 0.f;
          int m = 0;
          for (int j = 0; j < nbc; ++j) {
            re = fmaf(tmp[j], d2f(tw[m]), re);
            im = fmaf(-tmp[j], d2f(tw[nbc + m]), im);
            m += k;
            if (m >= nbc) m -= nbc;
          }
          hc[k] = re;
          if (k > 0) hc[nbc - k] = im;
        }
      } else {
        double tmp[NQ + 1];
        for (int j = 0; j < nbc; ++j) tmp[j] = fbs[t][row + S * j];
        gb_r2hc_direct(tmp, hc, nbc, tws[t]);
      }
      const R s1 = F32 ? (R)d2f(scs[t].x) : (R)scs[t].x, s2 = F32 ? (R)d2f(scs[t].y) : (R)scs[t].y;
      cf[0] += s2 * (s1 * hc[0]);
#pragma unroll
      for (int k = 1; k <= HM; ++k) {
        if (k <= h) {
          cf[2 * k - 1] += s2 * (s1 * hc[k]);
          cf[2 * k] += s2 * (s1 * hc[nbc - k]);
        }
      }
    }
#pragma unroll
    for (int q = 0; q < NQ; ++q) CF[lr * NQ + q] = cf[q];
  }
  // the expansion table, after the coefficients' loads are on their way (one
  // barrier for both); FP32 variant without FP64 instructions
  for (int w = threadIdx.x; w < nb * NQ; w += blockDim.x) {
    const int j = w / NQ, q = w % NQ;
    const int k = (q + 1) / 2, m = (j * k) % nb;
    if constexpr (F32) {
      const float scf = d2f(sc);
      E[w] = q == 0 ? scf : ((q & 1) ? 2.f * scf * d2f(tw_nb[m]) : -2.f * scf * d2f(tw_nb[nb + m]));
    } else {
      E[w] = q == 0 ? sc : ((q & 1) ? 2.0 * sc * tw_nb[m] : -2.0 * sc * tw_nb[nb + m]);
    }
  }
  cp_async_wait_all();  // this thread's momenta are in PS (only it reads them)
  __syncthreads();
  if (row >= S) return;
  R cr[NQ];
#pragma unroll
  for (int q = 0; q < NQ; ++q) cr[q] = CF[lr * NQ + q];
  const bool extras = e1 || e2 || e3;
  bool bad = false;
  for (int j = j0; j < j1; ++j) {
    R s = (R)0;
#pragma unroll
    for (int q = 0; q < NQ; ++q) s += cr[q] * E[j * NQ + q];
    double v;
    if constexpr (F32) v = any ? f2d(s) : 0.0;
    else v = any ? s : 0.0;
    const long long o = row + S * j;
    if (extras) {
      if (e1) v += e1[o];
      if (e2) v += e2[o];
      if (e3) v += e3[o];
    }
    dvdr[o] = v;
    bad |= gb_nonfinite(v);
    if (p) p[o] = (pre ? PS[(j - j0) * XT + threadIdx.x] : p[o]) - halfdt * v;
  }
  gb_flag_nonfinite(status, bad);
}

// intramolecular forces on B configurations (potenl_opt iopt = 4 path)
__global__ void __launch_bounds__(128) k_intra(const double *r, double *out, int nm, int B, int model,
                                               IntraPar ip, double *acc, int accumulate, unsigned *status) {
  __shared__ double sh[32 * 10];
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double vals[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (t < (long long)nm * B) {
    const double *x = r + t * 9;
    double xl[9], f[9], vir[9];
#pragma unroll
    for (int d = 0; d < 9; ++d) xl[d] = x[d];
    vals[0] = intra_molecule(model, xl, f, vir, ip);
    bool bad = gb_nonfinite(vals[0]);
#pragma unroll
    for (int d = 0; d < 9; ++d) {
      vals[1 + d] = vir[d];
      bad |= gb_nonfinite(f[d]);
    }
    gb_flag_nonfinite(status, bad);
    double *o = out + t * 9;
    if (accumulate) {
#pragma unroll
      for (int d = 0; d < 9; ++d) o[d] += f[d];
    } else {
#pragma unroll
      for (int d = 0; d < 9; ++d) o[d] = f[d];
    }
  }
  block_sum_atomic<10>(vals, sh, acc);
}

// virial_ke partial sums (kinetic.f90:1-54) per coordinate row:
// acc[0] += sum (r - rc) dvdr, acc[1] += sum (r - rc) dvdr2, acc[2+xyz], acc[5+xyz]
__global__ void __launch_bounds__(128) k_virial_ke(const double *r, const double *dvdr,
                                                   const double *dvdr2, int na, int nb, double *acc) {
  __shared__ double sh[32 * 8];
  const long long S = 3LL * na;
  const long long row = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  double vals[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (row < S) {
    double rc = 0.0;
    for (int k = 0; k < nb; ++k) rc = rc + r[row + S * k];
    rc = rc / (double)nb;
    double q1 = 0.0, q2 = 0.0;
    for (int k = 0; k < nb; ++k) {
      const double dr = r[row + S * k] - rc;
      q1 += dr * dvdr[row + S * k];
      q2 += dr * dvdr2[row + S * k];
    }
    const int x = (int)(row % 3);
    vals[0] = q1;
    vals[1] = q2;
    vals[2 + x] = q1;
    vals[5 + x] = q2;
  }
  block_sum_atomic<8>(vals, sh, acc);
}

}  // namespace

void launch_realft(cudaStream_t s, const double *in, double *out, int m, int n, int mode,
                   const double *tw) {
  const double scale = sqrt(1.0 / (double)n);
  const unsigned g = nblk(m, 128);
  switch (n) {
    case 1: k_copy<<<nblk(m, 256), 256, 0, s>>>(out, in, m); return;
    case 2: k_realft_pow2<2><<<g, 128, 0, s>>>(in, out, m, mode, tw, scale); return;
    case 4: k_realft_pow2<4><<<g, 128, 0, s>>>(in, out, m, mode, tw, scale); return;
    case 8: k_realft_pow2<8><<<g, 128, 0, s>>>(in, out, m, mode, tw, scale); return;
    case 16: k_realft_pow2<16><<<g, 128, 0, s>>>(in, out, m, mode, tw, scale); return;
    case 32: k_realft_pow2<32><<<g, 128, 0, s>>>(in, out, m, mode, tw, scale); return;
    case 64: k_realft_pow2<64><<<g, 64, 0, s>>>(in, out, m, mode, tw, scale); return;
    default: k_realft_direct<<<nblk(m, 64), 64, 0, s>>>(in, out, m, n, mode, tw, scale); return;
  }
}

void launch_rotate(cudaStream_t s, double *p, double *r, const double *monod, int na, int nb) {
  long long n = 3LL * na * nb;
  k_rotate<<<nblk(n, 256), 256, 0, s>>>(p, r, monod, na, nb);
}

void launch_axpy(cudaStream_t s, double *y, const double *x, double a, long long n) {
  k_axpy<<<nblk(n, 256), 256, 0, s>>>(y, x, a, n);
}

void launch_copy(cudaStream_t s, double *dst, const double *src, long long n) {
  k_copy<<<nblk(n, 256), 256, 0, s>>>(dst, src, n);
}

void launch_ring_contract(cudaStream_t s, const double *rnm, double *rb, int na, int nb, int nbc,
                          const double *tw_c) {
  long long n = 3LL * na;
  // scales 1/sqrt(nbc), sqrt(nbc/nb) (evolve_pi.f90:405-431), from the host
  k_ring_contract<<<nblk(n, 128), 128, 0, s>>>(rnm, rb, na, nb, nbc, tw_c, std::sqrt(1.0 / (double)nbc),
                                               std::sqrt((double)nbc / (double)nb));
}

template <int HM>
void launch_expand_hm(cudaStream_t s, bool mixed, double *dvdr, const double *fb1, int nbc1, const double *tw_c1,
                      const double *fb2, int nbc2, const double *tw_c2, const double *e1, const double *e2,
                      const double *e3, double *p, double halfdt, int na, int nb, const double *tw_nb,
                      unsigned *status) {
  const long long n = 3LL * na;
  const size_t smem = sizeof(double) * ((nb + XR) * (2 * HM + 1) + (nb <= 4 * XPJ ? XT * XPJ : 0));
  auto scale = [&](int nbc) {  // sqrt(1/nbc), sqrt(nb/nbc) of a contraction (force_contract)
    return nbc > 0 ? make_double2(sqrt(1.0 / (double)nbc), sqrt((double)nb / (double)nbc)) : make_double2(0.0, 0.0);
  };
  const double2 sc1 = scale(fb1 ? nbc1 : 0), sc2 = scale(fb2 ? nbc2 : 0);
  const double sc = sqrt(1.0 / (double)nb);
  if (mixed)
    k_expand_table<HM, float><<<nblk(n, XR), XT, smem, s>>>(dvdr, fb1, nbc1, tw_c1, fb2, nbc2, tw_c2, e1, e2, e3, p,
                                                            halfdt, na, nb, tw_nb, sc1, sc2, sc, status);
  else
    k_expand_table<HM, double><<<nblk(n, XR), XT, smem, s>>>(dvdr, fb1, nbc1, tw_c1, fb2, nbc2, tw_c2, e1, e2, e3,
                                                             p, halfdt, na, nb, tw_nb, sc1, sc2, sc, status);
}

void launch_expand_forces(cudaStream_t s, double *dvdr, const double *fb1, int nbc1,
                          const double *tw_c1, const double *fb2, int nbc2, const double *tw_c2,
                          const double *e1, const double *e2, const double *e3, double *p,
                          double halfdt, int na, int nb, const double *tw_nb, bool mixed, unsigned *status) {
  int nbc = 1;
  if (fb1) nbc = max(nbc, nbc1);
  if (fb2) nbc = max(nbc, nbc2);
  const int h = (nbc - 1) / 2;
  // modes beyond nb/2 do not exist; the table form needs HM <= nb/2 and 2HM+1 <= nb
  if (2 * h + 1 <= nb && h <= 4) {
    switch (h) {
      case 0: launch_expand_hm<0>(s, mixed, dvdr, fb1, nbc1, tw_c1, fb2, nbc2, tw_c2, e1, e2, e3, p, halfdt, na, nb, tw_nb, status); return;
      case 1: launch_expand_hm<1>(s, mixed, dvdr, fb1, nbc1, tw_c1, fb2, nbc2, tw_c2, e1, e2, e3, p, halfdt, na, nb, tw_nb, status); return;
      case 2: launch_expand_hm<2>(s, mixed, dvdr, fb1, nbc1, tw_c1, fb2, nbc2, tw_c2, e1, e2, e3, p, halfdt, na, nb, tw_nb, status); return;
      case 3: launch_expand_hm<3>(s, mixed, dvdr, fb1, nbc1, tw_c1, fb2, nbc2, tw_c2, e1, e2, e3, p, halfdt, na, nb, tw_nb, status); return;
      case 4: launch_expand_hm<4>(s, mixed, dvdr, fb1, nbc1, tw_c1, fb2, nbc2, tw_c2, e1, e2, e3, p, halfdt, na, nb, tw_nb, status); return;
    }
  }
  long long n = 3LL * na;
  k_expand_forces<<<nblk(n, 64), 64, 0, s>>>(dvdr, fb1, nbc1, tw_c1, fb2, nbc2, tw_c2, e1, e2, e3, p,
                                             halfdt, na, nb, tw_nb, status);
}

void launch_intra(cudaStream_t s, const double *r, double *out, int na, int B, int model,
                  const gb_params &P, double *acc, int accumulate, unsigned *status) {
  IntraPar ip;
  ip.reoh = P.reoh;
  ip.theta = P.theta;
  ip.rehh = 2.0 * sin(0.5 * P.theta) * P.reoh;
  ip.apot = P.apot;
  ip.bpot = P.bpot;
  ip.alp = P.alp;
  const int nm = na / 3;
  long long n = (long long)nm * B;
  k_intra<<<nblk(n, 128), 128, 0, s>>>(r, out, nm, B, model, ip, acc, accumulate, status);
}

void launch_virial_ke(cudaStream_t s, const double *r, const double *dvdr, const double *dvdr2,
                      int na, int nb, double *acc) {
  long long n = 3LL * na;
  k_virial_ke<<<nblk(n, 128), 128, 0, s>>>(r, dvdr, dvdr2, na, nb, acc);
}
