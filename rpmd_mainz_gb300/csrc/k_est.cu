// k_est.cu -- the estimators md_eq prints at output steps, on the resident state.
//
// One thread per molecule (its 3 atoms = 9 coordinate rows), beads looped, so
// that the per-molecule quantities (centroid of the molecule, its dipole) need
// no exchange between threads.  Sums (FP64) per block, then one atomic add per
// block and value:
//   acc[0]     sum_k sum_i |p|^2 / (2 m_i)                  kinetic_rpmd (kinetic.f90:248-265)
//   acc[1]     sum_i m_i sum_k |r_k - r_{k-1}|^2, ring        spring energy / (omega_n^2 / 2)
//                                                             (md_eq.f90:252-270)
//   acc[2..3]  tq1, tq2 = sum (r - r_centroid) . dvdr, dvdr2  virial_ke (kinetic.f90:1-54)
//   acc[4..9]  their x, y, z parts (tq1xyz, tq2xyz)
//   acc[10..12] sum over beads and molecules of the molecular dipole  dipole (md_tools.f90:75-128)
//   acc[13]    sum over beads and molecules of its length
// Per molecule (optional): rcm = center_water (md_tools.f90:367-390), the bead
// average of the SUM of the three atoms' positions (the reference does not
// divide by three), and mdip = the bead-averaged molecular dipole.
#include "gb_common.cuh"
#include "gb_kernels.h"

namespace {

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

constexpr int EST_T = 128;
constexpr int EST_NV = 14;  // sums per thread (acc layout above)

__global__ void __launch_bounds__(EST_T) k_estimators(const double *__restrict__ r, const double *__restrict__ p,
                                                      const double *__restrict__ dvdr,
                                                      const double *__restrict__ dvdr2,
                                                      const double *__restrict__ mass,
                                                      const double *__restrict__ z, int nm, int nb, double alpha,
                                                      double *acc, double *rcm, double *mdip) {
  __shared__ double sh[32 * EST_NV];
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  double v[EST_NV];
#pragma unroll
  for (int i = 0; i < EST_NV; ++i) v[i] = 0.0;
  if (m < nm) {
    const long long S = 9LL * nm;  // one bead: 3 na doubles
    const long long o = 9LL * m;
    double rc[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) rc[c] = 0.0;
    for (int k = 0; k < nb; ++k)
#pragma unroll
      for (int c = 0; c < 9; ++c) rc[c] += r[o + c + S * k];
#pragma unroll
    for (int c = 0; c < 9; ++c) rc[c] = rc[c] / (double)nb;
    double im2[3], ms[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      ms[a] = mass[3 * m + a];
      im2[a] = 1.0 / (2.0 * ms[a]);
    }
    const double zo = z[3 * m], alpha2 = 0.5 * (1.0 - alpha);
    const double fo = alpha * zo, f1 = z[3 * m + 1] + alpha2 * zo, f2 = z[3 * m + 2] + alpha2 * zo;
    double ring[3] = {0, 0, 0}, dsum[3] = {0, 0, 0}, cw[3] = {0, 0, 0};
    double prev[9];
#pragma unroll
    for (int c = 0; c < 9; ++c) prev[c] = r[o + c + S * (nb - 1)];  // bead 1 pairs with bead nb
    for (int k = 0; k < nb; ++k) {
      const long long b = o + S * k;
      double rk[9];
#pragma unroll
      for (int c = 0; c < 9; ++c) rk[c] = r[b + c];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        double pp = 0.0, dd = 0.0;
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          const int c = 3 * a + x;
          const double pc = p[b + c];
          pp += pc * pc;
          const double d = rk[c] - prev[c];
          dd += d * d;
          const double dr = rk[c] - rc[c];
          const double q1 = dr * dvdr[b + c], q2 = dr * dvdr2[b + c];
          v[2] += q1;
          v[3] += q2;
          v[4 + x] += q1;
          v[7 + x] += q2;
        }
        v[0] += im2[a] * pp;
        ring[a] += dd;
      }
      double dl = 0.0;
#pragma unroll
      for (int x = 0; x < 3; ++x) {
        const double d = fo * rk[x] + f1 * rk[3 + x] + f2 * rk[6 + x];
        dsum[x] += d;
        v[10 + x] += d;
        dl += d * d;
        cw[x] += rk[x] + rk[3 + x] + rk[6 + x];
      }
      v[13] += sqrt(dl);
#pragma unroll
      for (int c = 0; c < 9; ++c) prev[c] = rk[c];
    }
    if (nb == 1) ring[0] = ring[1] = ring[2] = 0.0;
    v[1] = ms[0] * ring[0] + ms[1] * ring[1] + ms[2] * ring[2];
    const double wt = 1.0 / (double)nb;
    if (rcm)
#pragma unroll
      for (int x = 0; x < 3; ++x) rcm[3 * m + x] = cw[x] * wt;
    if (mdip)
#pragma unroll
      for (int x = 0; x < 3; ++x) mdip[3 * m + x] = dsum[x] / (double)nb;
  }
  block_sum_atomic<EST_NV>(v, sh, acc);
}

}  // namespace

void launch_estimators(cudaStream_t s, const double *r, const double *p, const double *dvdr, const double *dvdr2,
                       const double *mass, const double *z, int na, int nb, double alpha, double *acc, double *rcm,
                       double *mdip) {
  const int nm = na / 3;
  if (nm <= 0) return;
  k_estimators<<<nblk(nm, EST_T), EST_T, 0, s>>>(r, p, dvdr, dvdr2, mass, z, nm, nb, alpha, acc, rcm, mdip);
}
