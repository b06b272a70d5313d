// k_therm.cu -- the thermostat kicks and the Berendsen box scaling that
// evolve_pi applies inside one step (evolve_pi.f90:72-80, 172-189, 281-290).
//
// Both thermostats act on the momenta in the bead representation, r(3,na,nb)
// order.  The random numbers are the reference's serial gaussian stream, drawn
// on the host in the order the reference draws them and passed in.
#include <algorithm>

#include "gb_common.cuh"
#include "gb_kernels.h"

namespace {

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

// ---- device random stream (gbrpmd_ctx_set_rng_mode, GB_RNG_DEVICE) ----
// Philox4x32-10, the counter-based generator of Salmon, Moraes, Dror and Shaw
// ("Parallel random numbers: as easy as 1, 2, 3", SC 2011): ten rounds of two
// 32 x 32 -> 64-bit multiplies on a 128-bit counter, the 64-bit key bumped by
// the golden-ratio Weyl constants between rounds.  Counter (element, kick);
// one normal deviate per element by the Box-Muller transform of the first two
// 32-bit outputs.  Statistically a stream of independent N(0, 1) numbers, not
// the reference's ran2 / gaussian sequence.
struct U4 {
  unsigned x, y, z, w;
};

GB_D U4 philox(U4 c, unsigned k0, unsigned k1) {
  const unsigned M0 = 0xD2511F53u, M1 = 0xCD9E8D57u, W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const unsigned hi0 = __umulhi(M0, c.x), lo0 = M0 * c.x;
    const unsigned hi1 = __umulhi(M1, c.z), lo1 = M1 * c.z;
    c = U4{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
    k0 += W0;
    k1 += W1;
  }
  return c;
}

GB_D double philox_normal(unsigned long long elem, unsigned long long kick, unsigned long long seed) {
  const U4 o = philox(U4{(unsigned)elem, (unsigned)(elem >> 32), (unsigned)kick, (unsigned)(kick >> 32)},
                      (unsigned)seed, (unsigned)(seed >> 32));
  // u1 in (0, 1], u2 in [0, 1) from 53-bit combinations of the outputs
  const double u1 = ((double)(((unsigned long long)o.x << 21) ^ (o.y >> 11)) + 1.0) * 0x1p-53;
  const double u2 = (double)(((unsigned long long)o.z << 21) ^ (o.w >> 11)) * 0x1p-53;
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

// PRL kick with device normals: kick number *ctr
__global__ void __launch_bounds__(256) k_prl_dev(double *__restrict__ p, const double *__restrict__ mass, long long N,
                                                 int na, double c1, double c2, double betan,
                                                 const unsigned long long *ctr, unsigned long long seed) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int j = (int)((i / 3) % na);
  const double c3 = __dmul_rn(c2, sqrt(mass[j] / betan));
  const double g = philox_normal((unsigned long long)i, *ctr, seed);
  p[i] = __dadd_rn(__dmul_rn(c1, p[i]), __dmul_rn(c3, g));
}

// PRG deviates on the device: aux[1] = sum of n - 1 squared normals (chi-square
// with n - 1 degrees of freedom), aux[2] = one more normal (ranno)
__global__ void __launch_bounds__(256) k_prg_draw(long long n, const unsigned long long *ctr,
                                                  unsigned long long seed, double *aux) {
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n - 1;
       i += (long long)gridDim.x * blockDim.x) {
    const double g = philox_normal((unsigned long long)i, *ctr, seed);
    v[0] += g * g;
  }
  block_sum_atomic<1>(v, sh, aux + 1);
  if (blockIdx.x == 0 && threadIdx.x == 0) aux[2] = philox_normal((unsigned long long)(n - 1), *ctr, seed);
}

__global__ void k_ctr_next(unsigned long long *ctr) { *ctr += 1; }

// parinello_therm_loc (module_thermostat.f90:56-82):
//   p = c1 p + c2 sqrt(m_j / betan) g,  g in the order bead, atom, xyz
// (products and the sum rounded separately, as the reference computes them)
__global__ void __launch_bounds__(256) k_prl(double *__restrict__ p, const double *__restrict__ mass,
                                             const double *__restrict__ g, long long N, int na, double c1,
                                             double c2, double betan) {
  const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  const int j = (int)((i / 3) % na);
  const double c3 = __dmul_rn(c2, sqrt(mass[j] / betan));
  p[i] = __dadd_rn(__dmul_rn(c1, p[i]), __dmul_rn(c3, g[i]));
}

// kinetic energy sum p^2 / (2 m) of parinello_therm (module_thermostat.f90:28-35)
__global__ void __launch_bounds__(256) k_kinetic(const double *__restrict__ p, const double *__restrict__ mass,
                                                 long long N, int na, double *out) {
  __shared__ double sh[32];
  double v[1] = {0.0};
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x) {
    const int j = (int)((i / 3) % na);
    v[0] += p[i] * p[i] / (2.0 * mass[j]);
  }
  block_sum_atomic<1>(v, sh, out);
}

// parinello_therm's rescaling (module_thermostat.f90:37-51); every thread forms
// the same alpha from the device kinetic energy *kt
__global__ void __launch_bounds__(256) k_prg_scale(double *__restrict__ p, long long N, const double *__restrict__ kt,
                                                   double c, double ktav, double ndof, double snfm1, double ranno,
                                                   int dev_draws) {
  if (dev_draws) {  // snfm1 and ranno drawn on the device (k_prg_draw)
    snfm1 = kt[1];
    ranno = kt[2];
  }
  const double ransq = ranno * ranno;
  const double fac = (1.0 - c) * ktav / (ndof * kt[0]);
  const double t1 = __dmul_rn(fac, snfm1 + ransq);  // no contraction into the sum below
  const double t2 = __dmul_rn(2.0 * ranno, sqrt(c * fac));
  double alpha = sqrt(c + t1 + t2);
  const double plusmin = ranno + sqrt(c / fac);
  alpha = plusmin >= 0.0 ? fabs(alpha) : -fabs(alpha);  // Fortran sign(alpha, plusmin)
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long long)gridDim.x * blockDim.x)
    p[i] = alpha * p[i];
}

// beren_baro's molecule shift (module_barostat.f90:111-126; per axis in
// beren_baro_nc, 67-82): every atom of water m on every bead moves by
// rcm_m (scale - 1), scale of the axis, rcm = center_water
// (md_tools.f90:367-390: the bead average of the sum of the three atoms'
// positions).  The shift is the same on every bead, so in the normal-mode
// positions rnm (when given) only the centroid row changes, by sqrt(nb) times it.
__global__ void __launch_bounds__(128) k_baro_shift(double *__restrict__ r, double *__restrict__ rnm, int nm, int nb,
                                                    double3 sm1, double sqnb) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= 3 * nm) return;
  const int m = idx / 3, x = idx % 3;
  const long long S = 9LL * nm;
  const long long o = 9LL * m + x;
  double pc = 0.0;
  for (int k = 0; k < nb; ++k) pc = pc + r[o + S * k] + r[o + 3 + S * k] + r[o + 6 + S * k];
  pc = pc * (1.0 / (double)nb);
  const double d = __dmul_rn(pc, x == 0 ? sm1.x : x == 1 ? sm1.y : sm1.z);
  for (int k = 0; k < nb; ++k)
#pragma unroll
    for (int a = 0; a < 3; ++a) r[o + 3 * a + S * k] = r[o + 3 * a + S * k] + d;
  if (rnm)
#pragma unroll
    for (int a = 0; a < 3; ++a) rnm[o + 3 * a] = rnm[o + 3 * a] + __dmul_rn(sqnb, d);
}

}  // namespace

void launch_prl(cudaStream_t s, double *p, const double *mass, const double *g, int na, int nb, double c1, double c2,
                double betan) {
  const long long N = 3LL * na * nb;
  k_prl<<<nblk(N, 256), 256, 0, s>>>(p, mass, g, N, na, c1, c2, betan);
}

void launch_kinetic(cudaStream_t s, const double *p, const double *mass, int na, int nb, double *out) {
  const long long N = 3LL * na * nb;
  const unsigned grid = std::min<unsigned>(nblk(N, 256), 1024u);
  k_kinetic<<<grid, 256, 0, s>>>(p, mass, N, na, out);
}

void launch_prg_scale(cudaStream_t s, double *p, int na, int nb, const double *kt, double c, double ktav, double ndof,
                      double snfm1, double ranno, int dev_draws) {
  const long long N = 3LL * na * nb;
  const unsigned grid = std::min<unsigned>(nblk(N, 256), 4096u);
  k_prg_scale<<<grid, 256, 0, s>>>(p, N, kt, c, ktav, ndof, snfm1, ranno, dev_draws);
}

void launch_prl_dev(cudaStream_t s, double *p, const double *mass, int na, int nb, double c1, double c2, double betan,
                    const unsigned long long *ctr, unsigned long long seed) {
  const long long N = 3LL * na * nb;
  k_prl_dev<<<nblk(N, 256), 256, 0, s>>>(p, mass, N, na, c1, c2, betan, ctr, seed);
}

void launch_prg_draw(cudaStream_t s, long long ndof, const unsigned long long *ctr, unsigned long long seed,
                     double *aux) {
  const unsigned grid = std::max(1u, std::min<unsigned>(nblk(ndof, 256), 1024u));
  k_prg_draw<<<grid, 256, 0, s>>>(ndof, ctr, seed, aux);
}

void launch_ctr_next(cudaStream_t s, unsigned long long *ctr) { k_ctr_next<<<1, 1, 0, s>>>(ctr); }

void launch_baro_shift(cudaStream_t s, double *r, double *rnm, int na, int nb, const double sm1[3]) {
  const int nm = na / 3;
  k_baro_shift<<<nblk(3LL * nm, 128), 128, 0, s>>>(r, rnm, nm, nb, make_double3(sm1[0], sm1[1], sm1[2]),
                                                   sqrt((double)nb));
}
