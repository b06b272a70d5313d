// gb_rng.h -- the reference's serial random stream (random.f90:1-72) with its
// saved state held in an explicit record.
//
// ran2 is L'Ecuyer's combined generator with a 32-entry Bays-Durham shuffle
// (the published "ran2" algorithm the reference transcribes); gaussian is the
// polar Box-Muller method, which keeps its second deviate for the next call.
// The library's gbrpmd_ran2 / gbrpmd_gaussian use one process-wide record, as
// the reference does (one trajectory per process); a batch replica carries its
// own record so that its stream is the one it would draw alone.
#pragma once

#include <cmath>
#include <cstddef>

struct RngState {
  int iv[32] = {0};
  int iy = 0;
  int idum2 = 123456789;
  int iset = 0;
  double gset = 0.0;
};

inline double rng_ran2(RngState &g, int *idum, double rmin, double rmax) {
  const int im1 = 2147483563, im2 = 2147483399, imm1 = im1 - 1;
  const int ia1 = 40014, ia2 = 40692, iq1 = 53668, iq2 = 52774, ir1 = 12211, ir2 = 3791;
  const int ntab = 32, ndiv = 1 + imm1 / ntab;
  const double am = 1.0 / im1, eps = 1.2e-7, rnmx = 1.0 - eps;
  int k, j;
  if (*idum <= 0) {
    *idum = (-*idum) > 1 ? -*idum : 1;
    g.idum2 = *idum;
    for (j = ntab + 8; j >= 1; --j) {
      k = *idum / iq1;
      *idum = ia1 * (*idum - k * iq1) - k * ir1;
      if (*idum < 0) *idum += im1;
      if (j <= ntab) g.iv[j - 1] = *idum;
    }
    g.iy = g.iv[0];
  }
  k = *idum / iq1;
  *idum = ia1 * (*idum - k * iq1) - k * ir1;
  if (*idum < 0) *idum += im1;
  k = g.idum2 / iq2;
  g.idum2 = ia2 * (g.idum2 - k * iq2) - k * ir2;
  if (g.idum2 < 0) g.idum2 += im2;
  j = 1 + g.iy / ndiv;
  g.iy = g.iv[j - 1] - g.idum2;
  g.iv[j - 1] = *idum;
  if (g.iy < 1) g.iy += imm1;
  const double u = am * g.iy;
  return ((rmax - rmin) * (u < rnmx ? u : rnmx)) + rmin;
}

inline double rng_gaussian(RngState &g, int *idum, double sigma) {
  if (g.iset == 0) {
    double v1, v2, rsq;
    do {
      v1 = 2.0 * rng_ran2(g, idum, 0.0, 1.0) - 1.0;
      v2 = 2.0 * rng_ran2(g, idum, 0.0, 1.0) - 1.0;
      rsq = v1 * v1 + v2 * v2;
    } while (rsq >= 1.0 || rsq == 0.0);
    const double fac = std::sqrt(-2.0 * std::log(rsq) / rsq);
    g.gset = v1 * fac;
    g.iset = 1;
    return sigma * v2 * fac;
  }
  g.iset = 0;
  return sigma * g.gset;
}

// sample_rpmd + pshift (module_thermostat.f90:199-264): Maxwell-Boltzmann bead
// momenta at beta / nb in the reference's draw order (bead, atom, xyz), then
// the total momentum removed
inline void rng_sample_rpmd(RngState &g, double *p, int na, int nb, const double *mass, double beta, int *irun) {
  const double betan = beta / (double)nb;
  for (int k = 0; k < nb; ++k)
    for (int j = 0; j < na; ++j)
      for (int l = 0; l < 3; ++l) {
        const double sigma = std::sqrt(mass[j] / betan);
        p[l + 3 * ((size_t)j + (size_t)na * k)] = rng_gaussian(g, irun, sigma);
      }
  double vx = 0.0, vy = 0.0, vz = 0.0, totmass = 0.0;
  for (int j = 0; j < na; ++j) totmass = totmass + mass[j];
  totmass = (double)nb * totmass;
  for (int k = 0; k < nb; ++k)
    for (int j = 0; j < na; ++j) {
      const double *q = p + 3 * ((size_t)j + (size_t)na * k);
      vx = vx + q[0];
      vy = vy + q[1];
      vz = vz + q[2];
    }
  vx = vx / totmass;
  vy = vy / totmass;
  vz = vz / totmass;
  for (int k = 0; k < nb; ++k)
    for (int j = 0; j < na; ++j) {
      double *q = p + 3 * ((size_t)j + (size_t)na * k);
      q[0] = q[0] - mass[j] * vx;
      q[1] = q[1] - mass[j] * vy;
      q[2] = q[2] - mass[j] * vz;
    }
}
