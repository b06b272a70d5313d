// gb_intra.cuh -- intramolecular water potentials for one molecule (FP64).
//
// x[0..8] = O, H1, H2 coordinates; f[0..8] receives +grad V; vir[9] (column
// major) and the energy are returned for accumulation.
//  model 0: intra_harmonic   (intra_harmonic.f90:1-98), Toukan-Rahman SPC/F
//           constants hard-coded as in the reference
//  model 1: intra_spcfw      (intra_spcfw.f90:1-125), virial W = sum r . dvdr,
//           diagonal only
//  model 2: intra_morse_harm (intra_morse_harm.f90:1-143)
#pragma once

#include "gb_common.cuh"

struct IntraPar {
  double reoh, theta, rehh, apot, bpot, alp;
};

GB_D double intra_molecule(int model, const double *x, double *f, double *vir, const IntraPar &ip) {
  const double dx1 = x[3] - x[0], dy1 = x[4] - x[1], dz1 = x[5] - x[2];
  const double dx2 = x[6] - x[0], dy2 = x[7] - x[1], dz2 = x[8] - x[2];
  const double dx3 = x[6] - x[3], dy3 = x[7] - x[4], dz3 = x[8] - x[5];
  const double dr1sq = dx1 * dx1 + dy1 * dy1 + dz1 * dz1;
  const double dr2sq = dx2 * dx2 + dy2 * dy2 + dz2 * dz2;
  const double dr3sq = dx3 * dx3 + dy3 * dy3 + dz3 * dz3;
  // one rsqrt per bond instead of a square root and a division
  const double i1 = rsqrt(dr1sq), i2 = rsqrt(dr2sq), i3 = rsqrt(dr3sq);
  const double dr1a = dr1sq * i1, dr2a = dr2sq * i2, dr3a = dr3sq * i3;
  const double dr1 = dr1a - ip.reoh, dr2 = dr2a - ip.reoh;
  double v, dvdr1, dvdr2, dvdr3;
  if (model == 0) {
    const double apot = 0.5993, bpot = 0.1466, cpot = -0.09435, dpot = 0.04984;
    const double dr3 = dr3a - ip.rehh;
    v = 0.5 * apot * (dr1 * dr1 + dr2 * dr2) + 0.5 * bpot * dr3 * dr3 + cpot * (dr1 + dr2) * dr3 +
        dpot * dr1 * dr2;
    dvdr1 = apot * dr1 + cpot * dr3 + dpot * dr2;
    dvdr2 = apot * dr2 + cpot * dr3 + dpot * dr1;
    dvdr3 = bpot * dr3 + cpot * (dr1 + dr2);
  } else {
    const double u = dr1sq + dr2sq - dr3sq;
    const double vv = 2.0 * dr1a * dr2a;
    const double v2 = 1.0 / (vv * vv);
    const double arg = u / vv;
    const double darg = -1.0 / sqrt(1.0 - arg * arg);
    const double dang = acos(arg) - ip.theta;
    const double dth1 = darg * ((2.0 * dr1a * vv - 2.0 * dr2a * u) * v2);
    const double dth2 = darg * ((2.0 * dr2a * vv - 2.0 * dr1a * u) * v2);
    const double dth3 = darg * ((-2.0 * dr3a * vv) * v2);
    if (model == 1) {
      v = 0.5 * ip.apot * (dr1 * dr1 + dr2 * dr2) + 0.5 * ip.bpot * (dang * dang);
      dvdr1 = ip.apot * dr1 + ip.bpot * dang * dth1;
      dvdr2 = ip.apot * dr2 + ip.bpot * dang * dth2;
      dvdr3 = ip.bpot * dang * dth3;
    } else {
      const double de = ip.apot, deb = ip.bpot, alp = ip.alp;
      const double alp2 = alp * alp, alp3 = alp * alp2, alp4 = alp3 * alp;
      const double f1 = 7.0 / 12.0, f2 = 7.0 / 3.0;
      const double drasq = dr1 * dr1, drbsq = dr2 * dr2;
      v = de * (alp2 * drasq - alp3 * dr1 * drasq + f1 * alp4 * drasq * drasq) +
          de * (alp2 * drbsq - alp3 * dr2 * drbsq + f1 * alp4 * drbsq * drbsq) + deb * (dang * dang);
      const double a1 = de * (2.0 * alp2 * dr1 - 3.0 * alp3 * drasq + f2 * alp4 * dr1 * drasq);
      const double a2 = de * (2.0 * alp2 * dr2 - 3.0 * alp3 * drbsq + f2 * alp4 * dr2 * drbsq);
      const double a3 = 2.0 * deb * dang;
      dvdr1 = a1 + a3 * dth1;
      dvdr2 = a2 + a3 * dth2;
      dvdr3 = a3 * dth3;
    }
  }
  const double dvdx1 = dvdr1 * dx1 * i1, dvdy1 = dvdr1 * dy1 * i1, dvdz1 = dvdr1 * dz1 * i1;
  const double dvdx2 = dvdr2 * dx2 * i2, dvdy2 = dvdr2 * dy2 * i2, dvdz2 = dvdr2 * dz2 * i2;
  const double dvdx3 = dvdr3 * dx3 * i3, dvdy3 = dvdr3 * dy3 * i3, dvdz3 = dvdr3 * dz3 * i3;
  f[0] = -dvdx1 - dvdx2;
  f[1] = -dvdy1 - dvdy2;
  f[2] = -dvdz1 - dvdz2;
  f[3] = dvdx1 - dvdx3;
  f[4] = dvdy1 - dvdy3;
  f[5] = dvdz1 - dvdz3;
  f[6] = dvdx2 + dvdx3;
  f[7] = dvdy2 + dvdy3;
  f[8] = dvdz2 + dvdz3;
  if (model == 1) {
    // W = sum_i r_i . dvdr_i, diagonal (intra_spcfw.f90:213-220)
    vir[0] = x[0] * f[0] + x[3] * f[3] + x[6] * f[6];
    vir[4] = x[1] * f[1] + x[4] * f[4] + x[7] * f[7];
    vir[8] = x[2] * f[2] + x[5] * f[5] + x[8] * f[8];
    vir[1] = vir[2] = vir[3] = vir[5] = vir[6] = vir[7] = 0.0;
  } else if (model == 2) {
    // upper triangle mirrored (intra_morse_harm.f90:124-138)
    vir[0] = dx1 * dvdx1 + dx2 * dvdx2 + dx3 * dvdx3;
    vir[3] = vir[1] = dx1 * dvdy1 + dx2 * dvdy2 + dx3 * dvdy3;
    vir[6] = vir[2] = dx1 * dvdz1 + dx2 * dvdz2 + dx3 * dvdz3;
    vir[4] = dy1 * dvdy1 + dy2 * dvdy2 + dy3 * dvdy3;
    vir[7] = vir[5] = dy1 * dvdz1 + dy2 * dvdz2 + dy3 * dvdz3;
    vir[8] = dz1 * dvdz1 + dz2 * dvdz2 + dz3 * dvdz3;
  } else {
    // vir(a,b) = sum over the three bonds of d_a * dvd_b (intra_harmonic.f90:86-94);
    // dvd_b is parallel to d, so vir(a,b) = vir(b,a) up to rounding: six sums
    vir[0] = dx1 * dvdx1 + dx2 * dvdx2 + dx3 * dvdx3;
    vir[3] = vir[1] = dy1 * dvdx1 + dy2 * dvdx2 + dy3 * dvdx3;
    vir[6] = vir[2] = dz1 * dvdx1 + dz2 * dvdx2 + dz3 * dvdx3;
    vir[4] = dy1 * dvdy1 + dy2 * dvdy2 + dy3 * dvdy3;
    vir[7] = vir[5] = dz1 * dvdy1 + dz2 * dvdy2 + dz3 * dvdy3;
    vir[8] = dz1 * dvdz1 + dz2 * dvdz2 + dz3 * dvdz3;
  }
  return v;
}
