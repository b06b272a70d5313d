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

GB_D double gb_rsqrt(double x) { return rsqrt(x); }
GB_D float gb_rsqrt(float x) { return rsqrtf(x); }
GB_D double gb_sqrt(double x) { return sqrt(x); }
GB_D float gb_sqrt(float x) { return sqrtf(x); }
GB_D double gb_acos(double x) { return acos(x); }
GB_D float gb_acos(float x) { return acosf(x); }

// T = double: the FP64 path.  T = float: the mixed path, which passes
// positions relative to the oxygen (so that FP32 keeps the bond vectors exact
// to its rounding); model 1's virial sum r . dvdr is then taken about the
// oxygen, which equals the reference's sum because the three forces add to zero.
template <typename T>
GB_D T intra_molecule_t(int model, const T *x, T *f, T *vir, const IntraPar &ipd) {
  const T reoh = (T)ipd.reoh, theta = (T)ipd.theta, rehh = (T)ipd.rehh;
  const T ip_apot = (T)ipd.apot, ip_bpot = (T)ipd.bpot, ip_alp = (T)ipd.alp;
  const T dx1 = x[3] - x[0], dy1 = x[4] - x[1], dz1 = x[5] - x[2];
  const T dx2 = x[6] - x[0], dy2 = x[7] - x[1], dz2 = x[8] - x[2];
  const T dx3 = x[6] - x[3], dy3 = x[7] - x[4], dz3 = x[8] - x[5];
  const T dr1sq = dx1 * dx1 + dy1 * dy1 + dz1 * dz1;
  const T dr2sq = dx2 * dx2 + dy2 * dy2 + dz2 * dz2;
  const T dr3sq = dx3 * dx3 + dy3 * dy3 + dz3 * dz3;
  // one rsqrt per bond instead of a square root and a division
  const T i1 = gb_rsqrt(dr1sq), i2 = gb_rsqrt(dr2sq), i3 = gb_rsqrt(dr3sq);
  const T dr1a = dr1sq * i1, dr2a = dr2sq * i2, dr3a = dr3sq * i3;
  const T dr1 = dr1a - reoh, dr2 = dr2a - reoh;
  T v, dvdr1, dvdr2, dvdr3;
  if (model == 0) {
    const T apot = (T)0.5993, bpot = (T)0.1466, cpot = (T)-0.09435, dpot = (T)0.04984;
    const T dr3 = dr3a - rehh;
    v = (T)0.5 * apot * (dr1 * dr1 + dr2 * dr2) + (T)0.5 * bpot * dr3 * dr3 + cpot * (dr1 + dr2) * dr3 +
        dpot * dr1 * dr2;
    dvdr1 = apot * dr1 + cpot * dr3 + dpot * dr2;
    dvdr2 = apot * dr2 + cpot * dr3 + dpot * dr1;
    dvdr3 = bpot * dr3 + cpot * (dr1 + dr2);
  } else {
    const T u = dr1sq + dr2sq - dr3sq;
    const T vv = (T)2 * dr1a * dr2a;
    const T v2 = (T)1 / (vv * vv);
    const T arg = u / vv;
    const T darg = (T)-1 / gb_sqrt((T)1 - arg * arg);
    const T dang = gb_acos(arg) - theta;
    const T dth1 = darg * (((T)2 * dr1a * vv - (T)2 * dr2a * u) * v2);
    const T dth2 = darg * (((T)2 * dr2a * vv - (T)2 * dr1a * u) * v2);
    const T dth3 = darg * (((T)-2 * dr3a * vv) * v2);
    if (model == 1) {
      v = (T)0.5 * ip_apot * (dr1 * dr1 + dr2 * dr2) + (T)0.5 * ip_bpot * (dang * dang);
      dvdr1 = ip_apot * dr1 + ip_bpot * dang * dth1;
      dvdr2 = ip_apot * dr2 + ip_bpot * dang * dth2;
      dvdr3 = ip_bpot * dang * dth3;
    } else {
      const T de = ip_apot, deb = ip_bpot, alp = ip_alp;
      const T alp2 = alp * alp, alp3 = alp * alp2, alp4 = alp3 * alp;
      const T f1 = (T)(7.0 / 12.0), f2 = (T)(7.0 / 3.0);
      const T drasq = dr1 * dr1, drbsq = dr2 * dr2;
      v = de * (alp2 * drasq - alp3 * dr1 * drasq + f1 * alp4 * drasq * drasq) +
          de * (alp2 * drbsq - alp3 * dr2 * drbsq + f1 * alp4 * drbsq * drbsq) + deb * (dang * dang);
      const T a1 = de * ((T)2 * alp2 * dr1 - (T)3 * alp3 * drasq + f2 * alp4 * dr1 * drasq);
      const T a2 = de * ((T)2 * alp2 * dr2 - (T)3 * alp3 * drbsq + f2 * alp4 * dr2 * drbsq);
      const T a3 = (T)2 * deb * dang;
      dvdr1 = a1 + a3 * dth1;
      dvdr2 = a2 + a3 * dth2;
      dvdr3 = a3 * dth3;
    }
  }
  const T dvdx1 = dvdr1 * dx1 * i1, dvdy1 = dvdr1 * dy1 * i1, dvdz1 = dvdr1 * dz1 * i1;
  const T dvdx2 = dvdr2 * dx2 * i2, dvdy2 = dvdr2 * dy2 * i2, dvdz2 = dvdr2 * dz2 * i2;
  const T dvdx3 = dvdr3 * dx3 * i3, dvdy3 = dvdr3 * dy3 * i3, dvdz3 = dvdr3 * dz3 * i3;
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
    vir[1] = vir[2] = vir[3] = vir[5] = vir[6] = vir[7] = (T)0;
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

GB_D double intra_molecule(int model, const double *x, double *f, double *vir, const IntraPar &ip) {
  return intra_molecule_t<double>(model, x, f, vir, ip);
}
