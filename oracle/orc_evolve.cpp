// orc_evolve.cpp -- oracle: RPMD integrators, estimators, thermostats, RATTLE.
// TEST INFRASTRUCTURE ONLY (see orc.h).
//
// Restates evolve_pi.f90, kinetic.f90 (virial_ke, kinetic_rpmd),
// module_thermostat.f90 (sample_rpmd, pshift, parinello_therm,
// parinello_therm_loc), module_barostat.f90 (beren_driver, beren_baro,
// beren_baro_nc), md_pressure.f90 (pressure, pres_lj_tail), md_rattle.f90 and
// evolve_rigid.f90 (evolve_rig_pi, bead_forces).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "orc.h"

namespace orc {

namespace {
void zero9(double *v) { for (int i = 0; i < 9; ++i) v[i] = 0.0; }
inline double &X(double *a, int i, int j) { return a[i + 3 * (size_t)j]; }
inline double X(const double *a, int i, int j) { return a[i + 3 * (size_t)j]; }
}  // namespace

// ring_contract (evolve_pi.f90:405-431): keep modes 0, 1..(nb_c-1)/2 and their
// partners, HC2R of length nb_c, scale sqrt(nb_c/nb)
void ring_contract(const double *r, double *r_c, int na, int nb, int nb_c) {
  const size_t S = 3 * (size_t)na;
  std::memcpy(r_c, r, sizeof(double) * S);
  for (int k = 1; k <= (nb_c - 1) / 2; ++k) {
    std::memcpy(r_c + S * k, r + S * k, sizeof(double) * S);
    std::memcpy(r_c + S * (nb_c - k), r + S * (nb - k), sizeof(double) * S);
  }
  realft(r_c, 3 * na, nb_c, -1);
  double scale_f = std::sqrt((double)nb_c / (double)nb);
  for (size_t i = 0; i < S * nb_c; ++i) r_c[i] = scale_f * r_c[i];
}

// force_contract (evolve_pi.f90:377-403): R2HC of length nb_c, scale
// sqrt(nb/nb_c), scatter into the kept normal modes of dvdr
void force_contract(double *dvdr, double *dvdr_c, int na, int nb, int nb_c) {
  const size_t S = 3 * (size_t)na;
  realft(dvdr_c, 3 * na, nb_c, +1);
  double scale_f = std::sqrt((double)nb / (double)nb_c);
  for (size_t i = 0; i < S; ++i) dvdr[i] = scale_f * dvdr_c[i];
  for (int k = 1; k <= (nb_c - 1) / 2; ++k)
    for (size_t i = 0; i < S; ++i) {
      dvdr[i + S * k] = scale_f * dvdr_c[i + S * k];
      dvdr[i + S * (nb - k)] = scale_f * dvdr_c[i + S * (nb_c - k)];
    }
}

// rp_contract_nm (evolve_pi.f90:324-375)
Status rp_contract_nm(const double *r, double &v, double *dvdr, int nb, int na,
                      const double box[3], const double *z, double vir[9], int nbdf, int iopt) {
  if ((nbdf - 1) % 2 != 0) return GB_E_CONTRACT;
  const size_t S = 3 * (size_t)na;
  std::vector<double> rb(S * nbdf, 0.0), dvdrb(S * nbdf, 0.0);
  std::memset(dvdr, 0, sizeof(double) * S * nb);
  zero9(vir);
  ring_contract(r, rb.data(), na, nb, nbdf);
  Status st = forces(rb.data(), v, dvdrb.data(), nbdf, na, box, z, vir, iopt);
  if (st) return st;
  force_contract(dvdr, dvdrb.data(), na, nb, nbdf);
  return GB_OK;
}

// virial_ke (kinetic.f90:1-54): centroid-virial kinetic energy estimator
void virial_ke(const double *r, const double *dvdr, const double *dvdr2, double &tv,
               double tvxyz[3], double &tq1, double &tq2, double beta, int na, int nb) {
  const size_t S = 3 * (size_t)na;
  std::vector<double> rc(S, 0.0);
  tq1 = tq2 = 0.0;
  double tq1xyz[3] = {0, 0, 0}, tq2xyz[3] = {0, 0, 0};
  for (int k = 0; k < nb; ++k)
    for (size_t i = 0; i < S; ++i) rc[i] = rc[i] + r[i + S * k];
  for (size_t i = 0; i < S; ++i) rc[i] = rc[i] / (double)nb;
  for (int k = 0; k < nb; ++k)
    for (int j = 0; j < na; ++j)
      for (int i = 0; i < 3; ++i) {
        size_t o = i + 3 * ((size_t)j + (size_t)na * k);
        double dr = r[o] - rc[i + 3 * (size_t)j];
        double drdvr = dr * dvdr[o];
        double drdvr2 = dr * dvdr2[o];
        tq1 = tq1 + drdvr;
        tq2 = tq2 + drdvr2;
        tq1xyz[i] = tq1xyz[i] + drdvr;
        tq2xyz[i] = tq2xyz[i] + drdvr2;
      }
  const int nc = 3;
  tq1 = 0.5 * tq1 / (double)nb;
  tq2 = 0.5 * tq2 / (double)nb;
  for (int i = 0; i < 3; ++i) {
    tq1xyz[i] = 0.5 * tq1xyz[i] / (double)nb;
    tq2xyz[i] = 0.5 * tq2xyz[i] / (double)nb;
  }
  double tc = 0.5 * (3 * na - nc - P.nctot) / beta;
  tv = tc + tq1 + tq2;
  for (int i = 0; i < 3; ++i) tvxyz[i] = tc / 3 + tq1xyz[i] + tq2xyz[i];
}

// kinetic_rpmd (kinetic.f90:248-265)
void kinetic_rpmd(const double *p, int na, double &tk, const double *mass, int nb) {
  tk = 0.0;
  for (int j = 0; j < nb; ++j)
    for (int i = 0; i < na; ++i) {
      const double *q = p + 3 * ((size_t)i + (size_t)na * j);
      tk = tk + (1.0 / (2.0 * mass[i])) * (q[0] * q[0] + q[1] * q[1] + q[2] * q[2]);
    }
}

// The estimators md_eq writes at an output step, each restated from its routine:
// spring energy md_eq.f90:252-270, temperature md_eq.f90:272, virial_ke
// kinetic.f90:1-54, pressure + pres_lj_tail md_pressure.f90:1-56, dipole
// md_tools.f90:75-128, center_water md_tools.f90:367-390, density md_eq.f90:196-198.
void md_eq_estimators(const double *r, const double *p, const double *dvdr, const double *dvdr2,
                      const double *mass, const double *z, int na, int nb, double beta, double v,
                      const double vir[9], const double box[3], double out[16], double *rcm, double *mdip) {
  const int nm = na / 3;
  const double toK = 3.157733e+5, hbar = 1.0, tokgcm3 = 6.147323129e-3;
  double tk;
  kinetic_rpmd(p, na, tk, mass, nb);
  double vrp = 0.0;
  const double omegan = (double)nb / (beta * hbar);
  if (nb > 0) {
    for (int i = 0; i < na; ++i)
      for (int k = 1; k <= nb; ++k) {
        int k1 = k, k2 = k == 1 ? nb : k - 1;
        const double *a = r + 3 * ((size_t)i + (size_t)na * (k1 - 1));
        const double *b = r + 3 * ((size_t)i + (size_t)na * (k2 - 1));
        double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
        double dist = (dx * dx + dy * dy + dz * dz);
        vrp = vrp + 0.5 * mass[i] * (omegan * omegan) * dist;
      }
  }
  double temp = toK * (2.0 * tk / ((double)(3 * na - P.nctot - 3) * (double)nb)) / (double)nb;
  double tv, tvxyz[3], tq1, tq2;
  virial_ke(r, dvdr, dvdr2, tv, tvxyz, tq1, tq2, beta, na, nb);
  // pressure
  double w = vir[0] + vir[4] + vir[8];
  w = -w / 3.0;
  double vol = box[0] * box[1] * box[2];
  double pres = (2.0 * tv / 3.0 + w) / vol;
  double ptail = 0.0;
  if (P.oo_gam == 0.0) {
    double pi = std::acos(-1.0);
    double rho = (double)nm / vol;
    double prefac = (16.0 * pi * (rho * rho) * P.oo_eps * (P.oo_sig * P.oo_sig * P.oo_sig)) / 3.0;
    ptail = prefac * ((2.0 / 3.0) * std::pow(P.oo_sig / P.rcut, 9) - std::pow(P.oo_sig / P.rcut, 3));
  }
  pres = pres + ptail;
  // dipole
  double alpha2 = 0.5 * (1.0 - P.alpha);
  double dipx = 0.0, dipy = 0.0, dipz = 0.0, dipm = 0.0;
  std::vector<double> md(3 * (size_t)nm, 0.0);
  for (int k = 0; k < nb; ++k)
    for (int j = 0; j < na; j += 3) {
      double fac1 = (z[j + 1] + alpha2 * z[j]);
      double fac2 = (z[j + 2] + alpha2 * z[j]);
      const double *ro = r + 3 * ((size_t)j + (size_t)na * k);
      double d[3];
      for (int x = 0; x < 3; ++x) d[x] = P.alpha * z[j] * ro[x] + fac1 * ro[3 + x] + fac2 * ro[6 + x];
      dipx = dipx + d[0];
      dipy = dipy + d[1];
      dipz = dipz + d[2];
      for (int x = 0; x < 3; ++x) md[3 * (size_t)(j / 3) + x] += d[x];
      dipm = dipm + std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    }
  dipm = dipm / (double)(nb * nm);
  dipx = dipx / (double)nb;
  dipy = dipy / (double)nb;
  dipz = dipz / (double)nb;
  if (mdip)
    for (size_t i = 0; i < md.size(); ++i) mdip[i] = md[i] / nb;
  // center_water: p(9, nm, nb) view of r
  if (rcm) {
    double wt = 1.0 / (double)nb;
    for (int j = 0; j < nm; ++j) {
      double pc[3] = {0, 0, 0};
      for (int k = 0; k < nb; ++k) {
        const double *q = r + 9 * ((size_t)j) + 3 * (size_t)na * k;
        for (int x = 0; x < 3; ++x) pc[x] = pc[x] + q[x] + q[3 + x] + q[6 + x];
      }
      for (int x = 0; x < 3; ++x) rcm[3 * (size_t)j + x] = pc[x] * wt;
    }
  }
  double wmass = mass[0] + mass[1] + mass[2];
  out[0] = tk;
  out[1] = vrp;
  out[2] = nb * v + tk + vrp;
  out[3] = temp;
  out[4] = tv;
  for (int x = 0; x < 3; ++x) out[5 + x] = tvxyz[x];
  out[8] = pres;
  out[9] = dipx;
  out[10] = dipy;
  out[11] = dipz;
  out[12] = dipx * dipx + dipy * dipy + dipz * dipz;
  out[13] = dipm;
  out[14] = tokgcm3 * (wmass * (double)nm / vol);
  out[15] = v;
}

// pshift (module_thermostat.f90:229-264)
void pshift(double *p, const double *mass, int na, int nb) {
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

// sample_rpmd (module_thermostat.f90:199-226): bead k outer, atom j, xyz l inner
void sample_rpmd(double *p, int na, int nb, const double *mass, double beta, Rng &g,
                 int &irun) {
  double betan = beta / (double)nb;
  for (int k = 0; k < nb; ++k)
    for (int j = 0; j < na; ++j)
      for (int l = 0; l < 3; ++l) {
        double sigma = std::sqrt(mass[j] / betan);
        p[l + 3 * ((size_t)j + (size_t)na * k)] = gaussian(g, irun, sigma);
      }
  pshift(p, mass, na, nb);
}

// parinello_therm (module_thermostat.f90:6-54): global stochastic velocity rescaling
void parinello_therm(double *p, const double *mass, double tau, int na, int nb, double dt,
                     Rng &g, int &irun, double beta) {
  double betan = beta / (double)nb;
  int ndof = (int)(3 * na * (double)nb - P.nctot - 3);
  double rt = gaussian(g, irun, 1.0);
  (void)rt;
  double ktav = (double)ndof / (2.0 * betan);
  double snfm1 = 0.0;
  for (int i = 1; i <= ndof - 1; ++i) {
    double ranno = gaussian(g, irun, 1.0);
    snfm1 = snfm1 + ranno * ranno;
  }
  double kt = 0.0;
  for (int k = 0; k < nb; ++k)
    for (int j = 0; j < na; ++j)
      for (int i = 0; i < 3; ++i) {
        double q = p[i + 3 * ((size_t)j + (size_t)na * k)];
        kt = kt + q * q / (2.0 * mass[j]);
      }
  double ranno = gaussian(g, irun, 1.0);
  double ransq = ranno * ranno;
  double c = std::exp(-dt / tau);
  double fac = (1.0 - c) * ktav / ((double)ndof * kt);
  double t1 = fac * (snfm1 + ransq);
  double t2 = 2 * ranno * std::sqrt(c * fac);
  double alpha = c + t1 + t2;
  alpha = std::sqrt(alpha);
  double plusmin = ranno + std::sqrt(c / fac);
  alpha = plusmin >= 0.0 ? std::fabs(alpha) : -std::fabs(alpha);
  for (size_t i = 0; i < 3 * (size_t)na * nb; ++i) p[i] = alpha * p[i];
}

// parinello_therm_loc (module_thermostat.f90:56-82): local Langevin kick
void parinello_therm_loc(double *p, const double *mass, double tau, int na, int nb, double dt,
                         Rng &g, int &irun, double beta) {
  double gamma = 1.0 / (2.0 * tau);
  double betan = beta / (double)nb;
  double c1 = std::exp(-0.5 * gamma * dt);
  double c2 = std::sqrt(1.0 - c1 * c1);
  for (int k = 0; k < nb; ++k)
    for (int j = 0; j < na; ++j) {
      double c3 = c2 * std::sqrt(mass[j] / betan);
      for (int i = 0; i < 3; ++i) {
        double &q = p[i + 3 * ((size_t)j + (size_t)na * k)];
        q = c1 * q + c3 * gaussian(g, irun, 1.0);
      }
    }
}

// pres_lj_tail (md_pressure.f90:37-56): LJ tail correction to the pressure
double pres_lj_tail(const double box[3], int na) {
  int nm = na / 3;
  double pi = std::acos(-1.0);
  double vol = box[0] * box[1] * box[2];
  double rho = (double)nm / vol;
  double prefac = (16.0 * pi * (rho * rho) * P.oo_eps * (P.oo_sig * P.oo_sig * P.oo_sig)) / 3.0;
  return prefac * ((2.0 / 3.0) * std::pow(P.oo_sig / P.rcut, 9) - std::pow(P.oo_sig / P.rcut, 3));
}

// pressure (md_pressure.f90:1-30) with pres_lj_tail
double pressure(const double vir[9], double tv, int na, const double box[3]) {
  double w = vir[0] + vir[4] + vir[8];
  w = -w / 3.0;
  double vol = box[0] * box[1] * box[2];
  double pres = (2.0 * tv / 3.0 + w) / vol;
  double ptail = 0.0;
  if (P.oo_gam == 0.0) ptail = pres_lj_tail(box, na);
  return pres + ptail;
}

// beren_baro (module_barostat.f90:88-129): isotropic Berendsen scaling of the
// box and of each water's center_water vector (md_tools.f90:367-390)
void beren_baro(const double vir[9], double tv, double dt, double *r, double box[3], int na, int nb) {
  double pres = pressure(vir, tv, na, box);
  int nm = na / 3;
  double compi = 13531.0;
  double bstat = compi / (3.0 * P.taub);
  double scale = std::fabs(1.0 - (dt * bstat) * (P.patm - pres));
  for (int d = 0; d < 3; ++d) box[d] = scale * box[d];
  std::vector<double> rcm(3 * (size_t)nm, 0.0);
  double wt = 1.0 / (double)nb;
  for (int j = 0; j < nm; ++j) {
    double pc[3] = {0, 0, 0};
    for (int k = 0; k < nb; ++k) {
      const double *q = r + 9 * (size_t)j + 3 * (size_t)na * k;
      for (int x = 0; x < 3; ++x) pc[x] = pc[x] + q[x] + q[3 + x] + q[6 + x];
    }
    for (int x = 0; x < 3; ++x) rcm[3 * (size_t)j + x] = pc[x] * wt;
  }
  for (int i = 0; i < nm; ++i)
    for (int k = 0; k < nb; ++k)
      for (int a = 0; a < 3; ++a) {
        double *q = r + 3 * ((size_t)(3 * i + a) + (size_t)na * k);
        for (int x = 0; x < 3; ++x) q[x] = q[x] + rcm[3 * (size_t)i + x] * (scale - 1.0);
      }
}

// beren_baro_nc (module_barostat.f90:28-86): each box axis scaled by the
// pressure along it, (-vir(j,j) + 2 tvxyz(j)) / vol plus the LJ tail (the
// reference skips the tail for oo_gam != 0 and for RPMDDFT runs, which this
// path does not have), and each water's center_water vector per axis
void beren_baro_nc(const double vir[9], const double tvxyz[3], double dt, double *r, double box[3], int na, int nb) {
  double ptail = 0.0;
  if (P.oo_gam == 0.0) ptail = pres_lj_tail(box, na);
  double vol = box[0] * box[1] * box[2];
  double pres[3];
  for (int j = 0; j < 3; ++j) {
    pres[j] = (-vir[4 * j] + 2.0 * tvxyz[j]) / vol;
    pres[j] = pres[j] + ptail;
  }
  int nm = na / 3;
  double compi = 13531.0;
  double bstat = compi / (3.0 * P.taub);
  double scale[3];
  for (int j = 0; j < 3; ++j) scale[j] = std::fabs(1.0 - (dt * bstat) * (P.patm - pres[j]));
  for (int j = 0; j < 3; ++j) box[j] = scale[j] * box[j];
  std::vector<double> rcm(3 * (size_t)nm, 0.0);
  double wt = 1.0 / (double)nb;
  for (int i = 0; i < nm; ++i) {
    double pc[3] = {0, 0, 0};
    for (int k = 0; k < nb; ++k) {
      const double *q = r + 9 * (size_t)i + 3 * (size_t)na * k;
      for (int x = 0; x < 3; ++x) pc[x] = pc[x] + q[x] + q[3 + x] + q[6 + x];
    }
    for (int x = 0; x < 3; ++x) rcm[3 * (size_t)i + x] = pc[x] * wt;
  }
  for (int i = 0; i < nm; ++i)
    for (int k = 0; k < nb; ++k)
      for (int a = 0; a < 3; ++a) {
        double *q = r + 3 * ((size_t)(3 * i + a) + (size_t)na * k);
        for (int j = 0; j < 3; ++j) q[j] = q[j] + rcm[3 * (size_t)i + j] * (scale[j] - 1.0);
      }
}

// beren_driver (module_barostat.f90:8-26)
void beren_driver(const double vir[9], double tv, const double tvxyz[3], double dt, double *r, double box[3], int na,
                  int nb) {
  if (P.iamcub) beren_baro(vir, tv, dt, r, box, na, nb);
  else beren_baro_nc(vir, tvxyz, dt, r, box, na, nb);
}

// evolve_pi (evolve_pi.f90:1-322), type = 'RPMD'
Status evolve_pi(double *p, double *r, double &v, double &vew, double &vlj, double &vint,
                 double *dvdr, double *dvdr2, double dt, const double *mass, int na, int nb,
                 double box[3], const double *z, double beta, double vir[9], double vir_lf[9],
                 Rng &g, int &irun, int nbaro, double *tv_out) {
  const size_t S = 3 * (size_t)na, N = S * nb;
  std::vector<double> dvdre(N, 0.0), rst(N), dvdrl(N, 0.0);
  std::vector<double> monod(3 * 4 * (size_t)nb, 0.0);
  double vir_itr[9], vir_lj[9], vir_ew[9], vir_hf[9], vir_ewc[9];
  zero9(vir_itr); zero9(vir_lj); zero9(vir_ew); zero9(vir_hf);
  vew = vlj = vint = 0.0;
  double tv = 0.0, tvxyz[3] = {0, 0, 0};
  double ve = 0.0;
  const int mts = P.mts;
  double dtsmall = dt / (double)mts;
  double halfdtsmall = 0.5 * dtsmall;
  double halfdt = 0.5 * dt;
  Status st;

  ring_rpmd(mass, monod.data(), na, nb, dtsmall, beta);

  if (P.therm == GB_THERM_PRG) parinello_therm(p, mass, P.ttau, na, nb, halfdt, g, irun, beta);
  else if (P.therm == GB_THERM_PRL) parinello_therm_loc(p, mass, P.ttau, na, nb, dt, g, irun, beta);
  for (size_t i = 0; i < N; ++i) p[i] = p[i] - halfdt * dvdr[i];
  for (size_t i = 0; i < N; ++i) p[i] = p[i] - halfdtsmall * dvdr2[i];

  realft(p, 3 * na, nb, +1);
  realft(r, 3 * na, nb, +1);

  for (int im = 1; im <= mts; ++im) {
    for (int k = 0; k < nb; ++k)
      for (int j = 0; j < na; ++j) {
        int ic = (j + 1) % 3;
        if (ic == 0) ic = 3;
        const double *m = &monod[(ic - 1) + 3 * 4 * (size_t)k];  // monod(ic,c,k) -> m[3*c]
        for (int i = 0; i < 3; ++i) {
          size_t o = i + 3 * ((size_t)j + (size_t)na * k);
          double pprime = p[o] * m[0] + r[o] * m[3];
          r[o] = p[o] * m[6] + r[o] * m[9];
          p[o] = pprime;
        }
      }
    std::memcpy(rst.data(), r, sizeof(double) * N);
    realft(rst.data(), 3 * na, nb, -1);
    st = forces(rst.data(), vint, dvdr2, nb, na, box, z, vir_itr, 4);
    if (st) return st;
    double tv_itr, tvxyz_itr[3], tq1, tq2;
    virial_ke(rst.data(), dvdr, dvdr2, tv_itr, tvxyz_itr, tq1, tq2, beta, na, nb);
    for (int i = 0; i < 9; ++i) vir_hf[i] += vir_itr[i];
    tv = tv + tv_itr;
    for (int i = 0; i < 3; ++i) tvxyz[i] += tvxyz_itr[i];
    if (im != mts) {
      realft(dvdr2, 3 * na, nb, +1);
      for (size_t i = 0; i < N; ++i) p[i] = p[i] - dtsmall * dvdr2[i];
    }
  }
  tv = tv / (double)mts;
  for (int i = 0; i < 3; ++i) tvxyz[i] = tvxyz[i] / (double)mts;
  for (int i = 0; i < 9; ++i) vir_hf[i] = vir_hf[i] / (double)mts;
  for (int i = 0; i < 9; ++i) vir[i] = vir_lf[i] + vir_hf[i];
  if (tv_out) *tv_out = tv;

  if (nbaro == 1) {  // evolve_pi.f90:176-189: beren_driver on the bead positions rst
    if (P.baro != GB_BARO_BER) return GB_E_UNSUPPORTED;  // mc_baro
    beren_driver(vir, tv, tvxyz, dt, rst.data(), box, na, nb);
    std::memcpy(r, rst.data(), sizeof(double) * N);
    realft(r, 3 * na, nb, +1);
  }

  const int nbdf1 = P.nbdf1, nbdf2 = P.nbdf2;
  if (nbdf1 > 0) {
    st = rp_contract_nm(r, vew, dvdr, nb, na, box, z, vir_ew, nbdf1, 2);
    if (st) return st;
    if (P.sig > 0.0) {
      st = rp_contract_nm(r, ve, dvdre.data(), nb, na, box, z, vir_ewc, nbdf1, 5);
      if (st) return st;
      vew = vew - ve;
      for (int i = 0; i < 9; ++i) vir_ew[i] -= vir_ewc[i];
      for (size_t i = 0; i < N; ++i) dvdr[i] -= dvdre[i];
    }
  }
  if (nbdf2 > 0) {
    st = rp_contract_nm(r, vlj, dvdrl.data(), nb, na, box, z, vir_lj, nbdf2, 3);
    if (st) return st;
  }
  realft(p, 3 * na, nb, -1);
  std::memcpy(r, rst.data(), sizeof(double) * N);
  for (size_t i = 0; i < N; ++i) p[i] = p[i] - halfdtsmall * dvdr2[i];

  if (nbdf1 > 0 && nbdf2 > 0) {
    for (size_t i = 0; i < N; ++i) dvdr[i] += dvdrl[i];
    realft(dvdr, 3 * na, nb, -1);
  } else if (nbdf1 > 0) {
    realft(dvdr, 3 * na, nb, -1);
  } else if (nbdf2 > 0) {
    realft(dvdrl.data(), 3 * na, nb, -1);
  }
  if (nbdf1 <= 0) {
    st = forces(r, vew, dvdr, nb, na, box, z, vir_ew, 2);
    if (st) return st;
  } else if (P.sig > 0.0) {
    st = forces(r, ve, dvdre.data(), nb, na, box, z, vir_ewc, 5);
    if (st) return st;
    vew = vew + ve;
    for (int i = 0; i < 9; ++i) vir_ew[i] += vir_ewc[i];
    for (size_t i = 0; i < N; ++i) dvdr[i] += dvdre[i];
  }
  if (nbdf2 <= 0) {
    st = forces(r, vlj, dvdrl.data(), nb, na, box, z, vir_lj, 3);
    if (st) return st;
  }
  if (nbdf1 <= 0 || nbdf2 <= 0)
    for (size_t i = 0; i < N; ++i) dvdr[i] += dvdrl[i];
  for (size_t i = 0; i < N; ++i) p[i] = p[i] - halfdt * dvdr[i];
  if (P.therm == GB_THERM_PRG) parinello_therm(p, mass, P.ttau, na, nb, halfdt, g, irun, beta);
  else if (P.therm == GB_THERM_PRL) parinello_therm_loc(p, mass, P.ttau, na, nb, dt, g, irun, beta);
  v = vew + vlj + vint;
  for (int i = 0; i < 9; ++i) {
    vir_lf[i] = vir_lj[i] + vir_ew[i];
    vir[i] = vir_lf[i] + vir_hf[i];
  }
  return GB_OK;
}

// ===========================================================================
// RATTLE (md_rattle.f90)
// ===========================================================================
void rattle_setup(Rattle &rt, int nm) {
  rattle_free(rt);
  rt.nm = nm;
  rt.rcb = new double[3 * (size_t)nm];
  rt.bond = new int[6 * (size_t)nm];
  double rehh = 2.0 * std::sin(0.5 * P.theta) * P.reoh;
  int nctot = 0;
  const int nbond = 3;
  for (int i = 1; i <= nm; ++i) {
    rt.rcb[nctot + 0] = P.reoh * P.reoh;
    rt.bond[2 * (nctot + 0)] = 3 * i - 2; rt.bond[2 * (nctot + 0) + 1] = 3 * i - 1;
    rt.rcb[nctot + 1] = P.reoh * P.reoh;
    rt.bond[2 * (nctot + 1)] = 3 * i - 2; rt.bond[2 * (nctot + 1) + 1] = 3 * i;
    rt.rcb[nctot + 2] = rehh * rehh;
    rt.bond[2 * (nctot + 2)] = 3 * i - 1; rt.bond[2 * (nctot + 2) + 1] = 3 * i;
    nctot = nctot + nbond;
  }
  P.nctot = nctot;
  P.nbond = nbond;
}

void rattle_free(Rattle &rt) {
  delete[] rt.rcb;
  delete[] rt.bond;
  rt.rcb = nullptr;
  rt.bond = nullptr;
  rt.nm = 0;
}

// rattle_s1 (md_rattle.f90:33-162), including the running vir(1,3) = vir(1,2) - ...
Status rattle_s1(const Rattle &rt, double *r, const double *rold, double *p, int nm,
                 const double *mass, double dt, double *dvdr, double vir[9], int na) {
  (void)na;
  zero9(vir);
  const double tol = 1e-6;
  const int itmax = 1000;
  int it = 0, nbtot = 0;
  const int nbond = P.nbond;
  auto V = [&](int a, int b) -> double & { return vir[a + 3 * b]; };
  for (int ik = 1; ik <= nm; ++ik) {
    bool done = false;
    it = 0;
    while (!done && it < itmax) {
      done = true;
      for (int i = 1; i <= nbond; ++i) {
        int b = i + nbtot - 1;
        int ii = rt.bond[2 * b] - 1, jj = rt.bond[2 * b + 1] - 1;
        double dx1 = X(r, 0, jj) - X(r, 0, ii), dy1 = X(r, 1, jj) - X(r, 1, ii),
               dz1 = X(r, 2, jj) - X(r, 2, ii);
        double d2 = dx1 * dx1 + dy1 * dy1 + dz1 * dz1;
        double diff = rt.rcb[b] - d2;
        if (std::fabs(diff) > rt.rcb[b] * tol) {
          double rm1 = 1.0 / mass[jj], rm2 = 1.0 / mass[ii];
          double dx2 = X(rold, 0, jj) - X(rold, 0, ii), dy2 = X(rold, 1, jj) - X(rold, 1, ii),
                 dz2 = X(rold, 2, jj) - X(rold, 2, ii);
          double dot = dx1 * dx2 + dy1 * dy2 + dz1 * dz2;
          double gamma = diff / (2.0 * (rm1 + rm2) * dot);
          double gdx = gamma * dx2, gdy = gamma * dy2, gdz = gamma * dz2;
          X(r, 0, jj) += rm1 * gdx; X(r, 1, jj) += rm1 * gdy; X(r, 2, jj) += rm1 * gdz;
          X(r, 0, ii) -= rm2 * gdx; X(r, 1, ii) -= rm2 * gdy; X(r, 2, ii) -= rm2 * gdz;
          gdx = gdx / dt; gdy = gdy / dt; gdz = gdz / dt;
          X(p, 0, jj) += gdx; X(p, 1, jj) += gdy; X(p, 2, jj) += gdz;
          X(p, 0, ii) -= gdx; X(p, 1, ii) -= gdy; X(p, 2, ii) -= gdz;
          gdx = 2.0 * gdx; gdy = 2.0 * gdy; gdz = 2.0 * gdz;
          V(0, 0) = V(0, 0) - gdx * dx2;
          V(0, 1) = V(0, 1) - gdx * dy2;
          V(0, 2) = V(0, 1) - gdx * dz2;
          V(1, 2) = V(1, 2) - gdy * dz2;
          V(1, 1) = V(1, 1) - gdy * dy2;
          V(2, 2) = V(2, 2) - gdz * dz2;
          X(dvdr, 0, jj) += gdx; X(dvdr, 1, jj) += gdy; X(dvdr, 2, jj) += gdz;
          X(dvdr, 0, ii) -= gdx; X(dvdr, 1, ii) -= gdy; X(dvdr, 2, ii) -= gdz;
          done = false;
        }
      }
      it = it + 1;
    }
    nbtot = nbtot + nbond;
  }
  if (it >= itmax) return GB_E_RATTLE1;
  if (P.nctot != nbtot) return GB_E_ARG;
  V(1, 0) = V(0, 1);
  V(2, 0) = V(0, 2);
  V(2, 1) = V(1, 2);
  return GB_OK;
}

// rattle_s2 (md_rattle.f90:164-271)
Status rattle_s2(const Rattle &rt, double *r, double *p, int nm, const double *mass, double dt,
                 double *dvdr, double vir[9], int na) {
  (void)na;
  zero9(vir);
  const double tol = 1e-6;
  const int itmax = 1000;
  int it = 0, nbtot = 0;
  const int nbond = P.nbond;
  double halfdt = 0.5 * dt;
  auto V = [&](int a, int b) -> double & { return vir[a + 3 * b]; };
  for (int ik = 1; ik <= nm; ++ik) {
    bool done = false;
    it = 0;
    while (!done && it <= itmax) {
      done = true;
      for (int i = 1; i <= nbond; ++i) {
        int b = i + nbtot - 1;
        int ii = rt.bond[2 * b] - 1, jj = rt.bond[2 * b + 1] - 1;
        double dx1 = X(r, 0, jj) - X(r, 0, ii), dy1 = X(r, 1, jj) - X(r, 1, ii),
               dz1 = X(r, 2, jj) - X(r, 2, ii);
        double rm1 = 1.0 / mass[jj], rm2 = 1.0 / mass[ii];
        double dvx1 = X(p, 0, jj) * rm1 - X(p, 0, ii) * rm2;
        double dvy1 = X(p, 1, jj) * rm1 - X(p, 1, ii) * rm2;
        double dvz1 = X(p, 2, jj) * rm1 - X(p, 2, ii) * rm2;
        double dot = dx1 * dvx1 + dy1 * dvy1 + dz1 * dvz1;
        double gamma = -dot / ((rm1 + rm2) * rt.rcb[b]);
        if (std::fabs(gamma) > tol) {
          double gdx = gamma * dx1, gdy = gamma * dy1, gdz = gamma * dz1;
          X(p, 0, jj) += gdx; X(p, 1, jj) += gdy; X(p, 2, jj) += gdz;
          X(p, 0, ii) -= gdx; X(p, 1, ii) -= gdy; X(p, 2, ii) -= gdz;
          gdx = gdx / halfdt; gdy = gdy / halfdt; gdz = gdz / halfdt;
          V(0, 0) = V(0, 0) - gdx * dx1;
          V(0, 1) = V(0, 1) - gdx * dy1;
          V(0, 2) = V(0, 1) - gdx * dz1;
          V(1, 2) = V(1, 2) - gdy * dz1;
          V(1, 1) = V(1, 1) - gdy * dy1;
          V(2, 2) = V(2, 2) - gdz * dz1;
          X(dvdr, 0, jj) += gdx; X(dvdr, 1, jj) += gdy; X(dvdr, 2, jj) += gdz;
          X(dvdr, 0, ii) -= gdx; X(dvdr, 1, ii) -= gdy; X(dvdr, 2, ii) -= gdz;
          done = false;
        }
      }
      it = it + 1;
    }
    nbtot = nbtot + nbond;
  }
  if (it >= itmax) return GB_E_RATTLE2;
  if (P.nctot != nbtot) return GB_E_ARG;
  V(1, 0) = V(0, 1);
  V(2, 0) = V(0, 2);
  V(2, 1) = V(1, 2);
  return GB_OK;
}

// bead_forces (evolve_rigid.f90:226-278): primitive ring-polymer springs
void bead_forces(const double *r, int na, int nb, double *dvdrb, double beta,
                 const double *mass) {
  const double hbar = 1.0;
  double omegan = nb / (beta * hbar);
  omegan = omegan * omegan;
  std::memset(dvdrb, 0, sizeof(double) * 3 * (size_t)na * nb);
  if (nb > 1) {
    for (int i = 0; i < na; ++i)
      for (int k = 1; k <= nb; ++k) {
        int k1, k2, k3;
        if (k == 1) { k1 = k; k2 = nb; k3 = 2; }
        else if (k == nb) { k1 = k; k2 = k - 1; k3 = 1; }
        else { k1 = k; k2 = k - 1; k3 = k + 1; }
        for (int c = 0; c < 3; ++c) {
          double dx1 = r[c + 3 * ((size_t)i + (size_t)na * (k1 - 1))];
          double dx2 = r[c + 3 * ((size_t)i + (size_t)na * (k2 - 1))];
          double dx3 = r[c + 3 * ((size_t)i + (size_t)na * (k3 - 1))];
          dvdrb[c + 3 * ((size_t)i + (size_t)na * (k - 1))] = mass[i] * omegan * (2.0 * dx1 - dx2 - dx3);
        }
      }
  }
}

// evolve_rig_pi (evolve_rigid.f90:100-224); with nbaro = 1 the Berendsen
// barostat on the bead positions, its kinetic term from virial_ke with the
// zeroed dvdr2 (evolve_rigid.f90:203-213)
Status evolve_rig_pi(const Rattle &rt, double *p, double *r, double &v, double &v_lf,
                     double &v_hf, double *dvdr, double *dvdr2, double dt, const double *mass,
                     int na, int nb, double box[3], const double *z, double beta,
                     double vir[9], double vir_lf[9], Rng &g, int &irun, int nbaro) {
  const size_t S = 3 * (size_t)na, N = S * nb;
  std::vector<double> rold(S);
  double vir_hf[9], vir_tmp[9];
  zero9(vir_hf);
  double halfdt = 0.5 * dt;
  int nstep = nb;
  double smalldt = dt / (double)nstep;
  double halfsmalldt = 0.5 * smalldt;
  int nm = na / 3;
  Status st;
  if (P.therm == GB_THERM_PRG) parinello_therm(p, mass, P.ttau, na, nb, halfdt, g, irun, beta);
  else if (P.therm == GB_THERM_PRL) parinello_therm_loc(p, mass, P.ttau, na, nb, halfdt, g, irun, beta);
  for (size_t i = 0; i < N; ++i) p[i] = p[i] - halfdt * dvdr[i];
  bead_forces(r, na, nb, dvdr2, beta, mass);
  for (int is = 1; is <= nstep; ++is) {
    for (int k = 0; k < nb; ++k) {
      double *rk = r + S * k, *pk = p + S * k, *fk = dvdr2 + S * k;
      for (int j = 0; j < na; ++j)
        for (int i = 0; i < 3; ++i) {
          rold[i + 3 * j] = X(rk, i, j);
          X(pk, i, j) = X(pk, i, j) - halfsmalldt * X(fk, i, j);
          X(rk, i, j) = X(rk, i, j) + X(pk, i, j) * smalldt / mass[j];
        }
      st = rattle_s1(rt, rk, rold.data(), pk, nm, mass, smalldt, fk, vir_hf, na);
      if (st) return st;
    }
    bead_forces(r, na, nb, dvdr2, beta, mass);
    for (size_t i = 0; i < N; ++i) p[i] = p[i] - halfsmalldt * dvdr2[i];
    for (int k = 0; k < nb; ++k) {
      st = rattle_s2(rt, r + S * k, p + S * k, nm, mass, smalldt, dvdr2 + S * k, vir_hf, na);
      if (st) return st;
    }
  }
  st = forces(r, v, dvdr, nb, na, box, z, vir_lf, 1);
  if (st) return st;
  for (size_t i = 0; i < N; ++i) p[i] = p[i] - halfdt * dvdr[i];
  zero9(vir_hf);
  for (int k = 0; k < nb; ++k) {
    st = rattle_s2(rt, r + S * k, p + S * k, nm, mass, dt, dvdr + S * k, vir_tmp, na);
    if (st) return st;
    for (int i = 0; i < 9; ++i) vir_hf[i] += vir_tmp[i];
  }
  if (P.therm == GB_THERM_PRG) parinello_therm(p, mass, P.ttau, na, nb, halfdt, g, irun, beta);
  else if (P.therm == GB_THERM_PRL) parinello_therm_loc(p, mass, P.ttau, na, nb, halfdt, g, irun, beta);
  for (int i = 0; i < 9; ++i) vir_hf[i] = vir_hf[i] / (double)nb;
  for (int i = 0; i < 9; ++i) vir[i] = vir_lf[i] + vir_hf[i] + vir[i];
  std::memset(dvdr2, 0, sizeof(double) * N);
  if (nbaro == 1) {
    if (P.baro != GB_BARO_BER) return GB_E_UNSUPPORTED;  // mc_baro
    double tv, tvxyz[3], tq1, tq2;
    virial_ke(r, dvdr, dvdr2, tv, tvxyz, tq1, tq2, beta, na, nb);
    beren_driver(vir, tv, tvxyz, dt, r, box, na, nb);
  }
  v_lf = v;
  v_hf = 0.0;
  return GB_OK;
}

// ring-polymer spring energy as md_eq computes it (md_eq.f90:119-136, 252-270)
static double spring_energy(const double *r, const double *mass, int na, int nb, double beta) {
  const double hbar = 1.0;
  double vrp = 0.0;
  double omegan = (double)nb / (beta * hbar);
  if (nb > 0)
    for (int i = 0; i < na; ++i)
      for (int k = 1; k <= nb; ++k) {
        int k1 = k, k2 = k == 1 ? nb : k - 1;
        const double *a = r + 3 * ((size_t)i + (size_t)na * (k1 - 1));
        const double *b = r + 3 * ((size_t)i + (size_t)na * (k2 - 1));
        double dx = a[0] - b[0], dy = a[1] - b[1], dz = a[2] - b[2];
        double dist = (dx * dx + dy * dy + dz * dz);
        vrp = vrp + 0.5 * mass[i] * (omegan * omegan) * dist;
      }
  return vrp;
}

// md_eq (md_eq.f90:55-323), the Andersen collisions included (therm = AND).
// pre_out[5 per pre-equilibration step]: tps, (nb v + tk + vrp)/na, vrp/na,
//   nb v/na, tk/na  (E_pre_eq.out, md_eq.f90:139-140)
// eq_out[12 per step]: the same five (E_eq.out), temperature (temp_eq.out),
//   tv tokjmol / nm (virial_ke_eq.out), v and tokjmol v / na (V_eq.out),
//   pressure in bar (pressure_eq.out), density (density_eq.out), box length
Status md_eq(double *p, double *r, double *dvdr, double *dvdr2, double dt, const double *mass, int na, int nb,
             double box[3], const double *z, double beta, int ne, int npre_eq, int npt, double ttaufs, Rng &g,
             int &irun, double *pre_out, double *eq_out) {
  const double toK = 3.157733e+5, toKjmol = 2625.49963, tobar = 2.9421e+8, tokgcm3 = 6.147323129e-3,
               tofs = 41.341373;
  int nbaro = npt ? 1 : 0;
  double vir[9] = {0}, vir_lf[9] = {0};
  double v, v1, v2, v3, tv, tk;
  const int nm = na / 3;
  double dtfs = dt / tofs;
  double thresh;
  if (!npt) {
    if (ttaufs > 0.0 && P.therm == GB_THERM_AND) thresh = dtfs / ttaufs;
    else thresh = std::max(0.01, 1.0 / std::sqrt((double)ne));
  } else {
    thresh = 0.01;
  }
  Status st;
  if (npt) {  // quick NVT pre-equilibration (md_eq.f90:93-157)
    int nq = std::min(20000, ne / 10);
    if (npre_eq != 0) nq = npre_eq;
    for (int jq = 1; jq <= nq; ++jq) {
      st = evolve_pi(p, r, v, v1, v2, v3, dvdr, dvdr2, dt, mass, na, nb, box, z, beta, vir, vir_lf, g, irun, 0,
                     nullptr);
      if (st) return st;
      double tps = 1.0e-3 * jq * dtfs;
      kinetic_rpmd(p, na, tk, mass, nb);
      double vrp = spring_energy(r, mass, na, nb, beta);
      if (pre_out) {
        double *o = pre_out + 5 * (size_t)(jq - 1);
        o[0] = tps;
        o[1] = (nb * v + tk + vrp) / na;
        o[2] = vrp / na;
        o[3] = (nb * v) / na;
        o[4] = tk / na;
      }
      if (P.therm == GB_THERM_AND)
        if (ran2(g, irun, 0.0, 1.0) < thresh) sample_rpmd(p, na, nb, mass, beta, g, irun);
    }
  }
  for (int je = 1; je <= ne; ++je) {  // md_eq.f90:181-318, jout = 1
    st = evolve_pi(p, r, v, v1, v2, v3, dvdr, dvdr2, dt, mass, na, nb, box, z, beta, vir, vir_lf, g, irun, nbaro,
                   nullptr);
    if (st) return st;
    double tps = 1.0e-3 * je * dtfs;
    double tvxyz[3], tq1, tq2;
    virial_ke(r, dvdr, dvdr2, tv, tvxyz, tq1, tq2, beta, na, nb);
    double pres = pressure(vir, tv, na, box);
    double vol = box[0] * box[1] * box[2];
    double wmass = mass[0] + mass[1] + mass[2];
    double den = tokgcm3 * (wmass * (double)nm / vol);
    kinetic_rpmd(p, na, tk, mass, nb);
    double vrp = spring_energy(r, mass, na, nb, beta);
    double temp = toK * (2.0 * tk / ((double)(3 * na - P.nctot - 3) * (double)nb)) / (double)nb;
    if (eq_out) {
      double *o = eq_out + 12 * (size_t)(je - 1);
      o[0] = tps;
      o[1] = (nb * v + tk + vrp) / na;
      o[2] = vrp / na;
      o[3] = (nb * v) / na;
      o[4] = tk / na;
      o[5] = temp;
      o[6] = tv * toKjmol / (double)nm;
      o[7] = v;
      o[8] = toKjmol * (v / na);
      o[9] = pres * tobar;
      o[10] = den;
      o[11] = box[0];
    }
    if (P.therm == GB_THERM_AND)
      if (ran2(g, irun, 0.0, 1.0) < thresh) sample_rpmd(p, na, nb, mass, beta, g, irun);
  }
  return GB_OK;
}

}  // namespace orc
