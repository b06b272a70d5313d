// orc_capi.cpp -- C entry points of the oracle library (liborc.so), loaded with
// ctypes by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline arm.
// TEST INFRASTRUCTURE ONLY (see orc.h).
#include <chrono>
#include <cmath>
#include <cstring>
#include <thread>
#include <vector>

#include "orc.h"

using namespace orc;

extern "C" {

void orc_set_params(const gb_params *p) { P = *p; }
void orc_get_params(gb_params *p) { *p = P; }
int orc_params_size(void) { return (int)sizeof(gb_params); }

// ---- random stream ----
int orc_rng_size(void) { return (int)sizeof(Rng); }
void orc_rng_reset(void *g) { rng_reset(*(Rng *)g); }
double orc_ran2(void *g, int *idum, double rmin, double rmax) { return ran2(*(Rng *)g, *idum, rmin, rmax); }
double orc_gaussian(void *g, int *idum, double sigma) { return gaussian(*(Rng *)g, *idum, sigma); }

// ---- set-up ----
int orc_setup_box_size_cub(const int *ncell, double rho, double wmass, double *box) {
  return setup_box_size_cub(ncell, rho, wmass, box);
}
int orc_cubic(double *r, int nm, const double *box, const int *ncell) { return cubic(r, nm, box, ncell); }
void orc_setup_ewald(int na, const double *box) { setup_ewald(na, box); }

// ---- transforms ----
void orc_realft(double *data, int m, int n, int mode) { realft(data, m, n, mode); }
void orc_realft_direct(double *data, int m, int n, int mode) { realft_direct(data, m, n, mode); }
void orc_ring_rpmd(const double *mass, double *monod, int na, int nb, double dt, double beta) {
  ring_rpmd(mass, monod, na, nb, dt, beta);
}

// ---- forces ----
int orc_forces(double *r, double *v, double *dvdr, int nb, int na, const double *box,
               const double *z, double *virial, int iopt) {
  return forces(r, *v, dvdr, nb, na, box, z, virial, iopt);
}
int orc_full_forces(double *r, int na, int nb, double *v, double *vew, double *voo, double *vint,
                    double *vir, const double *z, const double *box, double *dvdr, double *dvdr2) {
  return full_forces(r, na, nb, *v, *vew, *voo, *vint, vir, z, box, dvdr, dvdr2);
}
void orc_ewald_cubic(int n, const double *q, const double *r, double *v, double *vir,
                     double *dvdr, double boxl) {
  std::vector<int> mol(n);
  for (int j = 0; j < n; ++j) mol[j] = j / 3 + 1;
  std::memset(dvdr, 0, sizeof(double) * 3 * (size_t)n);
  ewald_cubic(n, mol.data(), q, r, *v, vir, dvdr, boxl);
}
int orc_nei_driver(const double *r, int na, int *list, int *point, int njump, double rcut,
                   const double *box) {
  return nei_driver(r, na, list, point, njump, rcut, box);
}
void orc_intra(const double *r, double *dvdr, int na, double *v, double *vir, int model) {
  std::memset(dvdr, 0, sizeof(double) * 3 * (size_t)na);
  if (model == 0) intra_harmonic(r, dvdr, na, *v, vir);
  else if (model == 1) intra_spcfw(r, dvdr, na, *v, vir);
  else intra_morse_harm(r, dvdr, na, *v, vir);
}

// ---- integrators ----
int orc_evolve_pi(double *p, double *r, double *v, double *vew, double *vlj, double *vint,
                  double *dvdr, double *dvdr2, double dt, const double *mass, int na, int nb,
                  double *box, const double *z, double beta, double *vir, double *vir_lf,
                  void *g, int *irun, int nbaro, double *tv) {
  return evolve_pi(p, r, *v, *vew, *vlj, *vint, dvdr, dvdr2, dt, mass, na, nb, box, z, beta, vir,
                   vir_lf, *(Rng *)g, *irun, nbaro, tv);
}
void orc_virial_ke(const double *r, const double *dvdr, const double *dvdr2, double *tv,
                   double *tvxyz, double *tq1, double *tq2, double beta, int na, int nb) {
  virial_ke(r, dvdr, dvdr2, *tv, tvxyz, *tq1, *tq2, beta, na, nb);
}
double orc_pressure(const double *vir, double tv, int na, const double *box) { return pressure(vir, tv, na, box); }
void orc_beren_driver(const double *vir, double tv, const double *tvxyz, double dt, double *r, double *box, int na,
                      int nb) {
  beren_driver(vir, tv, tvxyz, dt, r, box, na, nb);
}
void orc_kinetic_rpmd(const double *p, int na, double *tk, const double *mass, int nb) {
  kinetic_rpmd(p, na, *tk, mass, nb);
}
void orc_md_eq_estimators(const double *r, const double *p, const double *dvdr, const double *dvdr2,
                          const double *mass, const double *z, int na, int nb, double beta, double v,
                          const double *vir, const double *box, double *out, double *rcm, double *mdip) {
  md_eq_estimators(r, p, dvdr, dvdr2, mass, z, na, nb, beta, v, vir, box, out, rcm, mdip);
}
void orc_sample_rpmd(double *p, int na, int nb, const double *mass, double beta, void *g,
                     int *irun) {
  sample_rpmd(p, na, nb, mass, beta, *(Rng *)g, *irun);
}
void orc_ring_contract(const double *r, double *r_c, int na, int nb, int nb_c) {
  ring_contract(r, r_c, na, nb, nb_c);
}
void orc_force_contract(double *dvdr, double *dvdr_c, int na, int nb, int nb_c) {
  force_contract(dvdr, dvdr_c, na, nb, nb_c);
}

// ---- rigid path ----
static Rattle g_rattle;
void orc_rattle_setup(int nm) { rattle_setup(g_rattle, nm); }
int orc_rattle_s1(double *r, const double *rold, double *p, int nm, const double *mass, double dt,
                  double *dvdr, double *vir, int na) {
  return rattle_s1(g_rattle, r, rold, p, nm, mass, dt, dvdr, vir, na);
}
int orc_rattle_s2(double *r, double *p, int nm, const double *mass, double dt, double *dvdr,
                  double *vir, int na) {
  return rattle_s2(g_rattle, r, p, nm, mass, dt, dvdr, vir, na);
}
void orc_bead_forces(const double *r, int na, int nb, double *dvdrb, double beta,
                     const double *mass) {
  bead_forces(r, na, nb, dvdrb, beta, mass);
}
int orc_evolve_rig_pi(double *p, double *r, double *v, double *v_lf, double *v_hf, double *dvdr,
                      double *dvdr2, double dt, const double *mass, int na, int nb, double *box,
                      const double *z, double beta, double *vir, double *vir_lf, void *g,
                      int *irun, int nbaro) {
  return evolve_rig_pi(g_rattle, p, r, *v, *v_lf, *v_hf, dvdr, dvdr2, dt, mass, na, nb, box, z,
                       beta, vir, vir_lf, *(Rng *)g, *irun, nbaro);
}

// ---- md_eq step loop (md_eq.f90:182-323 without the file output) ----
// nsteps evolve_pi steps, each followed by the Andersen collision test
// ran2(irun) < thresh -> sample_rpmd (md_eq.f90:311-315) when therm = AND.
// energies[4*s + 0..3] = v, vew, vlj, vint after step s (may be NULL).
int orc_run_steps(double *p, double *r, double *dvdr, double *dvdr2, double dt, const double *mass,
                  int na, int nb, double *box, const double *z, double beta, int nsteps,
                  double thresh, void *g, int *irun, double *vir_lf, double *energies) {
  double vir[9];
  for (int s = 0; s < nsteps; ++s) {
    double v, vew, vlj, vint, tv;
    int st = evolve_pi(p, r, v, vew, vlj, vint, dvdr, dvdr2, dt, mass, na, nb, box, z, beta, vir,
                       vir_lf, *(Rng *)g, *irun, 0, &tv);
    if (st) return st;
    if (energies) {
      energies[4 * s + 0] = v;
      energies[4 * s + 1] = vew;
      energies[4 * s + 2] = vlj;
      energies[4 * s + 3] = vint;
    }
    if (P.therm == GB_THERM_AND)
      if (ran2(*(Rng *)g, *irun, 0.0, 1.0) < thresh) sample_rpmd(p, na, nb, mass, beta, *(Rng *)g, *irun);
  }
  return GB_OK;
}

int orc_md_eq(double *p, double *r, double *dvdr, double *dvdr2, double dt, const double *mass, int na, int nb,
              double *box, const double *z, double beta, int ne, int npre_eq, int npt, double ttaufs, void *g,
              int *irun, double *pre_out, double *eq_out) {
  return md_eq(p, r, dvdr, dvdr2, dt, mass, na, nb, box, z, beta, ne, npre_eq, npt, ttaufs, *(Rng *)g, *irun,
               pre_out, eq_out);
}

// ---- throughput of independent replicas on host threads ----
// Runs `nthreads` copies of the same trajectory state, each on its own thread
// for nsteps evolve_pi steps (no thermostat collisions), and returns the wall
// time in seconds (negative on failure).
double orc_bench_replicas(int nthreads, const double *p0, const double *r0, const double *dvdr0,
                          const double *dvdr20, double dt, const double *mass, int na, int nb,
                          const double *box0, const double *z, double beta, int nsteps) {
  const size_t N = 3 * (size_t)na * nb;
  std::vector<std::thread> th;
  std::vector<int> status(nthreads, 0);
  auto t0 = std::chrono::steady_clock::now();
  for (int t = 0; t < nthreads; ++t) {
    th.emplace_back([&, t]() {
      std::vector<double> p(p0, p0 + N), r(r0, r0 + N), f(dvdr0, dvdr0 + N), f2(dvdr20, dvdr20 + N);
      double box[3] = {box0[0], box0[1], box0[2]}, vir[9], vir_lf[9] = {0};
      Rng g;
      rng_reset(g);
      int irun = -1;
      for (int s = 0; s < nsteps; ++s) {
        double v, vew, vlj, vint;
        int st = evolve_pi(p.data(), r.data(), v, vew, vlj, vint, f.data(), f2.data(), dt, mass, na,
                           nb, box, z, beta, vir, vir_lf, g, irun, 0, nullptr);
        if (st) { status[t] = st; return; }
      }
    });
  }
  for (auto &x : th) x.join();
  auto t1 = std::chrono::steady_clock::now();
  for (int s : status)
    if (s) return -1.0;
  return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
