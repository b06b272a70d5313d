// orc.h -- CPU FP64 restatement ("oracle") of the reference RPMD path.
//
// TEST INFRASTRUCTURE ONLY.  Nothing in the product library links, calls or
// reads this code; only tests/, __graft_entry__.smoke() and bench.py (its CPU
// baseline arm) load liborc.so, and only to check or time against it.
//
// Every routine restates the reference Fortran routine named in its comment,
// keeping the reference's loop order and summation order, so that outputs agree
// with the reference to rounding.  Arrays use the Fortran column-major layout
// r(3,na,nb) -> r[i + 3*(j + na*k)] with 0-based i, j, k.
//
// Pinning: the force path (cubic Ewald with M-site, TEM-switched contraction
// correction, contraction to the centroid, Lennard-Jones, intra_morse_harm) and
// 20-step evolve_pi replays are checked against the reference's own golden run
// test/cmp/gentest.cmp (vmd_bead-*.xyz/.frc/.vel, output); see
// tests/test_oracle_golden.py.  The FFTW R2HC/HC2R transform is restated from
// FFTW's published definition (FFTW is an un-vendored, unpinned dependency,
// linked as -lfftw3 by sample_makefiles/make_no_cp2k.inc:12) and checked against
// numpy's real FFT.
#pragma once

#include <cstddef>
#include <cstdint>

#include "../include/gbrpmd.h"

namespace orc {

// The COMMON-block state (main.f90:53-72).  Read-only while forces run, so
// several trajectories may run on different threads.
extern gb_params P;

// Status codes mirror include/gbrpmd.h.
using Status = int;

// Saved state of ran2/gaussian (random.f90:1-72).
struct Rng {
  int iv[32];
  int iy;
  int idum2;
  int iset;
  double gset;
};
void rng_reset(Rng &g);
double ran2(Rng &g, int &idum, double rmin, double rmax);
double gaussian(Rng &g, int &idum, double sigma);

// ---- set-up (setup_options.f90, setup_positions.f90) ----
int setup_box_size_cub(const int ncell[3], double rho, double wmass, double box[3]);
Status cubic(double *r, int nm, const double box[3], const int ncell[3]);
void setup_ewald(int na, const double box[3]);

// ---- transforms (fourier.f90, md_pathi.f90) ----
void realft(double *data, int m, int n, int mode);
void realft_direct(double *data, int m, int n, int mode);
void ring_rpmd(const double *mass, double *monod, int na, int nb, double dt, double beta);

// ---- forces (md_forces.f90) ----
Status forces(double *r, double &v, double *dvdr, int nb, int na, const double box[3],
              const double *z, double virial[9], int iopt);
Status full_forces(double *r, int na, int nb, double &v, double &vew, double &voo,
                   double &vint, double vir[9], const double *z, const double box[3],
                   double *dvdr, double *dvdr2);
Status potenl_opt(double *r, double &v, double *dvdr, double vir[9], int na, int nb,
                  const double box[3], const double *z, const int *list, const int *point,
                  int iopt);

// components
void ewald_cubic(int n, const int *mol, const double *q, const double *r, double &v,
                 double vir[9], double *dvdr, double boxl);
void rwald(int n, const int *mol, const double *q, const double *r, double &v, double vir[9],
           double *dvdr, double rcut, double alpha, int mcell, int ncell);
void kwald(int n, const double *q, const double *r, double &v, double vir[9], double *dvdr,
           double alpha, double rkmax2, int kmax);
Status nei_driver(const double *r, int na, int *list, int *point, int njump, double rcut,
                  const double box[3]);
void lj_driver(const double *r, double *dvdr, double &v, double vir[9], const int *list,
               const int *point, int na, const double box[3], int njump);
void intra_harmonic(const double *r, double *dvdr, int na, double &v, double vir[9]);
void intra_spcfw(const double *r, double *dvdr, int na, double &v, double vir[9]);
void intra_morse_harm(const double *r, double *dvdr, int na, double &v, double vir[9]);
Status ewc_driver_tem(double *r, const double *z, double *dvdr, double &v, double vir[9],
                      int na, const double box[3], const int *list, const int *point);

// ---- integrator (evolve_pi.f90, kinetic.f90, module_thermostat.f90) ----
Status evolve_pi(double *p, double *r, double &v, double &vew, double &vlj, double &vint,
                 double *dvdr, double *dvdr2, double dt, const double *mass, int na, int nb,
                 double box[3], const double *z, double beta, double vir[9], double vir_lf[9],
                 Rng &g, int &irun, int nbaro, double *tv_out);
Status rp_contract_nm(const double *r, double &v, double *dvdr, int nb, int na,
                      const double box[3], const double *z, double vir[9], int nbdf, int iopt);
void ring_contract(const double *r, double *r_c, int na, int nb, int nb_c);
void force_contract(double *dvdr, double *dvdr_c, int na, int nb, int nb_c);
void virial_ke(const double *r, const double *dvdr, const double *dvdr2, double &tv,
               double tvxyz[3], double &tq1, double &tq2, double beta, int na, int nb);
void kinetic_rpmd(const double *p, int na, double &tk, const double *mass, int nb);
double pressure(const double vir[9], double tv, int na, const double box[3]);
double pres_lj_tail(const double box[3], int na);
void beren_baro(const double vir[9], double tv, double dt, double *r, double box[3], int na, int nb);
void beren_baro_nc(const double vir[9], const double tvxyz[3], double dt, double *r, double box[3], int na, int nb);
void beren_driver(const double vir[9], double tv, const double tvxyz[3], double dt, double *r, double box[3], int na,
                  int nb);
// md_eq's step loops (md_eq.f90:55-323) without file output: for ens != NVT
// the nq-step NVT pre-equilibration, then ne steps with nbaro = npt; per step
// the values md_eq prints (see orc_md_eq)
Status md_eq(double *p, double *r, double *dvdr, double *dvdr2, double dt, const double *mass, int na, int nb,
             double box[3], const double *z, double beta, int ne, int npre_eq, int npt, double ttaufs, Rng &g,
             int &irun, double *pre_out, double *eq_out);
// md_eq's output block (md_eq.f90:190-299): out[16] in the order of
// gbrpmd_ctx_estimators; rcm, mdip [nm][3] optional
void md_eq_estimators(const double *r, const double *p, const double *dvdr, const double *dvdr2,
                      const double *mass, const double *z, int na, int nb, double beta, double v,
                      const double vir[9], const double box[3], double out[16], double *rcm, double *mdip);
void sample_rpmd(double *p, int na, int nb, const double *mass, double beta, Rng &g,
                 int &irun);
void pshift(double *p, const double *mass, int na, int nb);
void parinello_therm(double *p, const double *mass, double tau, int na, int nb, double dt,
                     Rng &g, int &irun, double beta);
void parinello_therm_loc(double *p, const double *mass, double tau, int na, int nb, double dt,
                         Rng &g, int &irun, double beta);

// ---- rigid path (md_rattle.f90, evolve_rigid.f90) ----
struct Rattle {
  int nm = 0;
  double *rcb = nullptr;  // squared bond lengths, 3 per molecule
  int *bond = nullptr;    // bonded atom pairs (1-based atom indices), 2 per bond
};
void rattle_setup(Rattle &rt, int nm);
void rattle_free(Rattle &rt);
Status rattle_s1(const Rattle &rt, double *r, const double *rold, double *p, int nm,
                 const double *mass, double dt, double *dvdr, double vir[9], int na);
Status rattle_s2(const Rattle &rt, double *r, double *p, int nm, const double *mass, double dt,
                 double *dvdr, double vir[9], int na);
void bead_forces(const double *r, int na, int nb, double *dvdrb, double beta,
                 const double *mass);
Status evolve_rig_pi(const Rattle &rt, double *p, double *r, double &v, double &v_lf,
                     double &v_hf, double *dvdr, double *dvdr2, double dt, const double *mass,
                     int na, int nb, double box[3], const double *z, double beta,
                     double vir[9], double vir_lf[9], Rng &g, int &irun, int nbaro);

}  // namespace orc
