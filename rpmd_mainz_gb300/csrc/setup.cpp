// setup.cpp -- host-side set-up and the equilibration loop of the reference's
// driver, in the order main.f90 runs them:
//   setup_box_size (setup_options.f90:191-270, CUB lattice)
//   cubic          (setup_positions.f90:94-150)
//   setup_ewald    (setup_options.f90:104-189)
//   sample_rpmd + pshift (module_thermostat.f90:199-264), drawn from the
//                  library's ran2/gaussian stream
//   md_eq step loop (md_eq.f90:182-323): evolve, then the Andersen collision
//                  test ran2(irun) < thresh -> resample all momenta
#include <cmath>
#include <cstring>
#include <vector>

#include "gb_common.h"
#include "gb_context.h"
#include "gb_rng.h"

extern "C" double gbrpmd_ran2(int *idum, const double *rmin, const double *rmax);
extern RngState g_rng;  // api.cpp
const gb_params &current_params();

extern "C" {

int gbrpmd_setup_box_size(const int *ncellxyz, double rho, double wmass, double *boxlxyz, int *nm) {
  const double emass = 9.1093826e-31, toA = 0.5291772108;  // globals.inc
  if (ncellxyz[0] <= 0 || ncellxyz[1] <= 0 || ncellxyz[2] <= 0 || rho <= 0.0)
    return ctx_set_error(GB_E_ARG, "invalid lattice or density");
  const int n = ncellxyz[0] * ncellxyz[1] * ncellxyz[2];
  double vbox = (n * emass * wmass) / (rho * 1000.0);
  vbox = vbox / std::pow(toA * 1e-10, 3);
  const double totcell = (double)n;
  const double boxl = std::pow(vbox / totcell, 1.0 / 3.0);
  for (int i = 0; i < 3; ++i) boxlxyz[i] = boxl * ncellxyz[i];
  *nm = n;
  return GB_OK;
}

int gbrpmd_cubic_lattice(double *r, int nm, int nb, const double *boxlxyz, const int *ncellxyz,
                         double theta, double reoh) {
  if (ncellxyz[0] * ncellxyz[1] * ncellxyz[2] != nm) return ctx_set_error(GB_E_ARG, "* Problem in cubic setup!");
  const double hx = reoh, gx = reoh * std::cos(theta), gy = reoh * std::sin(theta);
  double del[3];
  for (int i = 0; i < 3; ++i) del[i] = boxlxyz[i] / (double)ncellxyz[i];
  int itel = 0;
  double dx = -del[0];
  for (int i = 0; i < ncellxyz[0]; ++i) {
    dx = dx + del[0];
    double dy = -del[1];
    for (int j = 0; j < ncellxyz[1]; ++j) {
      dy = dy + del[1];
      double dz = -del[2];
      for (int k = 0; k < ncellxyz[2]; ++k) {
        dz = dz + del[2];
        double *m = r + 9 * (size_t)itel++;
        m[0] = dx; m[1] = dy; m[2] = dz;
        m[3] = dx + hx; m[4] = dy + 0.0; m[5] = dz + 0.0;
        m[6] = dx + gx; m[7] = dy + gy; m[8] = dz + 0.0;
      }
    }
  }
  const size_t S = 9 * (size_t)nm;
  for (int b = 1; b < nb; ++b) std::memcpy(r + S * b, r, sizeof(double) * S);  // copy bead 1
  return GB_OK;
}

int gbrpmd_setup_ewald(int na, const double *boxlxyz, gb_params *P) {
  const double pi = std::acos(-1.0), cvar = 1.2;
  if (boxlxyz[0] == boxlxyz[1] && boxlxyz[0] == boxlxyz[2] && P->iamcub) {
    P->iamcub = 1;
    P->wrcut = std::fmin(0.5, cvar * std::pow((double)na, -1.0 / 6.0));
    if (P->ecut <= 0.0) {
      P->walpha = pi / P->wrcut;
      P->kmax = (int)P->walpha;
      P->rkmax = 2.0 * pi * P->walpha;
    } else {
      double s = std::sqrt(-std::log(P->ecut));
      P->walpha = s / P->wrcut;
      P->kmax = (int)(s * P->walpha / pi);
      P->rkmax = 2.0 * s * P->walpha;
    }
  } else {
    P->iamcub = 0;
    double rshort = std::fmin(boxlxyz[0], std::fmin(boxlxyz[1], boxlxyz[2]));
    P->wrcut = rshort * std::fmin(0.5, cvar * std::pow((double)na, -1.0 / 6.0));
    P->walpha = pi / P->wrcut;
    double rlong = std::fmax(boxlxyz[0], std::fmax(boxlxyz[1], boxlxyz[2]));
    P->rkmax = 2.0 * pi * P->walpha;
    P->kmax = (int)(P->walpha * rlong);
  }
  return GB_OK;
}

int gbrpmd_sample_rpmd(double *p, int na, int nb, const double *mass, double beta, int *irun) {
  rng_sample_rpmd(g_rng, p, na, nb, mass, beta, irun);
  return GB_OK;
}

// md_eq step loop on a resident context: nsteps evolve_pi steps, each followed
// by the Andersen collision test; energies[4*s .. 4*s+3] = v, vew, vlj, vint
// of step s when `energies` is not NULL (that needs one synchronisation per
// step).  Momenta for a collision are drawn on the host and uploaded.
int gbrpmd_run_md_eq(gb_context *c, int nsteps, double dt, double beta, double thresh, int *irun,
                     double *energies) {
  if (!c->own_params) c->P = current_params();
  const gb_params &P = c->P;
  std::vector<double> hmass, hp;
  if (P.therm == GB_THERM_AND) {
    hmass.resize(c->na);
    if (cudaMemcpyAsync(hmass.data(), c->mass, sizeof(double) * c->na, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
        cudaStreamSynchronize(c->stream) != cudaSuccess)
      return ctx_set_error(GB_E_CUDA, "mass download failed");
  }
  const double zero = 0.0, one = 1.0;
  c->th_rng = &g_rng;  // PRG / PRL kicks draw the same stream as the collisions
  c->th_idum = irun;
  struct Clear {
    gb_context *c;
    ~Clear() {
      c->th_rng = nullptr;
      c->th_idum = nullptr;
    }
  } clear{c};
  for (int s = 0; s < nsteps; ++s) {
    int st = dev_evolve_step(c, dt, beta);
    if (st) return st;
    // energies, and with a barostat the vir_lf the next step reads, need the
    // step's accumulators; the last step is always collected
    if (energies || c->nbaro || s == nsteps - 1)
      if ((st = dev_collect(c, 1, dt, beta))) return st;
    if (energies) {
      energies[4 * s + 0] = c->e_v;
      energies[4 * s + 1] = c->e_vew;
      energies[4 * s + 2] = c->e_vlj;
      energies[4 * s + 3] = c->e_vint;
    }
    if (P.therm == GB_THERM_AND && gbrpmd_ran2(irun, &zero, &one) < thresh) {
      hp.resize(3 * (size_t)c->na * c->nb);
      gbrpmd_sample_rpmd(hp.data(), c->na, c->nb, hmass.data(), beta, irun);
      if (cudaMemcpyAsync(c->p, hp.data(), sizeof(double) * hp.size(), cudaMemcpyHostToDevice, c->stream) !=
              cudaSuccess ||
          cudaStreamSynchronize(c->stream) != cudaSuccess)
        return ctx_set_error(GB_E_CUDA, "momentum upload failed");
    }
  }
  return GB_OK;
}

}  // extern "C"
