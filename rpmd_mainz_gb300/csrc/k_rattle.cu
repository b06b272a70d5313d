// k_rattle.cu -- RATTLE and the rigid ring-polymer step on the device (FP64).
//
// rattle_s1 / rattle_s2 (md_rattle.f90:33-271): three distance constraints per
// water (O-H1, O-H2, H1-H2; rattle_setup, md_rattle.f90:1-31), relative
// tolerance 1e-6, Gauss-Seidel sweeps over the molecule's bonds, at most 1000
// sweeps.  Molecules are independent, so one thread takes one molecule of one
// bead and runs the reference's sweep sequence.  The reference's constraint
// virial keeps a running quirk: vir(1,3) = vir(1,2) - gdx*dz is assigned, not
// accumulated, so the final vir(1,3) is vir(1,2) at the last correction minus
// that correction's term (md_rattle.f90:124, 233).  Each thread records its
// molecule's sums and last correction; a per-bead reduction rebuilds the value.
// The reference stops when the LAST molecule's sweep count reaches the limit
// (the counter is reset per molecule, md_rattle.f90:149, 258); the device
// raises the same status.
//
// evolve_rig_pi (evolve_rigid.f90:100-224): the nb velocity-Verlet substeps
// with primitive bead springs (bead_forces, evolve_rigid.f90:226-278) and
// RATTLE touch only one molecule's beads, so one block holds whole ring
// polymers and runs all substeps; the springs exchange bead positions through
// shared memory.
#include <cmath>
#include <vector>

#include "gb_common.cuh"
#include "gb_context.h"
#include "gb_kernels.h"

namespace {

constexpr double RTOL = 1e-6;
// sweep limit of both stages (md_rattle.f90 fixes maxit = 1000); lowered only
// through gbrpmd_rattle_set_itmax, which tests use to reach the error path
int g_rattle_itmax = 1000;

struct RatPar {
  double rcb[3];  // squared constrained lengths: reoh^2, reoh^2, rehh^2
  double rm[3];   // 1/mass of O, H1, H2
  double g2[3];   // 1 / ((rm1 + rm2) rcb) per bond (stage-2 multiplier)
  int itmax;      // sweep limit
};

// bond b of a molecule: atoms (ii, jj)
GB_D void bond_atoms(int b, int &ii, int &jj) {
  ii = b == 2 ? 1 : 0;
  jj = b == 0 ? 1 : 2;
}

// One molecule, stage 1; returns the sweeps used; rec[0..4] = v11, v12, v22,
// v33, v23 sums, rec[5] = the last correction's gdx*dz term, rec[6] = 1 if any
// correction.  The sweeps follow the reference's order and tests.  Every
// correction of bond b moves p, dvdr and the virial along the same vector (the
// bond at the start, rold), so the sweeps update r and sum gamma per bond, and
// p, dvdr and the virial sums take the summed gamma once at the end: the
// reference's sums, reassociated.  FP64 divisions cost ~10 FP64 operations on
// this GPU: those by dt become products with 1/dt.  Both change results by
// rounding only.
GB_D int rattle1_mol(double *r, const double *rold, double *p, double *f, double dt,
                     const RatPar &rp, double *rec) {
  const double idt = 1.0 / dt;
  double ov[3][3], gsum[3] = {0.0, 0.0, 0.0}, glast = 0.0;
  int blast = -1;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    int ii, jj;
    bond_atoms(b, ii, jj);
#pragma unroll
    for (int x = 0; x < 3; ++x) ov[b][x] = rold[3 * jj + x] - rold[3 * ii + x];
  }
  bool done = false;
  int it = 0;
  while (!done && it < rp.itmax) {
    done = true;
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      int ii, jj;
      bond_atoms(b, ii, jj);
      const double dx1 = r[3 * jj] - r[3 * ii], dy1 = r[3 * jj + 1] - r[3 * ii + 1], dz1 = r[3 * jj + 2] - r[3 * ii + 2];
      const double d2 = dx1 * dx1 + dy1 * dy1 + dz1 * dz1;
      const double diff = rp.rcb[b] - d2;
      if (fabs(diff) > rp.rcb[b] * RTOL) {
        const double rm1 = rp.rm[jj], rm2 = rp.rm[ii];
        const double dot = dx1 * ov[b][0] + dy1 * ov[b][1] + dz1 * ov[b][2];
        const double gamma = diff / (2.0 * (rm1 + rm2) * dot);
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          const double g = gamma * ov[b][x];
          r[3 * jj + x] += rm1 * g;
          r[3 * ii + x] -= rm2 * g;
        }
        gsum[b] += gamma;
        glast = gamma;
        blast = b;
        done = false;
      }
    }
    ++it;
  }
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    if (gsum[b] == 0.0) continue;
    int ii, jj;
    bond_atoms(b, ii, jj);
    const double g = gsum[b] * idt;
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      p[3 * jj + x] += g * ov[b][x];
      p[3 * ii + x] -= g * ov[b][x];
      f[3 * jj + x] += 2.0 * g * ov[b][x];
      f[3 * ii + x] -= 2.0 * g * ov[b][x];
    }
    const double g2 = 2.0 * g;
    rec[0] -= g2 * ov[b][0] * ov[b][0];
    rec[1] -= g2 * ov[b][0] * ov[b][1];
    rec[2] -= g2 * ov[b][1] * ov[b][1];
    rec[3] -= g2 * ov[b][2] * ov[b][2];
    rec[4] -= g2 * ov[b][1] * ov[b][2];
  }
  if (blast >= 0) {
    rec[5] = (2.0 * glast * idt * ov[blast][0]) * ov[blast][2];
    rec[6] = 1.0;
  }
  return it;
}

// One molecule, stage 2 (velocity constraints).  r does not change here, so
// the bond vectors are fixed and only p must follow every correction; dvdr and
// the virial sums take the summed gamma per bond at the end (as in stage 1).
GB_D int rattle2_mol(const double *r, double *p, double *f, double dt, const RatPar &rp,
                     double *rec) {
  const double ihalfdt = 2.0 / dt;
  double bv[3][3], gsum[3] = {0.0, 0.0, 0.0}, glast = 0.0;
  int blast = -1;
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    int ii, jj;
    bond_atoms(b, ii, jj);
#pragma unroll
    for (int x = 0; x < 3; ++x) bv[b][x] = r[3 * jj + x] - r[3 * ii + x];
  }
  bool done = false;
  int it = 0;
  while (!done && it <= rp.itmax) {
    done = true;
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      int ii, jj;
      bond_atoms(b, ii, jj);
      const double rm1 = rp.rm[jj], rm2 = rp.rm[ii];
      const double dvx1 = p[3 * jj] * rm1 - p[3 * ii] * rm2;
      const double dvy1 = p[3 * jj + 1] * rm1 - p[3 * ii + 1] * rm2;
      const double dvz1 = p[3 * jj + 2] * rm1 - p[3 * ii + 2] * rm2;
      const double dot = bv[b][0] * dvx1 + bv[b][1] * dvy1 + bv[b][2] * dvz1;
      const double gamma = -dot * rp.g2[b];
      if (fabs(gamma) > RTOL) {
#pragma unroll
        for (int x = 0; x < 3; ++x) {
          const double g = gamma * bv[b][x];
          p[3 * jj + x] += g;
          p[3 * ii + x] -= g;
        }
        gsum[b] += gamma;
        glast = gamma;
        blast = b;
        done = false;
      }
    }
    ++it;
  }
#pragma unroll
  for (int b = 0; b < 3; ++b) {
    if (gsum[b] == 0.0) continue;
    int ii, jj;
    bond_atoms(b, ii, jj);
    const double g = gsum[b] * ihalfdt;
#pragma unroll
    for (int x = 0; x < 3; ++x) {
      f[3 * jj + x] += g * bv[b][x];
      f[3 * ii + x] -= g * bv[b][x];
    }
    rec[0] -= g * bv[b][0] * bv[b][0];
    rec[1] -= g * bv[b][0] * bv[b][1];
    rec[2] -= g * bv[b][1] * bv[b][1];
    rec[3] -= g * bv[b][2] * bv[b][2];
    rec[4] -= g * bv[b][1] * bv[b][2];
  }
  if (blast >= 0) {
    rec[5] = (glast * ihalfdt * bv[blast][0]) * bv[blast][2];
    rec[6] = 1.0;
  }
  return it;
}

// RATTLE on B beads x nm molecules; records[b][m][8]
__global__ void k_rattle(int stage, double *r, const double *rold, double *p, double *f, int nm,
                         int B, double dt, RatPar rp, double *records, unsigned *status) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nm * B) return;
  const int m = (int)(t % nm);
  double rl[9], pl[9], fl[9], ro[9];
  double rec[8] = {0, 0, 0, 0, 0, 0, 0, 0};
#pragma unroll
  for (int d = 0; d < 9; ++d) {
    rl[d] = r[t * 9 + d];
    pl[d] = p[t * 9 + d];
    fl[d] = f[t * 9 + d];
  }
  int it;
  if (stage == 1) {
#pragma unroll
    for (int d = 0; d < 9; ++d) ro[d] = rold[t * 9 + d];
    it = rattle1_mol(rl, ro, pl, fl, dt, rp, rec);
    if (m == nm - 1 && it >= rp.itmax) atomicOr(status, ST_RATTLE1);
  } else {
    it = rattle2_mol(rl, pl, fl, dt, rp, rec);
    if (m == nm - 1 && it >= rp.itmax) atomicOr(status, ST_RATTLE2);
  }
#pragma unroll
  for (int d = 0; d < 9; ++d) {
    r[t * 9 + d] = rl[d];
    p[t * 9 + d] = pl[d];
    f[t * 9 + d] = fl[d];
  }
  double *o = records + t * 8;
#pragma unroll
  for (int d = 0; d < 8; ++d) o[d] = rec[d];
}

// per-bead constraint virial with the running vir(1,3) of the reference;
// vir_out[b][9] (written, or added with weight `w` when accumulate)
__global__ void k_rattle_virial(const double *records, int nm, int B, double *vir_out, double w,
                                int accumulate) {
  const int b = blockIdx.x;
  __shared__ double sh[5][256];
  __shared__ int shlast[256];
  double s[5] = {0, 0, 0, 0, 0};
  int last = -1;
  for (int m = threadIdx.x; m < nm; m += blockDim.x) {
    const double *rec = records + ((long long)b * nm + m) * 8;
#pragma unroll
    for (int d = 0; d < 5; ++d) s[d] += rec[d];
    if (rec[6] != 0.0) last = m;
  }
#pragma unroll
  for (int d = 0; d < 5; ++d) sh[d][threadIdx.x] = s[d];
  shlast[threadIdx.x] = last;
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot[5] = {0, 0, 0, 0, 0};
    int lm = -1;
    for (int t = 0; t < (int)blockDim.x; ++t) {
#pragma unroll
      for (int d = 0; d < 5; ++d) tot[d] += sh[d][t];
      lm = max(lm, shlast[t]);
    }
    const double v13 = lm >= 0 ? tot[1] - records[((long long)b * nm + lm) * 8 + 5] : 0.0;
    double v[9];
    v[0] = tot[0];            // (1,1)
    v[3] = tot[1];            // (1,2)
    v[6] = v13;               // (1,3)
    v[4] = tot[2];            // (2,2)
    v[8] = tot[3];            // (3,3)
    v[7] = tot[4];            // (2,3)
    v[1] = v[3];              // (2,1) = (1,2)
    v[2] = v[6];              // (3,1) = (1,3)
    v[5] = v[7];              // (3,2) = (2,3)
    double *o = vir_out + (accumulate ? 0 : (long long)b * 9);
    if (accumulate) {
      for (int d = 0; d < 9; ++d) atomicAdd(o + d, w * v[d]);
    } else {
      for (int d = 0; d < 9; ++d) o[d] = v[d];
    }
  }
}

// evolve_rig_pi substeps (evolve_rigid.f90:132-170) for whole ring polymers:
// thread = (molecule, bead), block = mpb molecules x nb beads
__global__ void k_rig_substeps(double *r, double *p, double *f2, int nm, int nb, int mpb, double smalldt,
                               double omegan2, RatPar rp, const double *mass3, unsigned *status) {
  extern __shared__ double shr[];  // [mpb][nb][9]
  const int ml = threadIdx.x / nb, k = threadIdx.x % nb;
  const int m = blockIdx.x * mpb + ml;
  const bool valid = ml < mpb && m < nm;
  const double halfsmalldt = 0.5 * smalldt;
  const double sdm[3] = {smalldt / mass3[0], smalldt / mass3[1], smalldt / mass3[2]};
  double rl[9], pl[9], fl[9], ro[9], rec[8];
  const long long S = 9LL * nm;  // doubles per bead
  if (valid) {
#pragma unroll
    for (int d = 0; d < 9; ++d) {
      rl[d] = r[S * k + 9LL * m + d];
      pl[d] = p[S * k + 9LL * m + d];
    }
  }
  auto springs = [&]() {
    if (valid) {
#pragma unroll
      for (int d = 0; d < 9; ++d) shr[(ml * nb + k) * 9 + d] = rl[d];
    }
    __syncthreads();
    if (valid) {
      const int km = k == 0 ? nb - 1 : k - 1, kp = k == nb - 1 ? 0 : k + 1;
#pragma unroll
      for (int d = 0; d < 9; ++d) {
        const double x1 = rl[d], x2 = shr[(ml * nb + km) * 9 + d], x3 = shr[(ml * nb + kp) * 9 + d];
        fl[d] = nb > 1 ? mass3[d / 3] * omegan2 * (2.0 * x1 - x2 - x3) : 0.0;
      }
    }
    __syncthreads();
  };
  springs();
  for (int is = 0; is < nb; ++is) {
    if (valid) {
#pragma unroll
      for (int d = 0; d < 9; ++d) {
        ro[d] = rl[d];
        pl[d] = pl[d] - halfsmalldt * fl[d];
        rl[d] = rl[d] + pl[d] * sdm[d / 3];
      }
#pragma unroll
      for (int d = 0; d < 8; ++d) rec[d] = 0.0;
      const int it = rattle1_mol(rl, ro, pl, fl, smalldt, rp, rec);
      if (m == nm - 1 && it >= rp.itmax) atomicOr(status, ST_RATTLE1);
    }
    springs();
    if (valid) {
#pragma unroll
      for (int d = 0; d < 9; ++d) pl[d] = pl[d] - halfsmalldt * fl[d];
#pragma unroll
      for (int d = 0; d < 8; ++d) rec[d] = 0.0;
      const int it = rattle2_mol(rl, pl, fl, smalldt, rp, rec);
      if (m == nm - 1 && it >= rp.itmax) atomicOr(status, ST_RATTLE2);
    }
  }
  if (valid) {
#pragma unroll
    for (int d = 0; d < 9; ++d) {
      r[S * k + 9LL * m + d] = rl[d];
      p[S * k + 9LL * m + d] = pl[d];
      f2[S * k + 9LL * m + d] = fl[d];
    }
  }
}

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

const gb_params &current_params();  // api.cpp

namespace {

// drop-in single-bead calls share one small device workspace
struct RattleWs {
  int nm = 0;
  double *r = nullptr, *rold = nullptr, *p = nullptr, *f = nullptr, *rec = nullptr, *vir = nullptr;
  double *mass = nullptr;
  unsigned *status = nullptr;
  cudaStream_t s = nullptr;
} g_ws;

RatPar make_rp(const gb_params &P, const double *mass3) {
  RatPar rp;
  rp.itmax = g_rattle_itmax;
  const double rehh = 2.0 * std::sin(0.5 * P.theta) * P.reoh;
  rp.rcb[0] = P.reoh * P.reoh;
  rp.rcb[1] = P.reoh * P.reoh;
  rp.rcb[2] = rehh * rehh;
  for (int i = 0; i < 3; ++i) rp.rm[i] = 1.0 / mass3[i];
  for (int b = 0; b < 3; ++b) {
    const int ii = b == 2 ? 1 : 0, jj = b == 0 ? 1 : 2;  // bond_atoms
    rp.g2[b] = 1.0 / ((rp.rm[jj] + rp.rm[ii]) * rp.rcb[b]);
  }
  return rp;
}

#define CK(x)                                             \
  do {                                                    \
    cudaError_t e_ = (x);                                 \
    if (e_ != cudaSuccess) return ctx_check_cuda(e_, #x); \
  } while (0)

int ws_ensure(int nm) {
  if (g_ws.nm >= nm && g_ws.r) return GB_OK;
  for (void *q : {(void *)g_ws.r, (void *)g_ws.rold, (void *)g_ws.p, (void *)g_ws.f, (void *)g_ws.rec,
                  (void *)g_ws.vir, (void *)g_ws.status})
    if (q) cudaFree(q);
  const size_t n = 9 * (size_t)nm;
  CK(cudaMalloc(&g_ws.r, sizeof(double) * n));
  CK(cudaMalloc(&g_ws.rold, sizeof(double) * n));
  CK(cudaMalloc(&g_ws.p, sizeof(double) * n));
  CK(cudaMalloc(&g_ws.f, sizeof(double) * n));
  CK(cudaMalloc(&g_ws.rec, sizeof(double) * 8 * (size_t)nm));
  CK(cudaMalloc(&g_ws.vir, sizeof(double) * 9));
  CK(cudaMalloc(&g_ws.status, sizeof(unsigned)));
  if (!g_ws.s) CK(cudaStreamCreateWithFlags(&g_ws.s, cudaStreamNonBlocking));
  CK(cudaMemsetAsync(g_ws.status, 0, sizeof(unsigned), g_ws.s));
  g_ws.nm = nm;
  return GB_OK;
}

int rattle_dropin(int stage, double *r, const double *rold, double *p, int nm, const double *mass,
                  double dt, double *dvdr, double *vir, int na) {
  if (na != 3 * nm) return ctx_set_error(GB_E_ARG, "na must be 3*nm");
  const gb_params &P = current_params();
  if (3 * nm != P.nctot) return ctx_set_error(GB_E_ARG, "number of bonds inconsistent in shake/rattle routine");
  int st = ws_ensure(nm);
  if (st) return st;
  const size_t n = 9 * (size_t)nm;
  cudaStream_t s = g_ws.s;
  CK(cudaMemcpyAsync(g_ws.r, r, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  if (stage == 1) CK(cudaMemcpyAsync(g_ws.rold, rold, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(g_ws.p, p, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  CK(cudaMemcpyAsync(g_ws.f, dvdr, sizeof(double) * n, cudaMemcpyHostToDevice, s));
  RatPar rp = make_rp(P, mass);
  k_rattle<<<nblk(nm, 128), 128, 0, s>>>(stage, g_ws.r, g_ws.rold, g_ws.p, g_ws.f, nm, 1, dt, rp,
                                         g_ws.rec, g_ws.status);
  k_rattle_virial<<<1, 256, 0, s>>>(g_ws.rec, nm, 1, g_ws.vir, 1.0, 0);
  if (stage == 1) CK(cudaMemcpyAsync(r, g_ws.r, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(p, g_ws.p, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(dvdr, g_ws.f, sizeof(double) * n, cudaMemcpyDeviceToHost, s));
  CK(cudaMemcpyAsync(vir, g_ws.vir, sizeof(double) * 9, cudaMemcpyDeviceToHost, s));
  CK(cudaGetLastError());
  unsigned stw = 0;
  CK(cudaMemcpyAsync(&stw, g_ws.status, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  if (stw) {
    CK(cudaMemsetAsync(g_ws.status, 0, sizeof(unsigned), g_ws.s));
    return stage == 1 ? ctx_set_error(GB_E_RATTLE1, "max iterations exceeded in rattle stage 1")
                      : ctx_set_error(GB_E_RATTLE2, "max iterations exceeded in rattle stage 2");
  }
  return GB_OK;
}

}  // namespace

int dev_rattle_set_itmax(int itmax) {
  if (itmax < 1) return ctx_set_error(GB_E_ARG, "rattle sweep limit must be >= 1");
  g_rattle_itmax = itmax;
  return GB_OK;
}

int dev_rattle_setup(int nm, const gb_params &P) {
  (void)P;
  if (3 * nm > 5000) return ctx_set_error(GB_E_ARG, "rattle: 3*nm exceeds nbondmax = 5000 (globals.inc:26)");
  return ws_ensure(nm);
}

int dev_rattle_s1(double *r, const double *rold, double *p, int nm, const double *mass, double dt,
                  double *dvdr, double *vir, int na) {
  return rattle_dropin(1, r, rold, p, nm, mass, dt, dvdr, vir, na);
}

int dev_rattle_s2(double *r, double *p, int nm, const double *mass, double dt, double *dvdr,
                  double *vir, int na) {
  return rattle_dropin(2, r, nullptr, p, nm, mass, dt, dvdr, vir, na);
}

int term_forces_rigid(gb_context *c);  // step.cpp: forces(r, v, dvdr, nb, ..., 1)

int dev_evolve_rig_pi(gb_context *c, double dt, double beta, double *vir_inout) {
  if (c->nbaro && c->P.baro != GB_BARO_BER)
    return ctx_set_error(GB_E_UNSUPPORTED, "only the Berendsen barostat (baro = BER) is on the device path");
  if (3 * c->nm != c->P.nctot) return ctx_set_error(GB_E_ARG, "number of bonds inconsistent in shake/rattle routine");
  const int nb = c->nb, nm = c->nm;
  const long long N = 3LL * c->na * nb;
  cudaStream_t s = c->stream;
  RatPar rp = make_rp(c->P, c->h_mass3);
  const double halfdt = 0.5 * dt, smalldt = dt / (double)nb;
  double omegan = nb / (beta * 1.0);
  omegan = omegan * omegan;
  // thermostat kick with halfdt (evolve_rigid.f90:124-128), then p -= dt/2 dvdr (132)
  int st = therm_kick(c, halfdt, beta);
  if (st) return st;
  launch_axpy(s, c->p, c->dvdr, -halfdt, N);
  // whole warps, but as many blocks as the molecules allow: the substeps are
  // FP64-bound, so every SM should hold some of them
  const int mpb = nb >= 32 ? 1 : (32 + nb - 1) / nb;
  const size_t smem = sizeof(double) * 9 * (size_t)mpb * nb;
  prof_begin(c, PR_RATTLE);
  k_rig_substeps<<<nblk(nm, mpb), mpb * nb, smem, s>>>(c->r, c->p, c->dvdr2, nm, nb, mpb, smalldt,
                                                      omegan, rp, c->mass, c->status);
  prof_end(c, PR_RATTLE, (double)nm * nb * nb);
  // intermolecular forces on all beads (evolve_rigid.f90:174)
  if ((st = term_forces_rigid(c))) return st;
  // p -= dt/2 dvdr; rattle stage 2 with dt, constraint virial (evolve_rigid.f90:181-190)
  launch_axpy(s, c->p, c->dvdr, -halfdt, N);
  double *rec = c->g;  // nb*nm*8 <= 3*na*nb doubles
  prof_begin(c, PR_RATTLE);
  k_rattle<<<nblk((long long)nm * nb, 128), 128, 0, s>>>(2, c->r, nullptr, c->p, c->dvdr, nm, nb, dt, rp,
                                                        rec, c->status);
  prof_end(c, PR_RATTLE, (double)nm * nb);
  double *vslot = c->acc + (size_t)ACC_INT * ACC_STRIDE;
  k_rattle_virial<<<nb, 256, 0, s>>>(rec, nm, nb, vslot + 1, 1.0, 1);
  c->plan.B_int = nb;  // vir_hf = sum_k vir_k / nb (evolve_rigid.f90:198)
  CK(cudaMemsetAsync(c->dvdr2, 0, sizeof(double) * N, s));
  c->launches += 6;
  if ((st = therm_kick(c, halfdt, beta))) return st;  // evolve_rigid.f90:192-196
  CK(cudaGetLastError());
  if (c->nbaro) {
    // Berendsen barostat (evolve_rigid.f90:203-213): vir = vir_lf + vir_hf +
    // the caller's vir; tv, tvxyz from virial_ke with the zeroed dvdr2 (one
    // call, kinetic.f90:1-54); the accumulators are read on the host
    double *ke = c->acc + (size_t)ACC_KE * ACC_STRIDE;
    CK(cudaMemsetAsync(ke, 0, sizeof(double) * ACC_STRIDE, s));
    launch_virial_ke(s, c->r, c->dvdr, c->dvdr2, c->na, nb, ke);
    c->launches += 1;
    if ((st = dev_collect(c, 2, dt, beta))) return st;
    double *vin = vir_inout ? vir_inout : c->rig_vir;
    double vir[9];
    for (int i = 0; i < 9; ++i) vir[i] = c->e_vir_lf[i] + c->e_vir_hf[i] + vin[i];
    if (!vir_inout)  // the drop-in caller updates its own vir
      for (int i = 0; i < 9; ++i) c->rig_vir[i] = vir[i];
    const double *K = c->h_acc + (size_t)ACC_KE * ACC_STRIDE;
    const double tq1 = 0.5 * K[0] / nb, tq2 = 0.5 * K[1] / nb;
    const double tc = 0.5 * (3 * c->na - 3 - c->P.nctot) / beta;
    const double tv = tc + tq1 + tq2;
    double tvxyz[3];
    for (int j = 0; j < 3; ++j) tvxyz[j] = tc / 3 + 0.5 * K[2 + j] / nb + 0.5 * K[5 + j] / nb;
    if ((st = beren_driver(c, vir, tv, tvxyz, dt, nullptr))) return st;
    CK(cudaGetLastError());
  }
  return GB_OK;
}
