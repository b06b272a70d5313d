// gb_kernels.h -- launchers of the device kernels (host-callable).
#pragma once

#include <cuda_runtime.h>

#include "gb_context.h"

// reciprocal-space kernel geometry (k_recip.cu)
int recip_sk_chunk();                // sites per structure-factor block
int recip_group_len();               // m values per structure-factor work item
size_t recip_sk_smem(int kmax);      // dynamic shared memory of the passes
size_t recip_force_smem(int kmax);
void recip_set_attributes();         // raises the kernels' shared-memory limit once
double3 recip_lat(const gb_context *c);  // k per integer index along each axis

// Geometry of one pair search.  Point i of configuration c sits at
// pos[c * cstride + i * pstride + {0,1,2}] (doubles).  `unit` selects the
// unit-box minimum image dx - nint(dx) (rwald, ewald_cubic.f90:121-126);
// otherwise dx - box * nint(dx / box) with dx/box computed as onbox * dx
// (neigh_list.f90:336-342).  Membership is decided by the FP64 test
// dx*dx + dy*dy + dz*dz < rcutsq rounded exactly as the reference rounds it.
struct PairGeom {
  const double *pos;
  long long cstride;
  int pstride;
  int npt;
  int unit;
  double box[3], onbox[3];
  double rcutsq;
  int excl_mol;  // skip pairs with i/3 == j/3 (same molecule; TEM correction)
  int full;      // 1: store each pair in both lists (no parity halving)
};

// ---- pair lists (k_pairs.cu) ----
// wrapped fractional coordinates; optional remainders lo and per-point values
// q (stored in frac.w)
void launch_frac32(cudaStream_t s, const PairGeom &g, int nconf, float4 *frac, float4 *lo = nullptr,
                   const double *q = nullptr, int4 *fx = nullptr);
// every pair within g.rcutsq; with a gate word, only when *gate != 0 (counts
// are then zeroed on the device, so the decision needs no host round trip)
// thr_dev (device): the superset radius squared of a shared list (ListSpread::w + 2)
void launch_build_list(cudaStream_t s, const PairGeom &g, int nconf, const float4 *frac,
                       PairList &pl, unsigned *status, const unsigned *gate = nullptr,
                       const float *thr_dev = nullptr);
// skin lists: displacement test against the rebuild positions, position save
// on a rebuild, and the filter from the superset to the exact list
void launch_skin_check(cudaStream_t s, const PairGeom &g, int nconf, const double *ref, double lim2,
                       unsigned *flag);
void launch_skin_save(cudaStream_t s, const PairGeom &g, int nconf, double *ref, const unsigned *flag,
                      unsigned *rebuilds);
// cell-sorted superset build: the cell grid (false: use the all-pairs build),
// the per-step skin test with cell counts (check = 0: *flag already set; also
// writes frac / lo as launch_frac32), and the gated scatter + build
bool list_cell_grid(const PairGeom &g, int nc[3], int *R, signed char *reach);
// A list shared by B configurations, built on their centroids (mixed real
// space): w (device, 4 floats) holds [0] the step's largest squared distance
// of a site from its centroid, [1] the squared margin of the current list,
// [2] its squared superset radius (the build threshold); base: cut-off +
// skin, dcap: the largest margin the stencil and capacity allow, dmin: the
// smallest margin; all in the list geometry's units.  w = nullptr: off.
struct ListSpread {
  float *w = nullptr;
  float base = 0.f, dcap = 0.f, dmin = 0.f;
};
void launch_cell_count(cudaStream_t s, const PairGeom &g, int nconf, float4 *frac, float4 *lo, const double *q,
                       const CellSort &cs, const double *ref, double lim2, int check, unsigned *flag,
                       int4 *fx = nullptr, const ListSpread &sp = ListSpread());
// site centroids of B configurations and their spread (ListSpread); a spread
// beyond the list's margin sets *moved (a rebuild), beyond dcap sets
// ST_LIST_OVERFLOW in status
void launch_site_centroid(cudaStream_t s, const double *r, double *cen, int na, int B, const ListSpread &sp,
                          unsigned *moved, unsigned *status);
// at a rebuild (*flag): the shared list's margin and superset radius from the
// step's spread; clears the spread word
void launch_spread_update(cudaStream_t s, const unsigned *flag, const ListSpread &sp);
// fixed-point coordinates of B configurations, and in slot order when slot_of
// and fxs are given
void launch_fx_slots(cudaStream_t s, const PairGeom &g, int B, const double *q, const int *slot_of, int4 *fx,
                     int4 *fxs);
// (also saves the reference positions and counts the rebuild, as launch_skin_save)
// fx: the points' fixed-point coordinates (copied into cs.fxs in slot order
// when the list stores slots)
// thr_dev (device): the superset radius squared of a shared list (ListSpread::w + 2)
void launch_build_sorted(cudaStream_t s, const PairGeom &g, int nconf, const float4 *frac, PairList &pl,
                         unsigned *status, const unsigned *gate, const CellSort &cs, double *ref,
                         unsigned *rebuilds, const int4 *fx = nullptr, const float *thr_dev = nullptr);
void launch_list_filter(cudaStream_t s, const PairGeom &g, int nconf, const float4 *frac,
                        const PairList &skin, PairList &pl, unsigned *status);
double list_total(cudaStream_t s, const PairList &pl);  // profiling only (synchronises)
int list_max(cudaStream_t s, const PairList &pl);       // diagnostics only (synchronises)

// ---- Ewald, unit box (k_pairs.cu, k_recip.cu) ----
// rs: M-site substituted positions scaled by 1/L, [B][na][3]; gz (optional,
// [B][na][3]) is zeroed by the same launch
void launch_msite(cudaStream_t s, const double *r, double *rs, int na, int B, double alpha,
                  double scale, double *gz = nullptr);
// box: nullptr for unit-box positions (cubic sum), else the box in bohr (non-cubic)
void launch_ewald_real(cudaStream_t s, const double *rs, const double *q, int na, int B,
                       const PairList &pl, double alpha, const double *box, double *g, double *acc);
// structure factors: per-site power tables, then chunk partials (2 launches)
void launch_recip_sk(cudaStream_t s, gb_context *c, const double *rs, const double *q, int B);
void launch_recip_weights(cudaStream_t s, gb_context *c, int B, double *acc);
void launch_recip_force(cudaStream_t s, gb_context *c, const double *rs, const double *q, int B,
                        double *g);
// ---- mixed precision (k_mixed.cu): FP32 arithmetic, full lists, hi/lo positions ----
// hi.w carries the site charge (launch_frac32 with q)
// box: side lengths of the fractional coordinates (1, 1, 1 for the cubic sum);
// np: lanes per site (8, 16, 32) / per oxygen (2, 4, 8)
// add = false: g is overwritten (no zeroing pass needed)
// fx: fixed-point fractional coordinates with the charge bits in w
// (frac_point); fxs: the same in slot order (lists of slots, PairList::slots);
// npair (profiling): in-cut entries counted
void launch_ewald_real_mx(cudaStream_t s, const int4 *fx, const int4 *fxs, int na, int B, const PairList &pl,
                          double alpha, double rcutsq, const double *box, int np, double *g, double *acc,
                          bool add = true, unsigned long long *npair = nullptr);
void launch_lj_mx(cudaStream_t s, const float4 *hi, const float4 *lo, int na, int B, const PairList &pl,
                  double sigsq, double rcutsq, const double *box, double dscale, int np, double *out, double *acc);
void launch_recip_sk_mx(cudaStream_t s, gb_context *c, const double *rs, const double *q, int B);
// the same structure-factor chunk partials on the tensor cores (k_recip_tc.cu);
// false (nothing launched) when kmax is beyond its tiles
bool launch_recip_sk_tc(cudaStream_t s, gb_context *c, int B, int nchunk);
int recip_sk_tc_chunk();
// the force pass on the tensor cores (k_recip_tc.cu; the default, GBRPMD_RF_TC=0
// for the CUDA-core pass); false (nothing launched) when kmax is beyond its K of 32
bool launch_recip_force_tc(cudaStream_t s, gb_context *c, int B, double *g);
bool recip_force_tc_on(const gb_context *c);  // the mixed force pass runs on the tensor cores
void launch_recip_weights_mx(cudaStream_t s, gb_context *c, int B, double *acc);
void launch_recip_force_mx(cudaStream_t s, gb_context *c, int B, double *g);
void recip_set_attributes_mx();
// out[b] = sign * chain_rule(scale * g[b]) (+= when accumulate); with g2,
// of scale * (g[b] + g2[b])
void launch_msite_chain(cudaStream_t s, const double *g, double *out, int na, int B, double alpha,
                        double scale, double sign, int accumulate, const double *g2 = nullptr,
                        unsigned *status = nullptr);

// ---- Lennard-Jones O-O (k_pairs.cu) ----
// r: [B][na][3] box units; list over oxygen points (shared if pl.nconf == 1)
void launch_lj(cudaStream_t s, const double *r, int na, int B, const PairList &pl, double sigsq,
               double rcutsq, const double *box, double dscale, double *out, double *acc);

// ---- TEM-switched correction (k_pairs.cu) ----
void launch_tem(cudaStream_t s, const double *rs, const double *q, int na, int B,
                const PairList &pl, double sig, const double *box, double *g, double *acc);

// ---- centroid of B configurations: rc = (sum_b r_b) / B, sequential in b ----
void launch_centroid(cudaStream_t s, const double *r, double *rc, int na, int B);

// ---- per-molecule terms (k_modes.cu) ----
// model: 0 intra_harmonic, 1 intra_spcfw, 2 intra_morse_harm
void launch_intra(cudaStream_t s, const double *r, double *out, int na, int B, int model,
                  const gb_params &P, double *acc, int accumulate, unsigned *status);
void launch_virial_ke(cudaStream_t s, const double *r, const double *dvdr, const double *dvdr2,
                      int na, int nb, double *acc);
// thermostat kicks and Berendsen shift inside evolve_pi (k_therm.cu)
void launch_prl(cudaStream_t s, double *p, const double *mass, const double *g, int na, int nb, double c1, double c2,
                double betan);
void launch_kinetic(cudaStream_t s, const double *p, const double *mass, int na, int nb, double *out);
void launch_prg_scale(cudaStream_t s, double *p, int na, int nb, const double *kt, double c, double ktav, double ndof,
                      double snfm1, double ranno, int dev_draws);
// device random stream (Philox4x32-10): kicks numbered by the device counter *ctr
void launch_prl_dev(cudaStream_t s, double *p, const double *mass, int na, int nb, double c1, double c2, double betan,
                    const unsigned long long *ctr, unsigned long long seed);
void launch_prg_draw(cudaStream_t s, long long ndof, const unsigned long long *ctr, unsigned long long seed,
                     double *aux);
void launch_ctr_next(cudaStream_t s, unsigned long long *ctr);
void launch_baro_shift(cudaStream_t s, double *r, double *rnm, int na, int nb, const double sm1[3]);
// md_eq's output-step estimators (k_est.cu): acc[14] sums, optional rcm / mdip [nm][3]
void launch_estimators(cudaStream_t s, const double *r, const double *p, const double *dvdr, const double *dvdr2,
                       const double *mass, const double *z, int na, int nb, double alpha, double *acc, double *rcm,
                       double *mdip);

// ---- normal modes (k_modes.cu) ----
void launch_realft(cudaStream_t s, const double *in, double *out, int m, int n, int mode,
                   const double *tw);
void launch_rotate(cudaStream_t s, double *p, double *r, const double *monod, int na, int nb);
void launch_axpy(cudaStream_t s, double *y, const double *x, double a, long long n);
void launch_copy(cudaStream_t s, double *dst, const double *src, long long n);
void launch_ring_contract(cudaStream_t s, const double *rnm, double *rb, int na, int nb, int nbc,
                          const double *tw_c);
// dvdr (bead rep) = HC2R_nb( expand(fb1) + expand(fb2) ) [+ bead-rep extras], then
// p -= halfdt * dvdr when p != nullptr; mixed: the expansion dot products in FP32
void launch_expand_forces(cudaStream_t s, double *dvdr, const double *fb1, int nbc1,
                          const double *tw_c1, const double *fb2, int nbc2, const double *tw_c2,
                          const double *e1, const double *e2, const double *e3, double *p,
                          double halfdt, int na, int nb, const double *tw_nb, bool mixed, unsigned *status);
void launch_fused_mts(cudaStream_t s, gb_context *c, double dt, int *used);
