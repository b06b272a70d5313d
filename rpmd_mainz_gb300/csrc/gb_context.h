// gb_context.h -- device context of one ring-polymer trajectory.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/gbrpmd.h"
#include "gb_kvec.h"
#include "gb_rng.h"

// One pair list: for each of `nconf` configurations and each of `npt` points,
// up to `cap` partner indices; the pair (i, j) is stored once, in the list of
// i when (i < j) == ((i + j) odd), which halves and balances the lists.
struct PairList {
  int nconf = 0, npt = 0, cap = 0;
  int *count = nullptr;  // [nconf][npt]
  int *idx = nullptr;    // [nconf][npt][cap]
  size_t bytes = 0;
  int i16 = 0;           // entries are unsigned short (npt <= 65535): idx is read as that type
  // entries are cell-order slots of the last rebuild, bit 15 set for a pair of
  // the same molecule (i16 lists of at most 32767 points; CellSort::fxs holds
  // the positions in slot order)
  int slots = 0;
};

// Which accumulator slots the last evaluation filled and with how many
// configurations, so that the bead-averaged energies can be formed.
// A pair list kept at cut-off + skin and rebuilt only when some point has moved
// more than skin/2 since its last rebuild (the decision is taken on the device);
// every use filters it into the exact list of pairs within the cut-off.
// cell sort of a superset build (k_pairs.cu): on when list_cell_grid finds a
// stencil that covers a small enough share of the box
struct CellSort {
  bool on = false;
  int nc[3] = {0, 0, 0}, R = 1;
  signed char reach[13 * 13] = {};  // stencil rows: largest |ox| within the cut-off, -1: none
  int *ccount = nullptr;         // [nconf][ncell], zero between steps
  int *cstart = nullptr;         // [nconf][ncell + 1]
  int *cellid = nullptr, *crank = nullptr, *sidx = nullptr;  // [nconf][npt]
  float4 *spos = nullptr;        // [nconf][npt]
  unsigned *ticket = nullptr;    // [2]: blocks done in the count kernel, a point moved
  size_t cell_bytes = 0, pt_bytes = 0;
  // slot order (PairList::slots): each point's cell-order slot at the last
  // rebuild and the fixed-point coordinates in that order, kept every step
  int *slot_of = nullptr;        // [nconf][npt]
  int4 *fxs = nullptr;           // [nconf][npt]
};

struct SkinList {
  PairList pl;                   // superset: pairs within cut-off + skin at the last rebuild
  CellSort cells;
  size_t idx_bytes = 0, cnt_bytes = 0;
  double *ref = nullptr;         // [nconf][npt][3] positions at the last rebuild
  size_t ref_bytes = 0;
  unsigned *flag = nullptr;      // device word: nonzero = rebuild at this use
  unsigned *rebuilds = nullptr;  // device counter of rebuilds
  bool valid = false;            // storage and key match the last use
  int nconf = 0, npt = 0, unit = 0, excl = 0, full = 0;
  long long pstride = 0, cstride = 0;
  double cutsq = 0.0, skin = 0.0, box[3] = {0, 0, 0};
  bool want16 = false;           // unsigned short entries asked for (used with the cell-sorted build)
  double extra = 0.0;            // margin added to cut-off + skin (a shared list's bead spread, twice)
  bool shared = false;           // built on the centroids of several configurations (ListSpread)
};
enum { LIST_EW = 0, LIST_LJ = 1, LIST_TEM = 2, LIST_N = 3 };

struct EnergyPlan {
  int B_ew = 0, B_tem = 0, B_lj = 0, B_ew2 = 0, B_tem2 = 0, B_lj2 = 0, B_int = 0;
  int evolve = 0, mts = 1;
};

struct gb_context {
  int na = 0, nb = 0, nm = 0;
  EnergyPlan plan;
  double qq = 0.0;  // sum of squared charges (Ewald self term)
  double last_beta = 1.0;  // beta of the last evolve_pi (virial kinetic energy)
  int generic_mts = 0;     // 1: run the MTS block as separate kernels (GBRPMD_GENERIC_MTS=1)
  cudaStream_t stream = nullptr;
  int device = 0;
  gb_params P{};  // parameters in force for this context (copied at each call)
  int own_params = 0;  // 1: P was set for this context (gbrpmd_ctx_set_params) and stays

  // trajectory state, layout r(3,na,nb)
  double *p = nullptr, *r = nullptr, *dvdr = nullptr, *dvdr2 = nullptr;
  double *rst = nullptr;   // bead positions scratch (swapped with r)
  double *rnm = nullptr;   // normal-mode positions
  double *mass = nullptr, *z = nullptr;
  double box[3] = {0, 0, 0};

  // force scratch
  double *f_a = nullptr, *f_b = nullptr, *f_c = nullptr;  // bead-rep term forces [nb][na][3]
  double *rb1 = nullptr, *fb1 = nullptr;  // contracted Ewald configurations and forces
  bool rb1_ready = false, rb2_ready = false;  // rb1 / rb2 written by the fused MTS kernel of this step
  double *rb2 = nullptr, *fb2 = nullptr;  // contracted LJ configurations and forces
  double *fb3 = nullptr;                  // contracted TEM forces
  double *g = nullptr;     // unit-box gradient scratch [nb][na][3]
  double *rs = nullptr;    // site positions scratch [nb][na][3]
  float4 *rs32 = nullptr;  // FP32 fractional coordinates for list prefilters [nb][na]
  float4 *lo32 = nullptr;  // their FP32 remainders (mixed precision) [nb][na]
  int4 *fx32 = nullptr;    // fixed-point fractional coordinates (2^-32) and charge bits (mixed real space) [nb][na]
  float4 *hi32 = nullptr;  // bead oxygen coordinates for the FP32 LJ kernel [nb][nm]
  float4 *olo32 = nullptr; // and their remainders [nb][nm]
  // the LJ term of evolve_pi runs beside the Ewald term on aux_stream (forked
  // from and joined to the step's stream) with its own list and frac buffers
  cudaStream_t aux_stream = nullptr;
  cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
  PairList pl_lj;
  size_t pl_lj_idx_bytes = 0, pl_lj_cnt_bytes = 0;
  float4 *rs32_lj = nullptr;  // [nb][nm]
  // the mixed Ewald term runs its k-space kernels on aux2_stream beside the
  // real-space kernel, which writes its gradients into g2
  cudaStream_t aux2_stream = nullptr;
  cudaEvent_t fork2_ev = nullptr, join2_ev = nullptr;
  double *g2 = nullptr;
  double *rc = nullptr;    // centroid scratch [na][3]
  // mixed real space of several configurations: one skin list on the site
  // centroids (superset radius cut-off + skin + twice the bead spread), the
  // configurations' fixed-point coordinates in its slot order, and the
  // spread words (ListSpread)
  double *rcen = nullptr;  // [na][3]
  int4 *fxs_b = nullptr;   // [nb][na]
  float *spread = nullptr; // [4]
  int ew_share = 1;        // GBRPMD_EW_SHARED=0: a list per configuration
  PairList pl;             // exact pair list of the current term (re-sized on demand)
  size_t pl_idx_bytes = 0, pl_cnt_bytes = 0;
  SkinList sl[LIST_N];     // per-term skin lists (Ewald real space, LJ, TEM)
  double list_skin = 0.1;  // skin as a fraction of the cut-off; 0: full rebuild at every use

  // reciprocal space
  int kmax_alloc = -1;           // k tables built for these kmax, rkmax, walpha,
  double k_rkmax = -1.0, k_walpha = -1.0;
  int k_iamcub = -1;              // box kind
  double k_box[3] = {0, 0, 0};    // and (non-cubic tables) box
  int ncol = 0, nkp = 0, ngrp = 0;  // (kx,ky) columns, k pairs (kx,ky,+-m), structure-factor items
  int nk = 0;                   // k vectors of the half space
  KCol *kcol = nullptr;         // [ncol] columns (gb_kvec.h)
  int4 *kgrp = nullptr;         // [ngrp] structure-factor work items
  int4 *kpair = nullptr;        // [nkp] kx, ky, m, kind
  double *kw = nullptr;         // [nkp] weights (4 pi / k^2) exp(-b k^2)
  double *kvir = nullptr;       // [nkp][GB_KVIR] virial factors (gb_kvec.h)
  double2 *ktab = nullptr;      // [nconf][na][3][kmax+1] per-site powers e^{i 2 pi m x}
  double *sk_part = nullptr;    // [nconf][nchunk][nkp][4] chunk partials of P, Q
  double *sk = nullptr;         // [nconf][nkp][8] force tables
  size_t ktab_bytes = 0, sk_part_bytes = 0, sk_bytes = 0;

  // tables and accumulators
  double *tw_nb = nullptr, *tw_c1 = nullptr, *tw_c2 = nullptr;  // twiddles for nb, nbdf1, nbdf2
  int tw_c1_n = 0, tw_c2_n = 0;
  double *monod = nullptr;  // [nb][4][3]
  double monod_dt = -1.0, monod_beta = -1.0;  // monodromy built for these dt, beta,
  int monod_mts = -1, monod_mass_version = -1;  // mts and masses
  double h_mass3[3] = {0, 0, 0};  // host copy of the O, H, H masses (ring_rpmd needs only these)
  int mass_version = 0;           // bumped when uploaded masses differ
  // host copies of the last uploaded masses and charges: a drop-in call that
  // passes the same arrays again copies nothing (a pageable copy would also
  // hold the host until the state copies before it are done)
  std::vector<double> h_mass_all, h_z_all;
  double *acc = nullptr;    // ACC_NSLOT * ACC_STRIDE
  double *est = nullptr;    // estimator sums [16] and per-molecule outputs [2][nm][3] (lazy)

  // thermostat kicks and barostat inside evolve_pi
  int nbaro = 0;                  // evolve_pi's nbaro (md_eq.f90:55-58: 1 for ens = 'NPT')
  RngState *th_rng = nullptr;     // the random stream the PRG / PRL kicks draw from,
  int *th_idum = nullptr;         // set by the caller of each step
  RngState own_rng;               // a stream owned by the context (gbrpmd_ctx_set_rng)
  int own_idum = 0;
  bool has_own_rng = false;
  double *d_gauss = nullptr;      // [3 na nb] gaussians of one PRL kick (device)
  double *h_gauss = nullptr;      // pinned staging of the same
  cudaEvent_t gauss_ev = nullptr; // the staging buffer's last copy
  bool gauss_pending = false;
  double *d_therm = nullptr;      // [4] device scratch (PRG kinetic energy, device draws)
  int rng_mode = GB_RNG_REFERENCE;  // GB_RNG_DEVICE: the kicks draw Philox normals on the device
  unsigned long long rng_seed = 0;
  unsigned long long *d_rngctr = nullptr;  // device kick counter of the device stream
  unsigned *status = nullptr;
  double *h_acc = nullptr;  // pinned host mirror
  unsigned *h_status = nullptr;

  // last step energies (host)
  double e_v = 0, e_vew = 0, e_vlj = 0, e_vint = 0, e_tv = 0;
  double e_vir[9] = {0}, e_vir_lf[9] = {0}, e_vir_hf[9] = {0};
  double vir_lf_in[9] = {0};
  // rigid water with the barostat on a resident context: the virial the
  // barostat reads (evolve_rigid.f90:200, vir = vir_lf + vir_hf + vir, the
  // caller's vir accumulating over the calls; md_eq zeroes it once,
  // md_eq.f90:60) accumulates here over the context's barostat steps
  double rig_vir[9] = {0};
  double acc_L = 0.0;  // box[0] of the last Ewald term launched (its sums are in that unit box)

  int64_t launches = 0;
  std::vector<void *> allocs;
  size_t alloc_bytes = 0;  // bytes of `allocs`
  // the evolve step as a CUDA graph (dev_step): captured on the second step
  // with an unchanged key, replayed while the key holds
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    bool valid = false;
    int seen = 0;            // consecutive plain steps run with this key
    double dt = 0, beta = 0, box[3] = {0, 0, 0};
    gb_params P{};
    int64_t launches = 0;    // kernels per replay
    EnergyPlan plan;
    bool mid = false;        // the replay records mid_ev
  } graph;
  // drop-in calls: an event after the MTS block (r and dvdr2 final), recorded
  // into the step (and its graph), so that their copies back to the host run on
  // copy_stream while the low-frequency forces still compute
  int want_mid = 0;
  bool mid_recorded = false;
  cudaEvent_t mid_ev = nullptr;
  cudaStream_t copy_stream = nullptr;
  int use_graphs = 1;        // GBRPMD_GRAPHS=0 turns replay off
  int list_cells = 1;        // GBRPMD_LIST_CELLS=0: all-pairs superset builds only
  int use_branches = 1;      // GBRPMD_BRANCHES=0: the LJ and k-space kernels stay on the step's stream
  // launch shapes chosen by gbrpmd_ctx_autotune (tune.cpp); results depend on
  // them only through the order of floating-point sums
  struct Tune {
    int ew_np = 16;   // lanes per site, FP32 real-space Ewald (8, 16, 32)
    int lj_np = 4;    // lanes per oxygen, FP32 LJ (2, 4, 8)
    int mts_mpb = 0;  // molecules per block of the MTS kernel (0: one wave over the SMs)
    int rf_g = 8;     // column shares (warps) per block, FP32 k-space force kernel (8, 16)
    int rf_ns = 1;    // sites per lane, FP32 k-space force kernel (1, 2)
    int rf_ks = 1;    // k-pair ranges (blocks per site tile), FP32 k-space force kernel (1..4)
    int done = 0;
  } tune;

  // optional per-region CUDA-event timing (gbrpmd_ctx_set_profiling)
  int prof = 0;
  struct Mark {
    int region;
    cudaEvent_t a, b;
    double units;  // work units of this launch (pairs, k*sites, molecule-beads ...)
  };
  std::vector<Mark> marks;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_next = 0;
  int *d_count = nullptr;  // device scratch for pair counts (profiling only)
  unsigned long long *d_npair = nullptr;  // in-cut pairs counted by the real-space kernel (profiling only)
  // watched kernel (gbrpmd_ctx_watch_region): events around one region's launch
  int watch = -1;
  cudaEvent_t watch_ev[2] = {nullptr, nullptr};
  bool watch_seen = false;
};

// profiled regions
enum ProfRegion : int {
  PR_MTS = 0,        // multiple-time-step block (kicks, transforms, rotation, intra, virial_ke)
  PR_LIST = 1,       // pair-list builds
  PR_EW_REAL = 2,    // real-space Ewald pairs (units: in-cut pairs)
  PR_RECIP_SK = 3,   // structure factors (units: k vectors x sites)
  PR_RECIP_W = 4,    // reduction / weights
  PR_RECIP_F = 5,    // reciprocal forces (units: k vectors x sites)
  PR_LJ = 6,         // Lennard-Jones pairs (units: list pairs x beads)
  PR_TEM = 7,        // TEM correction pairs
  PR_EXPAND = 8,     // contraction, force expansion, final kick
  PR_MSITE = 9,      // M-site substitution and chain rule
  PR_RATTLE = 10,    // rigid substeps and RATTLE
  PR_NREGION = 11
};
void prof_begin(gb_context *c, int region);
void prof_end(gb_context *c, int region, double units);
// records the watch event (0 before, 1 after) when `region` is watched, on the
// stream its kernel runs on (an event node inside a capture)
int watch_mark(gb_context *c, int region, cudaStream_t s, int which);

// ---- context lifetime and helpers (api.cpp) ----
int ctx_alloc(gb_context *c, int na, int nb);
void ctx_free(gb_context *c);
int ctx_set_error(int code, const std::string &msg);
int ctx_check_cuda(cudaError_t e, const char *what);

// ---- device orchestration (step.cu) ----
int dev_prepare(gb_context *c, double dt, double beta);  // twiddles, monodromy, k lists
int dev_full_forces(gb_context *c);                      // dvdr, dvdr2 from r
int dev_evolve_pi(gb_context *c, double dt, double beta);
// applies a shape the autotuner cached for c's key, if any (tune.cpp)
void tune_apply_cached(gb_context *c);
// a PRG / PRL thermostat kick on the bead momenta (no-op for other thermostats)
int therm_kick(gb_context *c, double dtk, double beta);
// evolve_rig_pi (k_rattle.cu); vir_inout unused on the device
int dev_evolve_rig_pi(gb_context *c, double dt, double beta, double *vir_inout);
// rigid water: no intramolecular potential (main.f90:151-159, iamrigid)
inline bool ctx_rigid(const gb_context *c) { return c->P.apot == 0.0 && c->P.bpot == 0.0; }
// one step of the context's integrator: evolve_rig_pi for rigid water, else evolve_pi
int dev_evolve_step(gb_context *c, double dt, double beta);
// one evolve_pi step, replayed from a captured CUDA graph when it can be
int dev_step(gb_context *c, double dt, double beta);
size_t dev_estimate_bytes(int na, int nb, const gb_params &P);
size_t ctx_device_bytes(const gb_context *c);  // device bytes the context holds now
void dev_graph_reset(gb_context *c);
int dev_forces(gb_context *c, const double *r, int B, double *out, int iopt);  // drop-in `forces`
int dev_collect(gb_context *c, int mode, double dt, double beta);  // sync, read accumulators
// beren_driver (module_barostat.f90:8-26): box on the host, waters of r (and
// the centroid row of rnm, when given) on the device
int beren_driver(gb_context *c, const double vir[9], double tv, const double tvxyz[3], double dt, double *rnm);
