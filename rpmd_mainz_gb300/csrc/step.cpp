// step.cpp -- host orchestration of the device RPMD path.
//
// dev_forces      <- forces      (md_forces.f90:1-110)
// dev_full_forces <- full_forces (md_forces.f90:305-472)
// dev_evolve_pi   <- evolve_pi   (evolve_pi.f90:1-322)
// Every kernel is launched on the context's stream; the energies are summed on
// the device into accumulator slots and turned into the reference's bead-averaged
// energies and virials by dev_collect after one synchronisation.
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#include <algorithm>

#include "gb_common.h"
#include "gb_context.h"
#include "gb_kernels.h"

namespace {

const double PI = 3.141592653589793238462643383279502884;

#define CK(x)                                             \
  do {                                                    \
    cudaError_t e_ = (x);                                 \
    if (e_ != cudaSuccess) return ctx_check_cuda(e_, #x); \
  } while (0)

double *slot(gb_context *c, int s) { return c->acc + (size_t)s * ACC_STRIDE; }

// reports a failed kernel launch (bad configuration, shared-memory limit) at once
int launch_status() {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GB_OK : ctx_check_cuda(e, "kernel launch");
}

std::vector<double> twiddles(int n) {
  std::vector<double> t(2 * (size_t)n);
  for (int m = 0; m < n; ++m) {
    double a = 2.0 * PI * (double)m / (double)n;
    t[m] = std::cos(a);
    t[n + m] = std::sin(a);
  }
  return t;
}

int upload_tw(gb_context *c, double **dst, int n) {
  std::vector<double> t = twiddles(n);
  if (*dst) cudaFree(*dst);
  CK(cudaMalloc(dst, sizeof(double) * t.size()));
  CK(cudaMemcpyAsync(*dst, t.data(), sizeof(double) * t.size(), cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  return GB_OK;
}

// ring_rpmd (md_pathi.f90:190-231) on the host; monod(ic, c, k) at ic + 3*(c + 4*k)
void ring_rpmd_host(const double *mass3, int nb, double dt, double beta, double *monod) {
  const double hbar = 1.0;
  for (int j = 0; j < 3; ++j) {
    monod[j + 3 * (0 + 4 * 0)] = 1.0;
    monod[j + 3 * (1 + 4 * 0)] = 0.0;
    monod[j + 3 * (2 + 4 * 0)] = dt / mass3[j];
    monod[j + 3 * (3 + 4 * 0)] = 1.0;
    if (nb > 1) {
      double betan = beta / (double)nb;
      double twown = 2.0 / (betan * hbar);
      double pibyn = std::acos(-1.0) / (double)nb;
      for (int k = 1; k <= nb / 2; ++k) {
        double wk = twown * std::sin(k * pibyn);
        double wt = wk * dt, wm = wk * mass3[j];
        double cwt = std::cos(wt), swt = std::sin(wt);
        monod[j + 3 * (0 + 4 * k)] = cwt;
        monod[j + 3 * (1 + 4 * k)] = -wm * swt;
        monod[j + 3 * (2 + 4 * k)] = swt / wm;
        monod[j + 3 * (3 + 4 * k)] = cwt;
      }
      for (int k = 1; k <= (nb - 1) / 2; ++k)
        for (int cc = 0; cc < 4; ++cc) monod[j + 3 * (cc + 4 * (nb - k))] = monod[j + 3 * (cc + 4 * k)];
    }
  }
}

// half-space k vectors with the reference's loop-exit membership
// (ewald_cubic.f90:292-520) as (kx, ky) columns and +-kz pairs (gb_kvec.h),
// plus the per-evaluation buffers for up to max(nb, 1) configurations
int build_kvectors(gb_context *c) {
  const int kmax = c->P.kmax;
  if (kmax < 0 || kmax > 4000) return ctx_set_error(GB_E_ARG, "kmax out of range");
  if (recip_sk_smem(kmax) > 227 * 1024 || recip_force_smem(kmax) > 227 * 1024)
    return ctx_set_error(GB_E_UNSUPPORTED, "kmax too large for the reciprocal-space kernels");
  const int cap_col = gb_kcap_col(kmax), cap_kp = gb_kcap_kp(kmax);
  std::vector<KCol> col(cap_col);
  std::vector<int4> kp(cap_kp), grp(cap_kp);
  std::vector<double> kw(cap_kp);
  KTables t;
  const bool cub = c->P.iamcub != 0;
  const int bad = cub ? gb_build_ktables(c->P, recip_group_len(), col.data(), cap_col, kp.data(), kw.data(), cap_kp,
                                         grp.data(), cap_kp, &t)
                      : gb_build_ktables_nc(c->P, c->box, recip_group_len(), col.data(), cap_col, kp.data(), kw.data(),
                                            cap_kp, grp.data(), cap_kp, &t);
  if (bad) return ctx_set_error(GB_E_ARG, "k-vector table capacity exceeded");
  for (void *p : {(void *)c->kcol, (void *)c->kgrp, (void *)c->kpair, (void *)c->kw, (void *)c->kvir,
                  (void *)c->ktab, (void *)c->sk_part, (void *)c->sk})
    if (p) cudaFree(p);
  c->kcol = nullptr;
  c->kgrp = c->kpair = nullptr;
  c->kw = c->kvir = c->sk_part = c->sk = nullptr;
  c->ktab = nullptr;
  c->ncol = t.ncol;
  c->nkp = t.nkp;
  c->ngrp = t.ngrp;
  c->nk = t.nk;
  const int nc = std::max(c->nb, 1);
  const int nchunk = (c->na + recip_sk_chunk() - 1) / recip_sk_chunk();
  c->ktab_bytes = sizeof(double2) * 3 * (size_t)(kmax + 1) * c->na * nc;
  c->sk_part_bytes = sizeof(double) * 4 * (size_t)std::max(t.nkp, 1) * nchunk * nc;
  c->sk_bytes = sizeof(double) * 8 * (size_t)std::max(t.nkp, 1) * nc;
  CK(cudaMalloc(&c->kcol, sizeof(KCol) * std::max(t.ncol, 1)));
  CK(cudaMalloc(&c->kgrp, sizeof(int4) * std::max(t.ngrp, 1)));
  CK(cudaMalloc(&c->kpair, sizeof(int4) * std::max(t.nkp, 1)));
  CK(cudaMalloc(&c->kw, sizeof(double) * std::max(t.nkp, 1)));
  CK(cudaMalloc(&c->kvir, sizeof(double) * GB_KVIR * std::max(t.nkp, 1)));
  std::vector<double> kvir(GB_KVIR * (size_t)std::max(t.nkp, 1));
  if (cub) gb_kvir_table(kp.data(), t.nkp, c->P.walpha, kvir.data());
  else gb_kvir_table_nc(kp.data(), t.nkp, c->P.walpha, c->box, kvir.data());
  CK(cudaMalloc(&c->ktab, c->ktab_bytes));
  CK(cudaMalloc(&c->sk_part, c->sk_part_bytes));
  CK(cudaMalloc(&c->sk, c->sk_bytes));
  // set-up copies go on the context's (non-blocking) stream and complete before
  // return: a plain cudaMemcpy from pageable memory may return before its DMA
  // lands and is not ordered with that stream's kernels
  CK(cudaMemcpyAsync(c->kcol, col.data(), sizeof(KCol) * t.ncol, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->kgrp, grp.data(), sizeof(int4) * t.ngrp, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->kpair, kp.data(), sizeof(int4) * t.nkp, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->kw, kw.data(), sizeof(double) * t.nkp, cudaMemcpyHostToDevice, c->stream));
  CK(cudaMemcpyAsync(c->kvir, kvir.data(), sizeof(double) * GB_KVIR * t.nkp, cudaMemcpyHostToDevice, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  recip_set_attributes();
  c->kmax_alloc = kmax;
  c->k_rkmax = c->P.rkmax;
  c->k_walpha = c->P.walpha;
  c->k_iamcub = c->P.iamcub;
  for (int d = 0; d < 3; ++d) c->k_box[d] = c->box[d];
  return GB_OK;
}

// pair-list storage of at least nconf x npt x cap entries
int ensure_list(gb_context *c, int nconf, int npt, int cap) {
  size_t need_idx = sizeof(int) * (size_t)nconf * npt * cap;
  size_t need_cnt = sizeof(int) * (size_t)nconf * npt;
  if (need_idx > c->pl_idx_bytes) {
    if (c->pl.idx) cudaFree(c->pl.idx);
    c->pl.idx = nullptr;
    CK(cudaMalloc(&c->pl.idx, need_idx));
    c->pl_idx_bytes = need_idx;
  }
  if (need_cnt > c->pl_cnt_bytes) {
    if (c->pl.count) cudaFree(c->pl.count);
    c->pl.count = nullptr;
    CK(cudaMalloc(&c->pl.count, need_cnt));
    c->pl_cnt_bytes = need_cnt;
  }
  c->pl.nconf = nconf;
  c->pl.npt = npt;
  c->pl.cap = cap;
  return GB_OK;
}

// partners expected within rc for npt points in volume vol, doubled plus margin
int list_cap(int npt, double rc, double vol) {
  double full = (double)npt * (4.0 / 3.0) * PI * rc * rc * rc / vol;
  int cap = (int)(1.1 * full) + 48;
  cap = std::min(cap, std::max(npt, 1));
  return (cap + 7) & ~7;  // rows of whole 16-byte groups (vector loads of the entries)
}

// c->pl = every pair within g.rcutsq (rounded as the reference rounds it) for
// nconf configurations of g, through skin list `which`: its superset at
// cut-off + skin is rebuilt on the device only when a point has moved by more
// than skin/2 since the last rebuild, then filtered into the exact list.
// Returns the number of launches through *nl.
// With superset = true the filter is skipped and *use points at the skin list
// itself (a consumer that tests the cut-off on its own); else *use = &c->pl.
// fx (optional) receives the points' fixed-point coordinates every step
// (frac_point); with want16 the superset stores unsigned short entries when the
// cell-sorted build is used and the points number at most 65535.
// shared (superset use only): the list is built on g, the centroids of
// shared->B configurations (computed here from shared->r into g.pos, every
// step), with extra = twice the largest spread margin added to its radius;
// the build takes the radius the device chose (ListSpread); fx is then not
// written (the caller writes the configurations' coordinates in slot order).
struct SharedList {
  ListSpread sp;
  const double *r = nullptr;
  int B = 0;
  double *cen = nullptr;
};

int make_list(gb_context *c, int which, const PairGeom &g, int nconf, double cut, double vol, int *nl,
              float4 *lo = nullptr, const double *q = nullptr, bool superset = false, PairList **use = nullptr,
              int4 *fx = nullptr, bool want16 = false, const SharedList *shared = nullptr, double extra = 0.0) {
  if (use) *use = &c->pl;
  int st = ensure_list(c, nconf, g.npt, list_cap(g.npt, cut, vol));
  if (st) return st;
  if (c->list_skin <= 0.0) {
    launch_frac32(c->stream, g, nconf, c->rs32, lo, q, fx);
    launch_build_list(c->stream, g, nconf, c->rs32, c->pl, c->status);
    *nl = 2;
    return GB_OK;
  }
  SkinList &S = c->sl[which];
  const double skin = c->list_skin * cut, scut = cut + skin + extra;
  bool same = S.valid && S.nconf == nconf && S.npt == g.npt && S.unit == g.unit && S.excl == g.excl_mol &&
              S.full == g.full &&
              S.pstride == g.pstride && S.cstride == g.cstride && S.cutsq == g.rcutsq && S.skin == skin &&
              S.want16 == want16 && S.extra == extra && S.shared == (shared != nullptr);
  for (int d = 0; d < 3; ++d) same = same && S.box[d] == g.box[d];
  if (!same) {
    S.valid = false;
    const int cap = list_cap(g.npt, scut, vol);
    const size_t need_idx = sizeof(int) * (size_t)nconf * g.npt * cap;
    const size_t need_cnt = sizeof(int) * (size_t)nconf * g.npt;
    const size_t need_ref = sizeof(double) * 3 * (size_t)nconf * g.npt;
    if (need_idx > S.idx_bytes) {
      if (S.pl.idx) cudaFree(S.pl.idx);
      S.pl.idx = nullptr;
      S.idx_bytes = 0;
      CK(cudaMalloc(&S.pl.idx, need_idx));
      S.idx_bytes = need_idx;
    }
    if (need_cnt > S.cnt_bytes) {
      if (S.pl.count) cudaFree(S.pl.count);
      S.pl.count = nullptr;
      S.cnt_bytes = 0;
      CK(cudaMalloc(&S.pl.count, need_cnt));
      S.cnt_bytes = need_cnt;
    }
    if (need_ref > S.ref_bytes) {
      if (S.ref) cudaFree(S.ref);
      S.ref = nullptr;
      S.ref_bytes = 0;
      CK(cudaMalloc(&S.ref, need_ref));
      S.ref_bytes = need_ref;
    }
    if (!S.flag) CK(cudaMalloc(&S.flag, sizeof(unsigned)));
    if (!S.rebuilds) {
      CK(cudaMalloc(&S.rebuilds, sizeof(unsigned)));
      CK(cudaMemsetAsync(S.rebuilds, 0, sizeof(unsigned), c->stream));
    }
    S.pl.nconf = nconf;
    S.pl.npt = g.npt;
    S.pl.cap = cap;
    // cell sort for the rebuilds when a stencil covers a small share of the box
    PairGeom gsc = g;
    gsc.rcutsq = scut * scut;
    CellSort &cs = S.cells;
    cs.on = c->list_cells && list_cell_grid(gsc, cs.nc, &cs.R, cs.reach);
    S.pl.i16 = want16 && cs.on && g.npt <= 65535 ? 1 : 0;
    S.pl.slots = S.pl.i16 && (fx || shared) && !g.excl_mol && g.npt <= 32767 ? 1 : 0;
    if (cs.on) {
      const size_t ncell = (size_t)cs.nc[0] * cs.nc[1] * cs.nc[2];
      const size_t need_cell = sizeof(int) * (size_t)nconf * (2 * ncell + 1);  // counts, then offsets
      const size_t need_pt = (4 * sizeof(int) + sizeof(float4) + sizeof(int4)) * (size_t)nconf * g.npt;
      if (need_cell > cs.cell_bytes) {
        if (cs.ccount) cudaFree(cs.ccount);
        cs.ccount = nullptr;
        cs.cell_bytes = 0;
        CK(cudaMalloc(&cs.ccount, need_cell));
        cs.cell_bytes = need_cell;
      }
      if (need_pt > cs.pt_bytes) {
        if (cs.spos) cudaFree(cs.spos);
        cs.spos = nullptr;
        cs.pt_bytes = 0;
        CK(cudaMalloc(&cs.spos, need_pt));
        cs.pt_bytes = need_pt;
      }
      if (!cs.ticket) CK(cudaMalloc(&cs.ticket, 2 * sizeof(unsigned)));
      cs.cstart = cs.ccount + (size_t)nconf * ncell;
      const size_t np = (size_t)nconf * g.npt;
      int4 *fxs = reinterpret_cast<int4 *>(cs.spos + np);
      cs.fxs = S.pl.slots && fx ? fxs : nullptr;
      cs.cellid = reinterpret_cast<int *>(fxs + np);
      cs.crank = cs.cellid + np;
      cs.sidx = cs.crank + np;
      cs.slot_of = cs.sidx + np;
      // slots of no rebuild yet: the first count writes every point to slot 0,
      // in bounds, and the rebuild that always follows a reconfiguration
      // rewrites them
      CK(cudaMemsetAsync(cs.slot_of, 0, sizeof(int) * np, c->stream));
      CK(cudaMemsetAsync(cs.ccount, 0, need_cell, c->stream));
      CK(cudaMemsetAsync(cs.ticket, 0, 2 * sizeof(unsigned), c->stream));
    }
  }
  // the cell count kernel writes the gate itself
  if (!S.cells.on) CK(cudaMemsetAsync(S.flag, same ? 0 : 1, sizeof(unsigned), c->stream));
  if (shared && nconf != 1) return ctx_set_error(GB_E_ARG, "a shared list has one configuration");
  int n = S.cells.on ? 0 : 1;  // the frac32 launch (else in the cell count)
  if (shared) {  // the centroids of this step (the list's points) and their spread (ListSpread)
    launch_site_centroid(c->stream, shared->r, shared->cen, g.npt, shared->B, shared->sp,
                         S.cells.on ? S.cells.ticket + 1 : S.flag, c->status);
    n += 1;
  }
  if (!S.cells.on) launch_frac32(c->stream, g, nconf, c->rs32, lo, q, shared ? nullptr : fx);
  // rebuild when a point moved by more than skin/2 (a hair less, for rounding)
  const double lim = 0.5 * skin * (1.0 - 1e-9);
  PairGeom gs = g;
  gs.rcutsq = scut * scut;
  if (S.cells.on) {  // skin test and cell counts in one kernel, then the gated sort and build
    cudaError_t e0 = cudaGetLastError();
    if (e0 != cudaSuccess) return ctx_check_cuda(e0, "a launch before the cell count");
    launch_cell_count(c->stream, g, nconf, c->rs32, lo, q, S.cells, S.ref, lim * lim, same ? 1 : 0, S.flag,
                      shared ? nullptr : fx, shared ? shared->sp : ListSpread());
    if ((e0 = cudaGetLastError()) != cudaSuccess) return ctx_check_cuda(e0, "cell count launch");
    launch_build_sorted(c->stream, gs, nconf, c->rs32, S.pl, c->status, S.flag, S.cells, S.ref, S.rebuilds,
                        shared ? nullptr : fx, shared ? shared->sp.w + 2 : nullptr);
    if ((e0 = cudaGetLastError()) != cudaSuccess) return ctx_check_cuda(e0, "cell build launch");
  } else {
    if (same) {
      launch_skin_check(c->stream, g, nconf, S.ref, lim * lim, S.flag);
      n += 1;
    }
    if (shared) {
      launch_spread_update(c->stream, S.flag, shared->sp);
      n += 1;
    }
    launch_build_list(c->stream, gs, nconf, c->rs32, S.pl, c->status, S.flag, shared ? shared->sp.w + 2 : nullptr);
    launch_skin_save(c->stream, g, nconf, S.ref, S.flag, S.rebuilds);
  }
  n += 3;  // cells: count, scatter (+ save), build; else zero, build, save
  if (superset && use) {
    *use = &S.pl;
    // profiling counts in-cut pairs: the exact list is made for the count only
    // (a list of slots is counted by its consumer instead)
    if (c->prof && !S.pl.slots) launch_list_filter(c->stream, g, nconf, c->rs32, S.pl, c->pl, c->status);
  } else {
    launch_list_filter(c->stream, g, nconf, c->rs32, S.pl, c->pl, c->status);
    n += 1;
  }
  S.valid = true;
  S.nconf = nconf;
  S.npt = g.npt;
  S.unit = g.unit;
  S.excl = g.excl_mol;
  S.full = g.full;
  S.pstride = g.pstride;
  S.cstride = g.cstride;
  S.cutsq = g.rcutsq;
  S.skin = skin;
  S.want16 = want16;
  S.extra = extra;
  S.shared = shared != nullptr;
  for (int d = 0; d < 3; ++d) S.box[d] = g.box[d];
  *nl = n;
  return GB_OK;
}

double boxmin(const gb_context *c) { return std::min(c->box[0], std::min(c->box[1], c->box[2])); }
double boxmax(const gb_context *c) { return std::max(c->box[0], std::max(c->box[1], c->box[2])); }

// ---- one force term on B configurations ----

// Ewald sum of B configurations (potenl_opt's M-site substitution and chain
// rule, md_forces.f90:186-213).  Cubic boxes (ewald_cubic.f90:1-76): positions
// scaled to the unit box, energy and gradient scaled back by 1/L and 1/L^2.
// Non-cubic boxes (ewald_nc, ewald_noncubic.f90:1-54): positions, cut-off and
// k vectors in bohr, no scaling; the same pair, structure-factor, weight and
// force kernels run with per-axis factors.
int term_ewald(gb_context *c, const double *r, int B, double *out, double sign, int accumulate, int s) {
  if (c->P.wm > 0.0 || c->P.wh > 0.0) return ctx_set_error(GB_E_UNSUPPORTED, "smeared-charge Ewald is not on the device path");
  const int na = c->na;
  const bool cub = c->P.iamcub != 0;
  const double L = c->box[0], onboxl = 1.0 / L;
  c->acc_L = L;  // the box the accumulated Ewald sums are scaled by (dev_collect)
  const double pscale = cub ? onboxl : 1.0, gscale = cub ? onboxl * onboxl : 1.0;
  prof_begin(c, PR_MSITE);
  launch_msite(c->stream, r, c->rs, na, B, c->P.alpha, pscale, c->g);  // and g = 0
  prof_end(c, PR_MSITE, (double)na * B);
  PairGeom g{};
  g.pos = c->rs;
  g.cstride = 3LL * na;
  g.pstride = 3;
  g.npt = na;
  g.unit = cub ? 1 : 0;
  for (int d = 0; d < 3; ++d) {
    g.box[d] = cub ? 1.0 : c->box[d];
    g.onbox[d] = cub ? 1.0 : 1.0 / c->box[d];
  }
  g.rcutsq = c->P.wrcut * c->P.wrcut;
  g.excl_mol = 0;
  const bool mixed = c->P.precision == GB_PREC_MIXED;
  g.full = mixed ? 1 : 0;  // the FP32 kernel walks full lists
  // mixed: the k-space kernels (low occupancy, and needing only the M-site
  // positions) run on aux2 beside the list upkeep and the real-space kernel,
  // which writes its own gradient buffer; joined before the chain rule
  const bool branch = mixed && !c->prof && c->use_branches && c->aux2_stream;
  int st0;
  if (branch) {
    recip_set_attributes_mx();
    CK(cudaEventRecord(c->fork2_ev, c->stream));
    CK(cudaStreamWaitEvent(c->aux2_stream, c->fork2_ev, 0));
    launch_recip_sk_mx(c->aux2_stream, c, c->rs, c->z, B);
    launch_recip_weights_mx(c->aux2_stream, c, B, slot(c, s));
    if ((st0 = watch_mark(c, PR_RECIP_F, c->aux2_stream, 0))) return st0;
    launch_recip_force_mx(c->aux2_stream, c, B, c->g);
    if ((st0 = watch_mark(c, PR_RECIP_F, c->aux2_stream, 1))) return st0;
    CK(cudaEventRecord(c->join2_ev, c->aux2_stream));
  }
  struct Join2 {  // an error return still joins the branch (a capture needs it)
    gb_context *c;
    bool on;
    ~Join2() {
      if (on) cudaStreamWaitEvent(c->stream, c->join2_ev, 0);
    }
  } join2{c, branch};
  int nl = 0;
  prof_begin(c, PR_LIST);
  PairList *pl = nullptr;  // mixed: the skin list itself, cut-off tested in the FP32 kernel
  const double vol = cub ? 1.0 : c->box[0] * c->box[1] * c->box[2];
  // mixed, several configurations: one list on the site centroids serves them
  // all (a superset whose radius adds twice the beads' largest distance from
  // their centroid, chosen on the device at each rebuild and bounded by dcap;
  // the kernel tests each configuration's own distances)
  bool share = false;
  double extra = 0.0;
  SharedList sh;
  PairGeom gc = g;
  if (mixed && B > 1 && c->ew_share && c->list_skin > 0.0) {
    const double unit = cub ? L : 1.0;                    // bohr per length unit of g
    const double rcu = c->P.wrcut, skinu = c->list_skin * rcu;
    const double dcap = std::max(3.0 / unit, 0.12 * rcu);  // at most 3 bohr, or 12 % of the cut-off, of spread
    extra = 2.0 * dcap;
    gc.pos = c->rcen;
    gc.cstride = 0;
    share = true;
    sh.sp.w = c->spread;
    sh.sp.base = (float)(rcu + skinu);
    sh.sp.dcap = (float)dcap;
    sh.sp.dmin = (float)(0.1 / unit);
    sh.r = c->rs;
    sh.B = B;
    sh.cen = c->rcen;
  }
  int st = share ? make_list(c, LIST_EW, gc, 1, c->P.wrcut, vol, &nl, nullptr, c->z, true, &pl, nullptr, true, &sh,
                             extra)
                 : make_list(c, LIST_EW, g, B, c->P.wrcut, vol, &nl, mixed ? c->lo32 : nullptr,
                             mixed ? c->z : nullptr, mixed, &pl, mixed ? c->fx32 : nullptr, mixed);
  if (st) return st;
  if (share) {  // the configurations' fixed-point coordinates, in the shared list's slot order
    launch_fx_slots(c->stream, g, B, c->z, pl->slots ? c->sl[LIST_EW].cells.slot_of : nullptr, c->fx32,
                    pl->slots ? c->fxs_b : nullptr);
    nl += 1;
  }
  prof_end(c, PR_LIST, (double)na * B);
  c->launches += nl;
  // in-cut pairs, each once (profiling fills c->pl with the exact list, or the
  // real-space kernel counts the entries of a list of slots)
  const bool count_in_kernel = c->prof && mixed && pl->slots;
  double npairs = c->prof && !count_in_kernel ? list_total(c->stream, c->pl) * (mixed ? 0.5 : 1.0) : 0.0;
  unsigned long long *npair_dev = nullptr;
  if (count_in_kernel) {
    if (!c->d_npair) CK(cudaMalloc(&c->d_npair, sizeof(unsigned long long)));
    CK(cudaMemsetAsync(c->d_npair, 0, sizeof(unsigned long long), c->stream));
    npair_dev = c->d_npair;
  }
  const int4 *fxs = mixed && pl->slots ? (share ? c->fxs_b : c->sl[LIST_EW].cells.fxs) : nullptr;
  const double ksites = (double)c->nk * na * B;
  if (branch) {
    if ((st0 = watch_mark(c, PR_EW_REAL, c->stream, 0))) return st0;
    launch_ewald_real_mx(c->stream, c->fx32, fxs, na, B, *pl, c->P.walpha, c->P.wrcut * c->P.wrcut, g.box,
                         c->tune.ew_np, c->g2, slot(c, s), false);
    if ((st0 = watch_mark(c, PR_EW_REAL, c->stream, 1))) return st0;
    join2.on = false;
    CK(cudaStreamWaitEvent(c->stream, c->join2_ev, 0));
    launch_msite_chain(c->stream, c->g, out, na, B, c->P.alpha, gscale, sign, accumulate, c->g2, c->status);
    c->launches += 7;
    return GB_OK;
  }
  if (mixed) {
    recip_set_attributes_mx();
    prof_begin(c, PR_EW_REAL);
    if ((st0 = watch_mark(c, PR_EW_REAL, c->stream, 0))) return st0;
    launch_ewald_real_mx(c->stream, c->fx32, fxs, na, B, *pl, c->P.walpha, c->P.wrcut * c->P.wrcut, g.box,
                         c->tune.ew_np, c->g, slot(c, s), true, npair_dev);
    if ((st0 = watch_mark(c, PR_EW_REAL, c->stream, 1))) return st0;
    prof_end(c, PR_EW_REAL, npairs);
    if (count_in_kernel) {  // profiling only: synchronises, after the region's end event
      unsigned long long h = 0;
      CK(cudaMemcpyAsync(&h, c->d_npair, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
      CK(cudaStreamSynchronize(c->stream));
      if (!c->marks.empty()) c->marks.back().units = 0.5 * (double)h;
    }
    prof_begin(c, PR_RECIP_SK);
    launch_recip_sk_mx(c->stream, c, c->rs, c->z, B);
    prof_end(c, PR_RECIP_SK, ksites);
    prof_begin(c, PR_RECIP_W);
    launch_recip_weights_mx(c->stream, c, B, slot(c, s));
    prof_end(c, PR_RECIP_W, (double)c->nkp * B);
    prof_begin(c, PR_RECIP_F);
    if ((st0 = watch_mark(c, PR_RECIP_F, c->stream, 0))) return st0;
    launch_recip_force_mx(c->stream, c, B, c->g);
    if ((st0 = watch_mark(c, PR_RECIP_F, c->stream, 1))) return st0;
    prof_end(c, PR_RECIP_F, ksites);
  } else {
    prof_begin(c, PR_EW_REAL);
    if ((st0 = watch_mark(c, PR_EW_REAL, c->stream, 0))) return st0;
    launch_ewald_real(c->stream, c->rs, c->z, na, B, c->pl, c->P.walpha, cub ? nullptr : c->box, c->g, slot(c, s));
    if ((st0 = watch_mark(c, PR_EW_REAL, c->stream, 1))) return st0;
    prof_end(c, PR_EW_REAL, npairs);
    prof_begin(c, PR_RECIP_SK);
    launch_recip_sk(c->stream, c, c->rs, c->z, B);
    prof_end(c, PR_RECIP_SK, ksites);
    prof_begin(c, PR_RECIP_W);
    launch_recip_weights(c->stream, c, B, slot(c, s));
    prof_end(c, PR_RECIP_W, (double)c->nkp * B);
    prof_begin(c, PR_RECIP_F);
    if ((st0 = watch_mark(c, PR_RECIP_F, c->stream, 0))) return st0;
    launch_recip_force(c->stream, c, c->rs, c->z, B, c->g);
    if ((st0 = watch_mark(c, PR_RECIP_F, c->stream, 1))) return st0;
    prof_end(c, PR_RECIP_F, ksites);
  }
  prof_begin(c, PR_MSITE);
  launch_msite_chain(c->stream, c->g, out, na, B, c->P.alpha, gscale, sign, accumulate, nullptr, c->status);
  prof_end(c, PR_MSITE, (double)na * B);
  c->launches += 7;
  return GB_OK;
}

int term_lj(gb_context *c, const double *r, int B, double *out, int accumulate, int s) {
  if (c->P.oo_gam != 0.0) return ctx_set_error(GB_E_UNSUPPORTED, "Buckingham O-O is not on the device path");
  const int na = c->na, nm = c->nm;
  if (!accumulate) CK(cudaMemsetAsync(out, 0, sizeof(double) * 3 * (size_t)na * B, c->stream));
  PairGeom g{};
  g.pstride = 9;
  g.npt = nm;
  g.unit = 0;
  for (int d = 0; d < 3; ++d) {
    g.box[d] = c->box[d];
    g.onbox[d] = 1.0 / c->box[d];
  }
  g.excl_mol = 0;
  const double vol = c->box[0] * c->box[1] * c->box[2];
  int nconf;
  double lcut;
  if (B > 3) {  // centroid neighbour list (md_forces.f90:34-53)
    launch_centroid(c->stream, r, c->rc, na, B);
    const double cut = std::min(c->P.rcut, 0.5 * boxmin(c));
    g.pos = c->rc;
    g.cstride = 0;
    g.rcutsq = cut * cut;
    nconf = 1;
    lcut = cut;
    c->launches += 1;
  } else {  // lj_basic / lj_cell: every pair within rcut, bead by bead
    g.pos = r;
    g.cstride = 3LL * na;
    g.rcutsq = c->P.rcut * c->P.rcut;
    nconf = B;
    lcut = c->P.rcut;
  }
  const bool mixed = c->P.precision == GB_PREC_MIXED;
  g.full = mixed ? 1 : 0;
  int nl = 0;
  prof_begin(c, PR_LIST);
  int st = make_list(c, LIST_LJ, g, nconf, lcut, vol, &nl);
  if (st) return st;
  prof_end(c, PR_LIST, (double)nm * nconf);
  c->launches += nl;
  const double npairs =
      c->prof ? list_total(c->stream, c->pl) * (nconf == 1 ? B : 1) * (mixed ? 0.5 : 1.0) : 0.0;
  prof_begin(c, PR_LJ);
  if (mixed) {
    PairGeom go = g;  // the bead oxygens of every configuration, as hi/lo FP32
    go.pos = r;
    go.cstride = 3LL * na;
    launch_frac32(c->stream, go, B, c->hi32, c->olo32);
    if ((st = watch_mark(c, PR_LJ, c->stream, 0))) return st;
    launch_lj_mx(c->stream, c->hi32, c->olo32, na, B, c->pl, c->P.oo_sig * c->P.oo_sig, c->P.rcut * c->P.rcut,
                 c->box, 48.0 * c->P.oo_eps, c->tune.lj_np, out, slot(c, s));
    c->launches += 1;
  } else {
    if ((st = watch_mark(c, PR_LJ, c->stream, 0))) return st;
    launch_lj(c->stream, r, na, B, c->pl, c->P.oo_sig * c->P.oo_sig, c->P.rcut * c->P.rcut, c->box,
              48.0 * c->P.oo_eps, out, slot(c, s));
  }
  if ((st = watch_mark(c, PR_LJ, c->stream, 1))) return st;
  prof_end(c, PR_LJ, npairs);
  c->launches += 1;
  return GB_OK;
}

int term_tem(gb_context *c, const double *r, int B, double *out, double sign, int accumulate, int s) {
  if (c->P.wm > 0.0 || c->P.wh > 0.0) return ctx_set_error(GB_E_UNSUPPORTED, "ewc_correction not yet implemented for smeared charges");
  const int na = c->na;
  const double sig = c->P.sig;
  const double alpha = std::fabs(c->P.alpha - 1.0) > 1e-4 ? c->P.alpha : 1.0;
  const double vol = c->box[0] * c->box[1] * c->box[2];
  PairGeom g{};
  g.npt = na;
  g.unit = 0;
  g.pstride = 3;
  for (int d = 0; d < 3; ++d) {
    g.box[d] = c->box[d];
    g.onbox[d] = 1.0 / c->box[d];
  }
  g.excl_mol = 1;
  launch_msite(c->stream, r, c->rs, na, B, alpha, 1.0);
  int nconf;
  double lcut;
  if (B > 1) {  // centroid list, cut sig + 5 bohr (md_forces.f90:69-89) -> ewc_list_tem
    if (sig > 0.5 * boxmax(c)) return ctx_set_error(GB_E_CUTOFF, "ewc_list : rcut too large");
    double cut = sig + 5.0;
    if (cut > 0.5 * boxmin(c)) cut = std::min(cut, 0.5 * boxmin(c));
    launch_centroid(c->stream, r, c->rc, na, B);
    g.pos = c->rc;
    g.cstride = 0;
    g.rcutsq = cut * cut;
    nconf = 1;
    lcut = cut;
    c->launches += 1;
  } else {  // ewc_basic_tem / ewc_cell_tem on the M-site positions
    if (3.0 * sig > boxmax(c)) {
      if (sig > 0.5 * boxmax(c)) return ctx_set_error(GB_E_CUTOFF, "ewc_basic : rcut too large");
    } else if (sig > 0.5 * boxmin(c)) {
      return ctx_set_error(GB_E_CUTOFF, "ewc_basic : rcut too large");
    }
    g.pos = c->rs;
    g.cstride = 3LL * na;
    g.rcutsq = sig * sig;
    nconf = B;
    lcut = sig;
  }
  CK(cudaMemsetAsync(c->g, 0, sizeof(double) * 3 * (size_t)na * B, c->stream));
  int nl = 0;
  prof_begin(c, PR_LIST);
  int st = make_list(c, LIST_TEM, g, nconf, lcut, vol, &nl);
  if (st) return st;
  prof_end(c, PR_LIST, (double)na * nconf);
  c->launches += nl;
  prof_begin(c, PR_TEM);
  launch_tem(c->stream, c->rs, c->z, na, B, c->pl, sig, c->box, c->g, slot(c, s));
  prof_end(c, PR_TEM, 0.0);
  launch_msite_chain(c->stream, c->g, out, na, B, alpha, 1.0, sign, accumulate, nullptr, c->status);
  c->launches += 3;
  return GB_OK;
}

int intra_model(const gb_params &P) {
  if (P.intra_model == GB_INTRA_SPCFW) return 1;
  if (P.alp == 0.0) return 0;
  return 2;
}

int term_intra(gb_context *c, const double *r, int B, double *out, int accumulate, int s) {
  if (c->P.intra_model != GB_INTRA_SPCFW && c->P.alp != 0.0 && c->P.alpb != 0.0)
    return ctx_set_error(GB_E_UNSUPPORTED, "intra_morse is not on the device path");
  launch_intra(c->stream, r, out, c->na, B, intra_model(c->P), c->P, slot(c, s), accumulate, c->status);
  c->launches += 1;
  return GB_OK;
}

// low-frequency forces of full_forces / evolve_pi: contracted terms from rnm,
// bead-representation terms from r; dvdr = expand + extras, optional kick
int low_frequency(gb_context *c, const double *rnm, const double *r, double *p, double halfdt) {
  const int nb = c->nb, na = c->na;
  const int nbdf1 = c->P.nbdf1, nbdf2 = c->P.nbdf2;
  const double sig = c->P.sig;
  const bool con1 = nb > 1 && nbdf1 > 0, con2 = nb > 1 && nbdf2 > 0;
  int st;
  struct Clear {  // the fused kernel's rings serve this evaluation only
    gb_context *c;
    ~Clear() { c->rb1_ready = c->rb2_ready = false; }
  } clear{c};
  // The LJ term on the contracted ring needs neither the Ewald term's inputs
  // nor its buffers: it runs on the aux stream (forked here, joined before the
  // expansion), with the context's LJ list and frac buffers swapped in, so that
  // its kernels fill the SMs the k-space kernels leave idle.  Not while
  // profiling (regions are timed on the step's stream).
  const bool branch = con2 && !c->prof && c->use_branches && c->aux_stream;
  bool joined = true;
  struct Join {  // an error return still joins the branch (a capture needs it)
    gb_context *c;
    bool *joined;
    ~Join() {
      if (!*joined) cudaStreamWaitEvent(c->stream, c->join_ev, 0);
    }
  } join{c, &joined};
  if (branch) {
    if ((nbdf2 - 1) % 2 != 0) return ctx_set_error(GB_E_CONTRACT, "* Beadiabatic factor must be ODD");
    CK(cudaEventRecord(c->fork_ev, c->stream));
    CK(cudaStreamWaitEvent(c->aux_stream, c->fork_ev, 0));
    struct Swap {  // the LJ branch's stream and buffers, restored on every exit
      gb_context *c;
      explicit Swap(gb_context *cc) : c(cc) { flip(); }
      ~Swap() { flip(); }
      void flip() {
        std::swap(c->stream, c->aux_stream);
        std::swap(c->pl, c->pl_lj);
        std::swap(c->pl_idx_bytes, c->pl_lj_idx_bytes);
        std::swap(c->pl_cnt_bytes, c->pl_lj_cnt_bytes);
        std::swap(c->rs32, c->rs32_lj);
      }
    };
    {
      Swap sw(c);
      if (!c->rb2_ready) launch_ring_contract(c->stream, rnm, c->rb2, na, nb, nbdf2, c->tw_c2);
      if ((st = term_lj(c, c->rb2, nbdf2, c->fb2, 0, ACC_LJ))) return st;
    }
    CK(cudaEventRecord(c->join_ev, c->aux_stream));
    joined = false;
    c->plan.B_lj = nbdf2;
    if (!c->rb2_ready) c->launches += 1;
  }
  if (con1) {
    if ((nbdf1 - 1) % 2 != 0) return ctx_set_error(GB_E_CONTRACT, "* Beadiabatic factor must be ODD");
    if (!c->rb1_ready) launch_ring_contract(c->stream, rnm, c->rb1, na, nb, nbdf1, c->tw_c1);
    if ((st = term_ewald(c, c->rb1, nbdf1, c->fb1, 1.0, 0, ACC_EW))) return st;
    c->plan.B_ew = nbdf1;
    if (sig > 0.0) {
      if ((st = term_tem(c, c->rb1, nbdf1, c->fb1, -1.0, 1, ACC_TEM))) return st;
      c->plan.B_tem = nbdf1;
    }
    if (!c->rb1_ready) c->launches += 1;
  }
  if (con2 && !branch) {
    if ((nbdf2 - 1) % 2 != 0) return ctx_set_error(GB_E_CONTRACT, "* Beadiabatic factor must be ODD");
    if (!c->rb2_ready) launch_ring_contract(c->stream, rnm, c->rb2, na, nb, nbdf2, c->tw_c2);
    if ((st = term_lj(c, c->rb2, nbdf2, c->fb2, 0, ACC_LJ))) return st;
    c->plan.B_lj = nbdf2;
    if (!c->rb2_ready) c->launches += 1;
  }
  const double *e1 = nullptr, *e2 = nullptr, *e3 = nullptr;
  if (nb == 1 || nbdf1 <= 0) {
    if ((st = term_ewald(c, r, nb, c->f_a, 1.0, 0, ACC_EW2))) return st;
    c->plan.B_ew2 = nb;
    e1 = c->f_a;
  } else if (sig > 0.0) {
    if ((st = term_tem(c, r, nb, c->f_b, 1.0, 0, ACC_TEM2))) return st;
    c->plan.B_tem2 = nb;
    e2 = c->f_b;
  }
  if (nb == 1 || nbdf2 <= 0) {
    if ((st = term_lj(c, r, nb, c->f_c, 0, ACC_LJ2))) return st;
    c->plan.B_lj2 = nb;
    e3 = c->f_c;
  }
  if (!joined) {
    joined = true;
    CK(cudaStreamWaitEvent(c->stream, c->join_ev, 0));
  }
  prof_begin(c, PR_EXPAND);
  launch_expand_forces(c->stream, c->dvdr, con1 ? c->fb1 : nullptr, nbdf1, c->tw_c1,
                       con2 ? c->fb2 : nullptr, nbdf2, c->tw_c2, e1, e2, e3, p, halfdt, na, nb,
                       c->tw_nb, c->P.precision == GB_PREC_MIXED, c->status);
  prof_end(c, PR_EXPAND, 3.0 * na * nb);
  c->launches += 1;
  return GB_OK;
}

}  // namespace

int dev_prepare(gb_context *c, double dt, double beta) {
  int st;
  if (!c->tw_nb && (st = upload_tw(c, &c->tw_nb, c->nb))) return st;
  if (c->P.nbdf1 > 0 && c->tw_c1_n != c->P.nbdf1) {
    if (c->P.nbdf1 > 63 || c->P.nbdf1 > c->nb) return ctx_set_error(GB_E_ARG, "RP contraction beads must not exceed nb (and 63 on the device)");
    if ((st = upload_tw(c, &c->tw_c1, c->P.nbdf1))) return st;
    c->tw_c1_n = c->P.nbdf1;
  }
  if (c->P.nbdf2 > 0 && c->tw_c2_n != c->P.nbdf2) {
    if (c->P.nbdf2 > 63 || c->P.nbdf2 > c->nb) return ctx_set_error(GB_E_ARG, "RP contraction beads must not exceed nb (and 63 on the device)");
    if ((st = upload_tw(c, &c->tw_c2, c->P.nbdf2))) return st;
    c->tw_c2_n = c->P.nbdf2;
  }
  // the non-cubic tables depend on the box as well (k vectors in bohr^-1)
  const bool kbox = !c->P.iamcub && (c->k_box[0] != c->box[0] || c->k_box[1] != c->box[1] || c->k_box[2] != c->box[2]);
  if (c->kmax_alloc != c->P.kmax || c->k_rkmax != c->P.rkmax || c->k_walpha != c->P.walpha ||
      c->k_iamcub != c->P.iamcub || kbox) {
    if ((st = build_kvectors(c))) return st;
  }
  if (dt > 0.0 && (dt != c->monod_dt || beta != c->monod_beta || c->P.mts != c->monod_mts ||
                   c->mass_version != c->monod_mass_version)) {
    std::vector<double> monod(12 * (size_t)c->nb);
    ring_rpmd_host(c->h_mass3, c->nb, dt / (double)c->P.mts, beta, monod.data());
    CK(cudaMemcpyAsync(c->monod, monod.data(), sizeof(double) * monod.size(), cudaMemcpyHostToDevice, c->stream));
    CK(cudaStreamSynchronize(c->stream));  // monod is a local vector
    c->monod_dt = dt;
    c->monod_beta = beta;
    c->monod_mts = c->P.mts;
    c->monod_mass_version = c->mass_version;
  }
  return GB_OK;
}

int dev_forces(gb_context *c, const double *r, int B, double *out, int iopt) {
  dev_graph_reset(c);  // other list configurations: a captured step would be stale
  int st;
  if ((st = dev_prepare(c, 0.0, 0.0))) return st;
  c->plan = EnergyPlan();
  CK(cudaMemsetAsync(c->acc, 0, sizeof(double) * ACC_NSLOT * ACC_STRIDE, c->stream));
  CK(cudaMemsetAsync(out, 0, sizeof(double) * 3 * (size_t)c->na * B, c->stream));
  if (iopt == 5) {
    if ((st = term_tem(c, r, B, out, 1.0, 1, ACC_TEM2))) return st;
    c->plan.B_tem2 = B;
    return launch_status();
  }
  if (iopt < 0 || iopt > 4) return ctx_set_error(GB_E_UNSUPPORTED, "iopt not on the device path");
  if (iopt <= 2) {
    if ((st = term_ewald(c, r, B, out, 1.0, 1, ACC_EW2))) return st;
    c->plan.B_ew2 = B;
  }
  if (iopt == 0 || iopt == 1 || iopt == 3) {
    if ((st = term_lj(c, r, B, out, 1, ACC_LJ2))) return st;
    c->plan.B_lj2 = B;
  }
  if (iopt == 0 || iopt == 4) {
    if ((st = term_intra(c, r, B, out, 1, ACC_INT))) return st;
    c->plan.B_int = B;
  }
  return launch_status();
}

int dev_full_forces(gb_context *c) {
  dev_graph_reset(c);  // other list configurations: a captured step would be stale
  int st;
  if ((st = dev_prepare(c, 0.0, 0.0))) return st;
  c->plan = EnergyPlan();
  const int nb = c->nb, na = c->na;
  CK(cudaMemsetAsync(c->acc, 0, sizeof(double) * ACC_NSLOT * ACC_STRIDE, c->stream));
  if ((st = term_intra(c, c->r, nb, c->dvdr2, 0, ACC_INT))) return st;
  c->plan.B_int = nb;
  const bool contract = nb > 1 && (c->P.nbdf1 > 0 || c->P.nbdf2 > 0);
  if (contract) {
    launch_realft(c->stream, c->r, c->rnm, 3 * na, nb, +1, c->tw_nb);
    c->launches += 1;
  }
  if ((st = low_frequency(c, c->rnm, c->r, nullptr, 0.0))) return st;
  return launch_status();
}

// One thermostat kick of evolve_pi (evolve_pi.f90:72-80, 281-290) on the bead
// momenta: parinello_therm (PRG, global rescaling) or parinello_therm_loc (PRL,
// local Langevin), drawing the reference's gaussian stream c->th_rng / th_idum
// on the host in the reference's order.  dtk: the time step the reference
// passes (halfdt for PRG, dt for PRL in evolve_pi; halfdt for both in
// evolve_rig_pi).
int therm_kick(gb_context *c, double dtk, double beta) {
  const gb_params &P = c->P;
  if (P.therm != GB_THERM_PRG && P.therm != GB_THERM_PRL) return GB_OK;
  const int na = c->na, nb = c->nb;
  const size_t N = 3 * (size_t)na * nb;
  const double betan = beta / (double)nb;
  if (c->rng_mode == GB_RNG_DEVICE) {  // device stream: no host work, graph-capturable
    if (P.therm == GB_THERM_PRL) {
      const double gamma = 1.0 / (2.0 * P.ttau);
      const double c1 = std::exp(-0.5 * gamma * dtk), c2 = std::sqrt(1.0 - c1 * c1);
      launch_prl_dev(c->stream, c->p, c->mass, na, nb, c1, c2, betan, c->d_rngctr, c->rng_seed);
      c->launches += 1;
    } else {
      const long long ndof = (long long)(3 * na * (double)nb - P.nctot - 3);
      CK(cudaMemsetAsync(c->d_therm, 0, sizeof(double) * 2, c->stream));
      launch_kinetic(c->stream, c->p, c->mass, na, nb, c->d_therm);
      launch_prg_draw(c->stream, ndof, c->d_rngctr, c->rng_seed, c->d_therm);
      launch_prg_scale(c->stream, c->p, na, nb, c->d_therm, std::exp(-dtk / P.ttau), (double)ndof / (2.0 * betan),
                       (double)ndof, 0.0, 0.0, 1);
      c->launches += 3;
    }
    launch_ctr_next(c->stream, c->d_rngctr);
    c->launches += 1;
    return GB_OK;
  }
  if (!c->th_rng || !c->th_idum)
    return ctx_set_error(GB_E_ARG, "PRG/PRL thermostat: no random stream (gbrpmd_ctx_set_rng)");
  RngState &g = *c->th_rng;
  int *idum = c->th_idum;
  if (!c->d_therm) CK(cudaMalloc(&c->d_therm, sizeof(double) * 4));
  if (P.therm == GB_THERM_PRL) {  // module_thermostat.f90:56-82
    const double gamma = 1.0 / (2.0 * P.ttau);
    const double c1 = std::exp(-0.5 * gamma * dtk);
    const double c2 = std::sqrt(1.0 - c1 * c1);
    if (!c->d_gauss) {
      CK(cudaMalloc(&c->d_gauss, sizeof(double) * N));
      CK(cudaMallocHost(&c->h_gauss, sizeof(double) * N));
      CK(cudaEventCreateWithFlags(&c->gauss_ev, cudaEventDisableTiming));
    }
    if (c->gauss_pending) CK(cudaEventSynchronize(c->gauss_ev));  // staging buffer free again
    for (size_t i = 0; i < N; ++i) c->h_gauss[i] = rng_gaussian(g, idum, 1.0);
    CK(cudaMemcpyAsync(c->d_gauss, c->h_gauss, sizeof(double) * N, cudaMemcpyHostToDevice, c->stream));
    CK(cudaEventRecord(c->gauss_ev, c->stream));
    c->gauss_pending = true;
    launch_prl(c->stream, c->p, c->mass, c->d_gauss, na, nb, c1, c2, betan);
    c->launches += 1;
    return GB_OK;
  }
  // parinello_therm (module_thermostat.f90:6-54)
  const int ndof = (int)(3 * na * (double)nb - P.nctot - 3);
  (void)rng_gaussian(g, idum, 1.0);  // rt: drawn, not used
  const double ktav = (double)ndof / (2.0 * betan);
  double snfm1 = 0.0;
  for (int i = 1; i <= ndof - 1; ++i) {
    const double ranno = rng_gaussian(g, idum, 1.0);
    snfm1 = snfm1 + ranno * ranno;
  }
  CK(cudaMemsetAsync(c->d_therm, 0, sizeof(double), c->stream));
  launch_kinetic(c->stream, c->p, c->mass, na, nb, c->d_therm);
  const double ranno = rng_gaussian(g, idum, 1.0);
  const double cc = std::exp(-dtk / P.ttau);
  launch_prg_scale(c->stream, c->p, na, nb, c->d_therm, cc, ktav, (double)ndof, snfm1, ranno, 0);
  c->launches += 2;
  return GB_OK;
}

// beren_driver (module_barostat.f90:8-26) on the context's bead positions r
// (and the centroid row of the normal-mode positions rnm, when given): the
// pressure from vir and the virial kinetic energy tv (beren_baro,
// module_barostat.f90:88-129, with pressure, md_pressure.f90:1-30) or, on
// non-cubic boxes, one pressure per axis from the virial's diagonal and tvxyz
// (beren_baro_nc, module_barostat.f90:28-86); the LJ tail (pres_lj_tail,
// md_pressure.f90:37-56) unless the O-O term is Buckingham.  The box scales on
// the host, the waters on the device.
int beren_driver(gb_context *c, const double vir[9], double tv, const double tvxyz[3], double dt, double *rnm) {
  const gb_params &P = c->P;
  if (P.baro != GB_BARO_BER)
    return ctx_set_error(GB_E_UNSUPPORTED, "only the Berendsen barostat (baro = BER) is on the device path");
  const int na = c->na, nm = na / 3;
  const double vol = c->box[0] * c->box[1] * c->box[2];
  double ptail = 0.0;
  if (P.oo_gam == 0.0) {
    const double pi = std::acos(-1.0), rho = (double)nm / vol;
    const double prefac = (16.0 * pi * (rho * rho) * P.oo_eps * (P.oo_sig * P.oo_sig * P.oo_sig)) / 3.0;
    ptail = prefac * ((2.0 / 3.0) * std::pow(P.oo_sig / P.rcut, 9) - std::pow(P.oo_sig / P.rcut, 3));
  }
  double pres[3];
  if (P.iamcub) {
    double w = vir[0] + vir[4] + vir[8];
    w = -w / 3.0;
    const double pc = (2.0 * tv / 3.0 + w) / vol + ptail;
    pres[0] = pres[1] = pres[2] = pc;
  } else {
    for (int j = 0; j < 3; ++j) pres[j] = (-vir[4 * j] + 2.0 * tvxyz[j]) / vol + ptail;
  }
  const double compi = 13531.0, bstat = compi / (3.0 * P.taub);
  double sm1[3];
  for (int j = 0; j < 3; ++j) {
    const double scale = std::fabs(1.0 - (dt * bstat) * (P.patm - pres[j]));
    c->box[j] = scale * c->box[j];
    sm1[j] = scale - 1.0;
  }
  launch_baro_shift(c->stream, c->r, rnm, na, c->nb, sm1);
  c->launches += 1;
  return GB_OK;
}

// Barostat of evolve_pi with nbaro = 1 (evolve_pi.f90:163-189): tv and tvxyz
// averaged over the MTS substeps, the virial as the previous call's vir_lf
// plus this step's high-frequency virial.  Needs the step's accumulators on
// the host: one synchronisation.
int barostat(gb_context *c, double dt) {
  const gb_params &P = c->P;
  if (P.baro != GB_BARO_BER)
    return ctx_set_error(GB_E_UNSUPPORTED, "only the Berendsen barostat (baro = BER) is on the device path");
  CK(cudaMemcpyAsync(c->h_acc, c->acc, sizeof(double) * ACC_NSLOT * ACC_STRIDE, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  const double *A = c->h_acc;
  const double *K = A + (size_t)ACC_KE * ACC_STRIDE;
  const int na = c->na, nb = c->nb, mts = P.mts;
  double vir[9];
  for (int i = 0; i < 9; ++i)
    vir[i] = c->vir_lf_in[i] + A[(size_t)ACC_INT * ACC_STRIDE + 1 + i] / nb / (double)mts;
  const double tq1 = 0.5 * K[0] / nb, tq2 = 0.5 * K[1] / nb;
  const double tc = 0.5 * (3 * na - 3 - P.nctot) / c->last_beta;
  const double tv = tc + (tq1 + tq2) / mts;
  double tvxyz[3];
  for (int j = 0; j < 3; ++j) tvxyz[j] = tc / 3 + (0.5 * K[2 + j] / nb + 0.5 * K[5 + j] / nb) / mts;
  int st = beren_driver(c, vir, tv, tvxyz, dt, nb > 1 ? c->rnm : nullptr);
  if (st) return st;
  // this step's low-frequency forces see the new box: the non-cubic k vectors
  // (bohr^-1) are rebuilt now (the cubic ones are in the unit box)
  return c->P.iamcub ? GB_OK : dev_prepare(c, 0.0, 0.0);
}

// r and dvdr2 are final once the MTS block (and the barostat) ran
int mark_mid(gb_context *c) {
  if (!c->want_mid || !c->mid_ev) return GB_OK;
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  CK(cudaStreamIsCapturing(c->stream, &cap));
  // inside a capture the record becomes an external event node of the graph
  if (cap == cudaStreamCaptureStatusActive) CK(cudaEventRecordWithFlags(c->mid_ev, c->stream, cudaEventRecordExternal));
  else CK(cudaEventRecord(c->mid_ev, c->stream));
  c->mid_recorded = true;
  return GB_OK;
}

int dev_evolve_pi(gb_context *c, double dt, double beta) {
  int st;
  c->mid_recorded = false;
  if (c->nbaro && c->graph.valid) dev_graph_reset(c);
  if ((st = dev_prepare(c, dt, beta))) return st;
  c->plan = EnergyPlan();
  c->plan.evolve = 1;
  c->last_beta = beta;
  const int nb = c->nb, na = c->na, mts = c->P.mts;
  c->plan.mts = mts;
  const long long N = 3LL * na * nb;
  const double dtsmall = dt / (double)mts, halfdtsmall = 0.5 * dtsmall, halfdt = 0.5 * dt;
  cudaStream_t s = c->stream;
  const double dt_therm = c->P.therm == GB_THERM_PRG ? halfdt : dt;  // evolve_pi.f90:73-77
  if ((st = therm_kick(c, dt_therm, beta))) return st;
  CK(cudaMemsetAsync(c->acc, 0, sizeof(double) * ACC_NSLOT * ACC_STRIDE, s));
  prof_begin(c, PR_MTS);
  // one fused kernel for power-of-two nb up to 64 (k_mts.cu)
  int fused = 0;
  if (!c->generic_mts) {
    if ((st = watch_mark(c, PR_MTS, s, 0))) return st;
    launch_fused_mts(s, c, dt, &fused);
    if (fused && (st = watch_mark(c, PR_MTS, s, 1))) return st;
  }
  if (fused) {
    c->plan.B_int = nb;
    c->launches += 1;
    prof_end(c, PR_MTS, (double)c->nm * nb * mts);
    if (c->nbaro && (st = barostat(c, dt))) return st;
    if ((st = mark_mid(c))) return st;
    if ((st = low_frequency(c, c->rnm, c->r, c->p, halfdt))) return st;
    if ((st = therm_kick(c, dt_therm, beta))) return st;
    return launch_status();
  }
  // evolve_pi.f90:82-88
  launch_axpy(s, c->p, c->dvdr, -halfdt, N);
  launch_axpy(s, c->p, c->dvdr2, -halfdtsmall, N);
  launch_realft(s, c->p, c->p, 3 * na, nb, +1, c->tw_nb);
  launch_realft(s, c->r, c->rnm, 3 * na, nb, +1, c->tw_nb);
  c->launches += 4;
  // multiple time steps under the intramolecular force (evolve_pi.f90:93-161)
  for (int im = 1; im <= mts; ++im) {
    launch_rotate(s, c->p, c->rnm, c->monod, na, nb);
    launch_realft(s, c->rnm, c->rst, 3 * na, nb, -1, c->tw_nb);
    CK(cudaMemsetAsync(slot(c, ACC_INT), 0, sizeof(double), s));  // vint of the last substep
    if ((st = term_intra(c, c->rst, nb, c->dvdr2, 0, ACC_INT))) return st;
    launch_virial_ke(s, c->rst, c->dvdr, c->dvdr2, na, nb, slot(c, ACC_KE));
    c->launches += 3;
    if (im != mts) {
      launch_realft(s, c->dvdr2, c->dvdr2, 3 * na, nb, +1, c->tw_nb);
      launch_axpy(s, c->p, c->dvdr2, -dtsmall, N);
      c->launches += 2;
    }
  }
  c->plan.B_int = nb;
  // momenta back to beads; r := rst (evolve_pi.f90:222-228)
  launch_realft(s, c->p, c->p, 3 * na, nb, -1, c->tw_nb);
  std::swap(c->r, c->rst);
  launch_axpy(s, c->p, c->dvdr2, -halfdtsmall, N);
  c->launches += 2;
  prof_end(c, PR_MTS, (double)c->nm * nb * mts);
  if (c->nbaro && (st = barostat(c, dt))) return st;
  if ((st = mark_mid(c))) return st;
  // low-frequency forces and the closing kick (evolve_pi.f90:194-279)
  if ((st = low_frequency(c, c->rnm, c->r, c->p, halfdt))) return st;
  if ((st = therm_kick(c, dt_therm, beta))) return st;
  return launch_status();
}

int dev_evolve_step(gb_context *c, double dt, double beta) {
  if (ctx_rigid(c)) {
    c->last_beta = beta;
    return dev_evolve_rig_pi(c, dt, beta, nullptr);
  }
  return dev_evolve_pi(c, dt, beta);
}

void dev_graph_reset(gb_context *c) {
  if (c->graph.exec) cudaGraphExecDestroy(c->graph.exec);
  c->graph.exec = nullptr;
  c->graph.valid = false;
  c->graph.seen = 0;
}

// The fused step makes all of its decisions on the device (skin-list rebuilds
// included) and no host synchronisation, so once the parameters, dt, beta and
// box are unchanged the host side of a step repeats exactly: the second such
// step is captured into a graph and later steps replay it.  Anything that
// changes the key (or a device status error, which invalidates the skin
// lists) drops the graph.
int dev_step(gb_context *c, double dt, double beta) {
  auto &G = c->graph;
  if (ctx_rigid(c)) return dev_evolve_step(c, dt, beta);  // its force call drops step graphs
  const bool eligible = c->use_graphs && !c->prof && !c->generic_mts &&
                        (c->nb == 2 || c->nb == 4 || c->nb == 8 || c->nb == 16 || c->nb == 32 || c->nb == 64) &&
                        (c->rng_mode == GB_RNG_DEVICE || (c->P.therm != GB_THERM_PRG && c->P.therm != GB_THERM_PRL)) &&
                        !c->nbaro;
  const bool same = eligible && G.dt == dt && G.beta == beta && G.box[0] == c->box[0] && G.box[1] == c->box[1] &&
                    G.box[2] == c->box[2] && std::memcmp(&G.P, &c->P, sizeof(gb_params)) == 0;
  if (!same) {
    dev_graph_reset(c);
    G.dt = dt;
    G.beta = beta;
    for (int d = 0; d < 3; ++d) G.box[d] = c->box[d];
    G.P = c->P;
  }
  if (same && G.valid) {
    CK(cudaGraphLaunch(G.exec, c->stream));
    c->launches += G.launches;
    c->plan = G.plan;
    c->last_beta = beta;
    c->mid_recorded = G.mid;
    return GB_OK;
  }
  if (!eligible || G.seen < 1) {  // plain step; the next one with this key is captured
    int st = dev_evolve_pi(c, dt, beta);
    if (st) return st;
    if (eligible) G.seen += 1;
    return GB_OK;
  }
  int sp = dev_prepare(c, dt, beta);  // set-up copies synchronise: never inside the capture
  if (sp) return sp;
  const int64_t l0 = c->launches;
  CK(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
  int st = dev_evolve_pi(c, dt, beta);
  cudaGraph_t graph = nullptr;
  cudaError_t e = cudaStreamEndCapture(c->stream, &graph);
  if (st) {
    if (graph) cudaGraphDestroy(graph);
    return st;
  }
  if (e != cudaSuccess) return ctx_check_cuda(e, "cudaStreamEndCapture");
  // node priorities: the k-space branch keeps the priority of its stream
  e = cudaGraphInstantiate(&G.exec, graph, cudaGraphInstantiateFlagUseNodePriority);
  cudaGraphDestroy(graph);
  if (e != cudaSuccess) {
    G.exec = nullptr;
    return ctx_check_cuda(e, "cudaGraphInstantiate");
  }
  G.valid = true;
  G.launches = c->launches - l0;
  G.plan = c->plan;
  G.mid = c->mid_recorded;
  CK(cudaGraphLaunch(G.exec, c->stream));  // the captured step has not run yet
  return GB_OK;
}

// forces(r, v, dvdr, nb, ..., iopt = 1) of evolve_rig_pi (evolve_rigid.f90:174)
int term_forces_rigid(gb_context *c) {
  dev_graph_reset(c);  // other list configurations: a captured step would be stale
  int st;
  if ((st = dev_prepare(c, 0.0, 0.0))) return st;
  c->plan = EnergyPlan();
  CK(cudaMemsetAsync(c->acc, 0, sizeof(double) * ACC_NSLOT * ACC_STRIDE, c->stream));
  if ((st = term_ewald(c, c->r, c->nb, c->dvdr, 1.0, 0, ACC_EW2))) return st;
  c->plan.B_ew2 = c->nb;
  if ((st = term_lj(c, c->r, c->nb, c->dvdr, 1, ACC_LJ2))) return st;
  c->plan.B_lj2 = c->nb;
  return launch_status();
}

int dev_collect(gb_context *c, int mode, double dt, double beta) {
  (void)dt;
  (void)beta;
  CK(cudaMemcpyAsync(c->h_acc, c->acc, sizeof(double) * ACC_NSLOT * ACC_STRIDE, cudaMemcpyDeviceToHost, c->stream));
  CK(cudaMemcpyAsync(c->h_status, c->status, sizeof(unsigned), cudaMemcpyDeviceToHost, c->stream));
  CK(cudaStreamSynchronize(c->stream));
  CK(cudaGetLastError());
  unsigned stw = *c->h_status;
  if (stw) {
    CK(cudaMemsetAsync(c->status, 0, sizeof(unsigned), c->stream));
    for (SkinList &L : c->sl) L.valid = false;  // a list may have overflowed: rebuild at next use
    dev_graph_reset(c);
    if (stw & ST_LIST_OVERFLOW) return ctx_set_error(GB_E_LIST, "neighbour list too small");
    if (stw & ST_RATTLE1) return ctx_set_error(GB_E_RATTLE1, "max iterations exceeded in rattle stage 1");
    if (stw & ST_RATTLE2) return ctx_set_error(GB_E_RATTLE2, "max iterations exceeded in rattle stage 2");
    if (stw & ST_NONFINITE) return ctx_set_error(GB_E_NONFINITE, "non-finite force");
    return ctx_set_error(GB_E_NONFINITE, "device status error");
  }
  const double *A = c->h_acc;
  auto S = [&](int s) { return A + (size_t)s * ACC_STRIDE; };
  // the box of the step's Ewald evaluation: a barostat after the forces (the
  // rigid step) has scaled c->box since
  const double L = c->acc_L > 0.0 ? c->acc_L : c->box[0];
  const double qq = c->qq;
  const double vself = c->P.walpha / std::sqrt(PI) * qq;
  const EnergyPlan &pl = c->plan;
  double vew = 0.0, vlj = 0.0, vint = 0.0;
  double vir_ew[9] = {0}, vir_lj[9] = {0}, vir_int[9] = {0};
  const double Le = c->P.iamcub ? L : 1.0;  // the cubic sum runs in the unit box
  auto add_ewald = [&](int s, int B) {
    if (!B) return;
    vew += (S(s)[0] - B * vself) / Le / B;
    for (int i = 0; i < 9; ++i) vir_ew[i] += S(s)[1 + i] / Le / B;
  };
  auto add_tem = [&](int s, int B, double sign) {
    if (!B) return;
    vew += sign * S(s)[0] / B;
    for (int i = 0; i < 9; ++i) vir_ew[i] += sign * S(s)[1 + i] / B;
  };
  auto add_lj = [&](int s, int B) {
    if (!B) return;
    vlj += 4.0 * c->P.oo_eps * S(s)[0] / B;
    for (int i = 0; i < 9; ++i) vir_lj[i] += 48.0 * c->P.oo_eps * S(s)[1 + i] / B;
  };
  add_ewald(ACC_EW, pl.B_ew);
  add_tem(ACC_TEM, pl.B_tem, -1.0);
  add_ewald(ACC_EW2, pl.B_ew2);
  add_tem(ACC_TEM2, pl.B_tem2, 1.0);
  add_lj(ACC_LJ, pl.B_lj);
  add_lj(ACC_LJ2, pl.B_lj2);
  if (pl.B_int) {
    vint = S(ACC_INT)[0] / pl.B_int;
    double div = pl.evolve ? (double)pl.mts : 1.0;
    for (int i = 0; i < 9; ++i) vir_int[i] = S(ACC_INT)[1 + i] / pl.B_int / div;
  }
  c->e_vew = vew;
  c->e_vlj = vlj;
  c->e_vint = vint;
  c->e_v = vew + vlj + vint;
  for (int i = 0; i < 9; ++i) {
    c->e_vir_lf[i] = vir_lj[i] + vir_ew[i];
    c->e_vir_hf[i] = vir_int[i];
    c->e_vir[i] = c->e_vir_lf[i] + c->e_vir_hf[i];
  }
  if (pl.evolve) {
    // evolve_pi's vir_lf output is the next call's vir_lf input (the barostat reads it)
    for (int i = 0; i < 9; ++i) c->vir_lf_in[i] = c->e_vir_lf[i];
    const int nb = c->nb;
    double tq1 = 0.5 * S(ACC_KE)[0] / nb, tq2 = 0.5 * S(ACC_KE)[1] / nb;
    double tc = 0.5 * (3 * c->na - 3 - c->P.nctot) / c->last_beta;
    c->e_tv = tc + (tq1 + tq2) / pl.mts;
  }
  (void)mode;
  return GB_OK;
}

// Device bytes a context of (na, nb) with parameters P holds once it has run
// evolve_pi: the arrays of ctx_alloc, the k-space tables (build_kvectors) and
// the exact and skin pair lists of the Ewald, LJ and TEM terms (make_list, skin
// 0.1), plus a tenth for allocation granularity and small tables.  Used to admit
// batch replicas by memory footprint before anything is allocated.
size_t dev_estimate_bytes(int na, int nb, const gb_params &P) {
  const size_t N = 3 * (size_t)na * nb, nm = na / 3;
  size_t b = sizeof(double) * (15 * N + 5 * (size_t)na + 12 * (size_t)nb + ACC_NSLOT * ACC_STRIDE);
  b += sizeof(float4) * (3 * (size_t)na * nb + 2 * nm * nb);
  b += sizeof(int4) * (size_t)na * nb + sizeof(double) * 3 * (size_t)na + 4 * sizeof(float);  // shared-list buffers
  const int kmax = std::max(P.kmax, 0);
  const int cap_col = gb_kcap_col(kmax), cap_kp = gb_kcap_kp(kmax);
  std::vector<KCol> col(cap_col);
  std::vector<int4> kp(cap_kp), grp(cap_kp);
  std::vector<double> kw(cap_kp);
  KTables t;
  if (!gb_build_ktables(P, recip_group_len(), col.data(), cap_col, kp.data(), kw.data(), cap_kp, grp.data(),
                        cap_kp, &t)) {
    const size_t nc = std::max(nb, 1), nchunk = (na + recip_sk_chunk() - 1) / recip_sk_chunk();
    b += sizeof(double2) * 3 * (size_t)(kmax + 1) * na * nc;
    b += sizeof(double) * (4 * (size_t)std::max(t.nkp, 1) * nchunk + 8 * (size_t)t.nkp) * nc;
    b += sizeof(KCol) * t.ncol + sizeof(int4) * (t.ngrp + t.nkp) + sizeof(double) * t.nkp;
  }
  // pair lists: one exact list sized for the largest term, one skin list per term
  size_t exact = 0;
  auto lists = [&](size_t nconf, int npt, double cut, double vol) {
    const size_t cap = list_cap(npt, cut, vol), scap = list_cap(npt, 1.1 * cut, vol);
    exact = std::max(exact, sizeof(int) * nconf * npt * (cap + 1));
    return sizeof(int) * nconf * npt * (scap + 1) + sizeof(double) * 3 * nconf * npt;
  };
  // the LJ and TEM cut-offs are in bohr: the box holds nm molecules at the
  // density of liquid water, 29.9 A^3 each
  const double vol = (double)nm * 29.9 / (0.5291772108 * 0.5291772108 * 0.5291772108);
  const size_t bew = (nb > 1 && P.nbdf1 > 0) ? P.nbdf1 : nb;
  const size_t blj = (nb > 1 && P.nbdf2 > 0) ? P.nbdf2 : nb;
  b += lists(bew, na, P.wrcut, 1.0);
  b += lists(blj > 3 ? 1 : blj, (int)nm, P.rcut, vol);
  if (P.sig > 0.0) b += lists(1, na, P.sig + 5.0, vol);
  b += exact;
  return b + b / 10;
}

size_t ctx_device_bytes(const gb_context *c) {
  size_t b = c->alloc_bytes + c->ktab_bytes + c->sk_part_bytes + c->sk_bytes + c->pl_idx_bytes + c->pl_cnt_bytes;
  b += sizeof(KCol) * c->ncol + sizeof(int4) * (c->ngrp + c->nkp) + sizeof(double) * 10 * c->nkp;
  for (const SkinList &L : c->sl) b += L.idx_bytes + L.cnt_bytes + L.ref_bytes;
  return b;
}
