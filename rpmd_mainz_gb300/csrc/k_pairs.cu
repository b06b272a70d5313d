// k_pairs.cu -- pair lists and pair-force kernels (FP64).
//
// Pair lists.  The reference finds pairs through head/chain linked cells
// (linked_cell.f90) or O(N^2) loops (neigh_list.f90, ewc_basic_tem); the set
// of pairs is always "minimum-image distance below the cut-off", so the device
// builds that set directly: a tiled all-pairs scan whose FP32 prefilter on
// wrapped fractional coordinates rejects far pairs and accepts near ones, and
// whose FP64 test, rounded exactly like the reference's
// dx*dx + dy*dy + dz*dz < rcut*rcut, decides the pairs inside a narrow band
// around the cut-off.  Each pair is stored once, in the list of i when
// (i < j) == ((i + j) odd), which halves the lists and balances their lengths;
// full lists (PairGeom::full, for the FP32 kernels) store it in both.
//
// Pair forces (FP64).  A few lanes per (configuration, point) walk its half
// list, keep the point's own force in registers and scatter the partner's force
// with FP64 atomics; energy and virial are reduced per block and added to an
// accumulator slot.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>

#include "gb_common.cuh"
#include "gb_kernels.h"

namespace {

constexpr int LB_T = 128;

// wrapped fractional coordinates u in [0, 1) as FP32 (frac); with lo, also the
// remainder u - frac as a second FP32, so that frac + lo carries u to ~1e-14
// point t = (c, i): frac[t] (and lo[t]) from g.pos; returns frac[t].
// fx (optional): the same coordinates in 32-bit fixed point, u * 2^32 rounded
// and taken modulo 2^32, with the charge's FP32 bits in w.  A wrapping
// difference of two of them, read as a signed integer, is the minimum-image
// difference (|d| < 1/2) in units of 2^-32 exactly, so one integer subtraction
// and one conversion give it to FP32 rounding of the difference itself.
GB_D int4 fixed_point(const PairGeom &g, int c, int i, const double *q) {
  const double *x = g.pos + c * g.cstride + (long long)i * g.pstride;
  unsigned fxd[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double u = g.unit ? x[d] : x[d] * g.onbox[d];
    u -= floor(u);
    fxd[d] = (unsigned)__double2ull_rn(u * 4294967296.0);  // u = 1 (rounded) wraps to 0
  }
  return make_int4((int)fxd[0], (int)fxd[1], (int)fxd[2], __float_as_int(q ? (float)q[i] : 0.0f));
}

GB_D float4 frac_point(const PairGeom &g, long long t, int c, int i, float4 *frac, float4 *lo, const double *q,
                       int4 *fx = nullptr) {
  const double *x = g.pos + c * g.cstride + (long long)i * g.pstride;
  float f[3], e[3];
  unsigned fxd[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    double u = g.unit ? x[d] : x[d] * g.onbox[d];
    u -= floor(u);
    fxd[d] = (unsigned)__double2ull_rn(u * 4294967296.0);  // u = 1 (rounded) wraps to 0
    const float uf = (float)u;
    // remainder against the rounded value, before 1.0f wraps to 0: hi + lo is
    // then u or u - 1, both the same point of the periodic box
    e[d] = (float)(u - (double)uf);
    f[d] = uf >= 1.0f ? 0.0f : uf;
  }
  const float4 h = make_float4(f[0], f[1], f[2], q ? (float)q[i] : 0.0f);
  frac[t] = h;
  if (lo) lo[t] = make_float4(e[0], e[1], e[2], 0.0f);
  if (fx) fx[t] = make_int4((int)fxd[0], (int)fxd[1], (int)fxd[2], __float_as_int(h.w));
  return h;
}

__global__ void k_frac32(PairGeom g, int nconf, float4 *frac, float4 *lo, const double *q, int4 *fx) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nconf * g.npt) return;
  frac_point(g, t, (int)(t / g.npt), (int)(t % g.npt), frac, lo, q, fx);
}

// exact FP64 minimum-image test, rounded as the reference rounds it
GB_D bool exact_pair_in(const PairGeom &g, const double *a, const double *b) {
  double dx = __dsub_rn(a[0], b[0]), dy = __dsub_rn(a[1], b[1]), dz = __dsub_rn(a[2], b[2]);
  if (g.unit) {
    dx = __dsub_rn(dx, nint_d(dx));
    dy = __dsub_rn(dy, nint_d(dy));
    dz = __dsub_rn(dz, nint_d(dz));
  } else {
    dx = __dsub_rn(dx, __dmul_rn(g.box[0], nint_d(__dmul_rn(g.onbox[0], dx))));
    dy = __dsub_rn(dy, __dmul_rn(g.box[1], nint_d(__dmul_rn(g.onbox[1], dy))));
    dz = __dsub_rn(dz, __dmul_rn(g.box[2], nint_d(__dmul_rn(g.onbox[2], dz))));
  }
  return dsq3(dx, dy, dz) < g.rcutsq;
}

// Block (i-tile, j-chunk, configuration): each thread tests its point i against
// a chunk of partners staged through shared memory.  Hits go to a 32-entry
// staging row per thread in shared memory; a full row (and the rest at the end
// of the chunk) reserves its slots in the point's list with one atomic add and
// is copied out, so the order of the flushed groups inside a list is arbitrary.
constexpr int LB_STAGE = 32;

// FULL: store every pair in both lists (else the parity rule above); EXCL:
// skip pairs of the same molecule.  Four partners at a time: their FP32
// distances first, then the rare near pairs one by one.
template <bool FULL, bool EXCL>
__global__ void __launch_bounds__(LB_T) k_build_list2(PairGeom g, const float4 *frac, int *count,
                                                      int *idx, int cap, float3 len, float thr_lo,
                                                      float thr_hi, unsigned *status, const unsigned *gate,
                                                      int jchunk, const float *thr_dev) {
  __shared__ float4 tile[LB_T];
  __shared__ int stage[LB_T][LB_STAGE + 1];
  if (gate && *gate == 0u) return;  // skin list still valid: nothing to rebuild
  // thr_dev: a superset radius chosen on the device (a shared list); every
  // pair inside it is taken, without the exact band test
  const bool dev_thr = thr_dev != nullptr;
  if (dev_thr) thr_hi = thr_dev[0];
  const int c = blockIdx.z;
  const int i = blockIdx.x * LB_T + threadIdx.x;
  const int npt = g.npt;
  const int j0 = blockIdx.y * jchunk, j1 = min(npt, j0 + jchunk);
  const float4 *fr = frac + (long long)c * npt;
  const double *base = g.pos + c * g.cstride;
  float4 fi = make_float4(0.f, 0.f, 0.f, 0.f);
  double pi[3] = {0, 0, 0};
  if (i < npt) {
    fi = fr[i];
    const double *x = base + (long long)i * g.pstride;
    pi[0] = x[0];
    pi[1] = x[1];
    pi[2] = x[2];
  }
  int *cnt = count + (long long)c * npt + (i < npt ? i : 0);
  int *my = idx + ((long long)c * npt + (i < npt ? i : 0)) * cap;
  int *st = stage[threadIdx.x];
  int nst = 0;
  bool over = false;
  auto flush = [&]() {
    const int slot = atomicAdd(cnt, nst);
    for (int k = 0; k < nst; ++k) {
      if (slot + k < cap) my[slot + k] = st[k];
      else over = true;
    }
    nst = 0;
  };
  auto dist2 = [&](const float4 &fj) {
    float dx = fi.x - fj.x, dy = fi.y - fj.y, dz = fi.z - fj.z;
    dx = (dx - rintf(dx)) * len.x;
    dy = (dy - rintf(dy)) * len.y;
    dz = (dz - rintf(dz)) * len.z;
    return dx * dx + dy * dy + dz * dz;
  };
  auto near = [&](int j, float d2) {  // d2 < thr_hi
    if (j == i) return;
    if (!FULL && (i < j) != (((i + j) & 1) != 0)) return;
    if (EXCL && (i / 3) == (j / 3)) return;
    if (dev_thr || d2 < thr_lo || exact_pair_in(g, pi, base + (long long)j * g.pstride)) {
      st[nst++] = j;
      if (nst == LB_STAGE) flush();
    }
  };
  for (int jt = j0; jt < j1; jt += LB_T) {
    const int jl = jt + threadIdx.x;
    tile[threadIdx.x] = jl < j1 ? fr[jl] : make_float4(0.5f, 0.5f, 0.5f, 0.f);
    __syncthreads();
    if (i < npt) {
      const int jmax = min(LB_T, j1 - jt);
      int jj = 0;
      for (; jj + 4 <= jmax; jj += 4) {
        float d2[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) d2[u] = dist2(tile[jj + u]);
#pragma unroll
        for (int u = 0; u < 4; ++u)
          if (d2[u] < thr_hi) near(jt + jj + u, d2[u]);
      }
      for (; jj < jmax; ++jj) {
        const float d2 = dist2(tile[jj]);
        if (d2 < thr_hi) near(jt + jj, d2);
      }
    }
    __syncthreads();
  }
  if (i < npt && nst > 0) flush();
  if (over) atomicOr(status, ST_LIST_OVERFLOW);
}

// ---- cell-sorted build (skin supersets) ----
// The wrapped fractional box is cut into nx * ny * nz cells of side at least
// 1/R of the largest accepted distance, so that every pair within it joins
// points whose cells differ by at most R per axis (R = 1..6, nx, ny, nz >=
// 2R + 1: the (2R+1)^3 stencil cells are distinct; rows and row ends whose
// cells lie wholly beyond that distance are pruned).  Every step k_cell_count
// takes the skin test (moved points) and counts the points per cell; its last
// block turns the counts into cell offsets when a rebuild is due and clears
// them.  On a rebuild k_cell_scatter writes the points in cell order and
// k_build_sorted runs one warp per point: the x-rows of stencil cells are
// contiguous runs of the cell order, which the lanes read in
// coalesced 32-slot steps; hits are appended through a ballot (no atomics).
// The FP32 prefilter and the FP64 band test are those of k_build_list2.
constexpr int CELL_RMAX = 6;  // largest stencil radius in cells
constexpr int BUILD_RUNS_MAX = 2 * (2 * CELL_RMAX + 1) * (2 * CELL_RMAX + 1);  // slot runs of a stencil
struct CellSortDev {
  int nx, ny, nz, R;
  // per stencil row (oz, oy): the largest |ox| whose cells can hold a pair
  // within the cut-off, -1 when none can ([2R+1][2R+1])
  signed char reach[(2 * CELL_RMAX + 1) * (2 * CELL_RMAX + 1)];
  int *ccount;     // [nconf][ncell], zero between steps
  int *cstart;     // [nconf][ncell + 1]
  int *cellid;     // [nconf][npt]
  int *crank;      // [nconf][npt] rank in the cell (arbitrary order)
  float4 *spos;    // [nconf][npt] fractional positions in cell order, the point's index in w (int bits)
  int *sidx;       // [nconf][npt] point of each cell-order slot
  int *slot_of;    // [nconf][npt] slot of each point at the last rebuild
  int4 *fxs;       // [nconf][npt] fixed-point positions in slot order (null: not kept)
  unsigned *ticket;  // [0] blocks done in the count kernel, [1] a point moved
};

// (clamped both ways: a wrapped coordinate is in [0, 1], and a non-finite one
// converts to 0, so no input can index outside the grid)
GB_D int cell_of(float u, int n) { return max(min((int)(u * (float)n), n - 1), 0); }

// fractional distance from u to cell c (unwrapped index, may lie outside
// 0..n-1) of an axis of n cells; 0 inside it
GB_D float cell_gap(float u, int c, int n) {
  const float lo = (float)c / (float)n, hi = (float)(c + 1) / (float)n;
  return fmaxf(fmaxf(lo - u, u - hi), 0.0f);
}

// (also writes the points' fractional coordinates, as k_frac32)
__global__ void __launch_bounds__(256) k_cell_count(PairGeom g, int nconf, float4 *frac, float4 *lo, const double *q,
                                                    CellSortDev cs, const double *ref, double lim2, int check,
                                                    unsigned *flag, int4 *fx, ListSpread sp) {
  __shared__ bool last;
  __shared__ int part[256];
  const long long n = (long long)nconf * g.npt;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int ncell = cs.nx * cs.ny * cs.nz;
  bool moved = false;
  if (t < n) {
    const int c = (int)(t / g.npt), i = (int)(t % g.npt);
    if (check) {
      const double *x = g.pos + c * g.cstride + (long long)i * g.pstride;
      const double *r0 = ref + 3 * t;
      const double dx = x[0] - r0[0], dy = x[1] - r0[1], dz = x[2] - r0[2];
      moved = !(dx * dx + dy * dy + dz * dz <= lim2);  // NaN counts as moved
    }
    const float4 f = frac_point(g, t, c, i, frac, lo, q, fx);
    // slot-ordered copy under the last rebuild's order (a rebuild in this step
    // rewrites it in k_cell_scatter)
    if (cs.fxs) cs.fxs[(long long)c * g.npt + cs.slot_of[t]] = fx[t];
    const int cell = (cell_of(f.z, cs.nz) * cs.ny + cell_of(f.y, cs.ny)) * cs.nx + cell_of(f.x, cs.nx);
    cs.cellid[t] = cell;
    cs.crank[t] = atomicAdd(cs.ccount + (long long)c * ncell + cell, 1);
  }
  if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) atomicOr(cs.ticket + 1, 1u);
  __threadfence();
  __syncthreads();
  if (threadIdx.x == 0) last = atomicAdd(cs.ticket, 1u) == gridDim.x - 1;
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the decision of this step: the gate of the scatter and build kernels;
  // the moved word is cleared for the next step (no memset per step)
  __shared__ bool s_rebuild;
  if (threadIdx.x == 0) {
    s_rebuild = !check || *(volatile unsigned *)(cs.ticket + 1) != 0u;
    *flag = s_rebuild ? 1u : 0u;
    cs.ticket[1] = 0u;
    if (sp.w) {  // a shared list: its margin for the bead spread, chosen at each rebuild
      volatile float *w = sp.w;
      if (s_rebuild) {
        const float dres = fminf(sp.dcap, 1.25f * sqrtf(w[0]) + sp.dmin);
        const float rl = sp.base + 2.0f * dres;
        w[1] = dres * dres;
        w[2] = rl * rl * (1.0f + 1e-5f);
      }
      w[0] = 0.0f;  // the next step's spread
    }
  }
  __syncthreads();
  const bool rebuild = s_rebuild;
  volatile int *cnt = cs.ccount;
  for (int c = 0; c < nconf; ++c) {
    volatile int *cc = cnt + (long long)c * ncell;
    if (rebuild) {  // exclusive scan: contiguous chunks per thread, then the chunk offsets
      const int per = (ncell + 255) / 256, a = threadIdx.x * per, b = min(ncell, a + per);
      int sum = 0;
      for (int k = a; k < b; ++k) sum += cc[k];
      // exclusive scan of the 256 chunk sums: within warps by shuffles, then
      // the 8 warp totals
      const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
      int inc = sum;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += v;
      }
      if (lane == 31) part[wid] = inc;
      __syncthreads();
      int woff = 0;
      for (int w = 0; w < wid; ++w) woff += part[w];
      int run = woff + inc - sum;
      __syncthreads();
      int *st = cs.cstart + (long long)c * (ncell + 1);
      for (int k = a; k < b; ++k) {
        st[k] = run;
        run += cc[k];
      }
      if (threadIdx.x == 255) st[ncell] = run;
      __syncthreads();
    }
    for (int k = threadIdx.x; k < ncell; k += blockDim.x) cc[k] = 0;
  }
  if (threadIdx.x == 0) *cs.ticket = 0u;
}

// (also the skin-list bookkeeping of k_skin_save: reference positions and the
// rebuild count)
__global__ void k_cell_scatter(PairGeom g, int nconf, const float4 *frac, CellSortDev cs, int *lcount,
                               const unsigned *gate, double *ref, unsigned *rebuilds, const int4 *fx) {
  if (*gate == 0u) return;
  const int npt = g.npt;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) atomicAdd(rebuilds, 1u);
  if (t >= (long long)nconf * npt) return;
  lcount[t] = 0;
  const int c = (int)(t / npt), i = (int)(t % npt);
  const double *x = g.pos + c * g.cstride + (long long)i * g.pstride;
  ref[3 * t] = x[0];
  ref[3 * t + 1] = x[1];
  ref[3 * t + 2] = x[2];
  const int ncell = cs.nx * cs.ny * cs.nz;
  const long long pos = (long long)c * npt + cs.cstart[(long long)c * (ncell + 1) + cs.cellid[t]] + cs.crank[t];
  const float4 f = frac[t];
  cs.spos[pos] = make_float4(f.x, f.y, f.z, __int_as_float(i));  // the point's index rides in w
  cs.sidx[pos] = i;
  if (cs.slot_of) cs.slot_of[t] = (int)(pos - (long long)c * npt);
  if (cs.fxs) cs.fxs[pos] = fx[t];
}

// IT: the list entry type (int, or unsigned short when npt <= 65535)
// SLOTS: store the partner's cell-order slot, bit 15 set for the same
// molecule (unsigned short entries, npt <= 32767), instead of its index
template <bool FULL, bool EXCL, typename IT, bool SLOTS = false>
__global__ void __launch_bounds__(LB_T) k_build_sorted(PairGeom g, int nconf, CellSortDev cs, int *count, IT *idx,
                                                       int cap, float3 len, float thr_lo, float thr_hi,
                                                       unsigned *status, const unsigned *gate,
                                                       const float *thr_dev) {
  __shared__ signed char s_reach[sizeof(cs.reach)];
  __shared__ int s_run[LB_T / 32][BUILD_RUNS_MAX], s_pre[LB_T / 32][BUILD_RUNS_MAX];
  if (*gate == 0u) return;
  // thr_dev: a superset radius chosen on the device (a shared list); every
  // pair inside it is taken, without the exact band test
  const bool dev_thr = thr_dev != nullptr;
  if (dev_thr) thr_hi = thr_dev[0];
  const float thr_row = thr_hi * (1.0f + 1e-4f);  // the row trimming's bound, with a margin for rounding
  for (int t = threadIdx.x; t < (int)sizeof(cs.reach); t += blockDim.x) s_reach[t] = cs.reach[t];
  __syncthreads();
  const int npt = g.npt;
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // one warp per point
  const int lane = threadIdx.x & 31;
  if (w >= (long long)nconf * npt) return;  // the whole warp
  const int c = (int)(w / npt);
  const int kk = (int)(w - (long long)c * npt);
  const int ncell = cs.nx * cs.ny * cs.nz;
  const float4 *sp = cs.spos + (long long)c * npt;
  const int *si = cs.sidx + (long long)c * npt;
  const int *st = cs.cstart + (long long)c * (ncell + 1);
  const int i = si[kk];
  const float4 fi = sp[kk];
  const double *base = g.pos + c * g.cstride;
  const double *xi = base + (long long)i * g.pstride;
  const double pi[3] = {xi[0], xi[1], xi[2]};
  const int x0 = cell_of(fi.x, cs.nx), y0 = cell_of(fi.y, cs.ny), z0 = cell_of(fi.z, cs.nz);
  IT *my = idx + ((long long)c * npt + i) * cap;
  int n = 0;  // the same in every lane
  // The stencil rows' runs of cell-order slots (one or two per row, the x
  // cells wrapped) are staged first: each lane takes a row and loads its cell
  // offsets, so that the offsets of all rows arrive in one round trip; the
  // runs, kept in scan order, are then walked as one sequence of candidate
  // slots, four 32-slot groups per round (their loads issued together) across
  // run boundaries.  Hits keep the scan order (rows in (oz, oy) order, runs in
  // x order, slots in cell order), the order of the single-row walk.
  const int wl = threadIdx.x >> 5;
  int *runs = s_run[wl];    // [nrun] first slot of each run
  int *pre = s_pre[wl];     // [nrun] inclusive prefix sums of the run lengths
  const int R = cs.R, W = 2 * R + 1, nrows = W * W;
  auto wrap = [](int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); };  // |offset| <= R < n
  int nrun = 0;  // the same in every lane
  for (int q0 = 0; q0 < nrows; q0 += 32) {
    const int q = q0 + lane;
    int a0 = 0, a1 = 0, b0 = 0, b1 = 0;
    if (q < nrows) {
      const int rx = s_reach[q];
      // the row's cells (unwrapped indices zz, yy) as far as this point can
      // reach them: its distance to the row in y and z leaves an x extent
      const int zz = z0 + q / W - R, yy = y0 + q % W - R;
      const float gy = cell_gap(fi.y, yy, cs.ny) * len.y, gz = cell_gap(fi.z, zz, cs.nz) * len.z;
      const float rem = thr_row - gy * gy - gz * gz;
      int xa = 0, xb = -1;
      if (rx >= 0 && rem > 0.0f) {  // else no cell of this row is within the cut-off
        const float ex = sqrtf(rem) / len.x * (float)cs.nx;  // x extent in cells
        const float cx = fi.x * (float)cs.nx;
        xa = max(x0 - rx, (int)floorf(cx - ex - 1e-3f));
        xb = min(x0 + rx, (int)floorf(cx + ex + 1e-3f));
      }
      if (xa <= xb) {  // the x cells, wrapped into one or two runs
        const int z = wrap(zz, cs.nz), y = wrap(yy, cs.ny);
        const int row = (z * cs.ny + y) * cs.nx;
        if (xa >= 0 && xb < cs.nx) {
          a0 = st[row + xa], a1 = st[row + xb + 1];
        } else if (xa < 0) {
          a0 = st[row], a1 = st[row + xb + 1];
          b0 = st[row + cs.nx + xa], b1 = st[row + cs.nx];
        } else {
          a0 = st[row + xa], a1 = st[row + cs.nx];
          b0 = st[row], b1 = st[row + xb - cs.nx + 1];
        }
      }
    }
    const bool ha = a1 > a0, hb = b1 > b0;
    const int cnt = (int)ha + (int)hb;
    int incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    int pos = nrun + incl - cnt;
    if (ha) runs[pos] = a0, pre[pos++] = a1 - a0;
    if (hb) runs[pos] = b0, pre[pos] = b1 - b0;
    nrun += __shfl_sync(0xffffffffu, incl, 31);
  }
  __syncwarp();
  // inclusive prefix of the lengths, 32 runs at a time with a carry
  int carry = 0;
  for (int r0 = 0; r0 < nrun; r0 += 32) {
    const int r = r0 + lane;
    int v = r < nrun ? pre[r] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int u = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += u;
    }
    if (r < nrun) pre[r] = carry + v;
    carry += __shfl_sync(0xffffffffu, v, 31);
  }
  __syncwarp();
  const int total = carry;
  int j = 0;  // this lane's run: its candidate index only grows
  for (int kb = 0; kb < total; kb += 128) {
    float4 fj[4];
    int ks[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int gi = kb + 32 * u + lane;
      ks[u] = -1;
      fj[u] = make_float4(2.f, 2.f, 2.f, 0.f);
      if (gi < total) {
        while (pre[j] <= gi) ++j;
        const int k = runs[j] + gi - (j ? pre[j - 1] : 0);
        ks[u] = k;
        fj[u] = sp[k];
      }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      if (kb + 32 * u >= total) break;  // the same in every lane
      const int k = ks[u];
      bool hit = false;
      int jj = 0;
      if (k >= 0) {
        float dx = fi.x - fj[u].x, dy = fi.y - fj[u].y, dz = fi.z - fj[u].z;
        dx = (dx - rintf(dx)) * len.x;
        dy = (dy - rintf(dy)) * len.y;
        dz = (dz - rintf(dz)) * len.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        if (d2 < thr_hi) {
          jj = __float_as_int(fj[u].w);
          hit = jj != i && (FULL || (i < jj) == (((i + jj) & 1) != 0)) && (!EXCL || (i / 3) != (jj / 3)) &&
                (dev_thr || d2 < thr_lo || exact_pair_in(g, pi, base + (long long)jj * g.pstride));
        }
      }
      const unsigned m = __ballot_sync(0xffffffffu, hit);
      if (hit) {
        const int pos = n + __popc(m & ((1u << lane) - 1u));
        if (pos < cap) my[pos] = SLOTS ? (IT)(k | ((i / 3) == (jj / 3) ? 0x8000 : 0)) : (IT)jj;
      }
      n += __popc(m);
    }
  }
  if (lane == 0) {
    count[(long long)c * npt + i] = n;
    if (n > cap) atomicOr(status, ST_LIST_OVERFLOW);
  }
}

// ---- skin lists ----
// flag |= 1 when a point of any configuration has moved by more than sqrt(lim2)
// since ref was taken (ref: [nconf][npt][3])
__global__ void k_skin_check(PairGeom g, int nconf, const double *ref, double lim2, unsigned *flag) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool moved = false;
  if (t < (long long)nconf * g.npt) {
    const int c = (int)(t / g.npt), i = (int)(t % g.npt);
    const double *x = g.pos + c * g.cstride + (long long)i * g.pstride;
    const double *r0 = ref + 3 * t;
    const double dx = x[0] - r0[0], dy = x[1] - r0[1], dz = x[2] - r0[2];
    moved = !(dx * dx + dy * dy + dz * dz <= lim2);  // NaN counts as moved
  }
  if (__any_sync(0xffffffffu, moved) && (threadIdx.x & 31) == 0) atomicOr(flag, 1u);
}

// on a rebuild: zero the superset list's counts
__global__ void k_skin_zero(int *count, long long n, const unsigned *flag) {
  if (*flag == 0u) return;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < n) count[t] = 0;
}

// on a rebuild: remember the positions it was made from
__global__ void k_skin_save(PairGeom g, int nconf, double *ref, const unsigned *flag, unsigned *rebuilds) {
  if (*flag == 0u) return;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t == 0) atomicAdd(rebuilds, 1u);
  if (t >= (long long)nconf * g.npt) return;
  const int c = (int)(t / g.npt), i = (int)(t % g.npt);
  const double *x = g.pos + c * g.cstride + (long long)i * g.pstride;
  ref[3 * t] = x[0];
  ref[3 * t + 1] = x[1];
  ref[3 * t + 2] = x[2];
}

// exact list from the superset: one warp per (configuration, point); the same
// FP32 prefilter and reference-rounded FP64 band test as the full build, lanes
// append in list order through a ballot (IT: the superset's entry type)
template <typename IT>
__global__ void __launch_bounds__(128) k_list_filter(PairGeom g, int nconf, const float4 *frac,
                                                     const int *scount, const IT *sidx, int scap,
                                                     int *count, int *idx, int cap, float3 len,
                                                     float thr_lo, float thr_hi, unsigned *status) {
  const long long w = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (w >= (long long)nconf * g.npt) return;
  const int c = (int)(w / g.npt), i = (int)(w % g.npt);
  const float4 *fr = frac + (long long)c * g.npt;
  const double *base = g.pos + c * g.cstride;
  const float4 fi = fr[i];
  const double *pi = base + (long long)i * g.pstride;
  const int n = min(scount[w], scap);
  const IT *L = sidx + w * scap;
  int *out = idx + w * cap;
  int written = 0;
  for (int t0 = 0; t0 < n; t0 += 32) {
    const int t = t0 + lane;
    int j = 0;
    bool ok = false;
    if (t < n) {
      j = L[t];
      const float4 fj = fr[j];
      float dx = fi.x - fj.x, dy = fi.y - fj.y, dz = fi.z - fj.z;
      dx = (dx - rintf(dx)) * len.x;
      dy = (dy - rintf(dy)) * len.y;
      dz = (dz - rintf(dz)) * len.z;
      const float d2 = dx * dx + dy * dy + dz * dz;
      if (d2 < thr_hi) ok = d2 < thr_lo || exact_pair_in(g, pi, base + (long long)j * g.pstride);
    }
    const unsigned m = __ballot_sync(0xffffffffu, ok);
    const int pos = written + __popc(m & ((1u << lane) - 1u));
    if (ok && pos < cap) out[pos] = j;
    written += __popc(m);
  }
  if (lane == 0) {
    count[w] = min(written, cap);
    if (written > cap) atomicOr(status, ST_LIST_OVERFLOW);
  }
}

// ---- M-site substitution and scaling (md_forces.f90:179-188, ewald_cubic.f90:20-22) ----
// (zeroes the same entries of gz when given: the gradient buffer the Ewald
// kernels then accumulate into)
__global__ void k_msite(const double *r, double *rs, int nm, int B, double alpha, double alpha2,
                        double scale, double *gz) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nm * B * 3) return;
  const int d = (int)(t % 3);
  const long long mb = t / 3;  // molecule index over all configurations
  const double *m = r + mb * 9;
  double *o = rs + mb * 9;
  const double ro = alpha * m[d] + alpha2 * (m[3 + d] + m[6 + d]);
  o[d] = scale * ro;
  o[3 + d] = scale * m[3 + d];
  o[6 + d] = scale * m[6 + d];
  if (gz) {
    double *z = gz + mb * 9;
    z[d] = 0.0;
    z[3 + d] = 0.0;
    z[6 + d] = 0.0;
  }
}

// out = sign * chain_rule(scale * g)  (md_forces.f90:206-215)
__global__ void k_msite_chain(const double *g, const double *g2, double *out, int nm, int B, double alpha,
                              double alpha2, double scale, double sign, int accumulate, unsigned *status) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)nm * B * 3) return;
  const int d = (int)(t % 3);
  const long long mb = t / 3;
  const double *m = g + mb * 9;
  double *o = out + mb * 9;
  double m0 = m[d], m1 = m[3 + d], m2 = m[6 + d];
  if (g2) {  // a second gradient buffer (the real-space part, computed beside the k-space part)
    const double *n = g2 + mb * 9;
    m0 += n[d];
    m1 += n[3 + d];
    m2 += n[6 + d];
  }
  const double go = scale * m0;
  const double h1 = scale * m1 + alpha2 * go;
  const double h2 = scale * m2 + alpha2 * go;
  const double oo = alpha * go;
  gb_flag_nonfinite(status, gb_nonfinite(oo) || gb_nonfinite(h1) || gb_nonfinite(h2));
  if (accumulate) {
    o[d] += sign * oo;
    o[3 + d] += sign * h1;
    o[6 + d] += sign * h2;
  } else {
    o[d] = sign * oo;
    o[3 + d] = sign * h1;
    o[6 + d] = sign * h2;
  }
}

// ---- real-space Ewald (rwald, ewald_cubic.f90:78-233) in the unit box ----
// rwald (ewald_cubic.f90:78-233) on a pair list, FP64.  Per pair one rsqrt
// gives 1/dr, so that dr, erfc/dr and (sfac e - du)/dr^2 need no sqrt and no
// division; only t = p/(p + x) of the A&S 7.1.26 erfc approximation divides.
// The minimum image uses rint: every listed pair has drsq < wrcut^2 <= 1/4, so
// no component sits at a rounding tie, where rint and Fortran's nint differ.
// The virial is symmetric (dx dvy = dy dvx up to rounding): six sums, mirrored
// when the block sums are added.
//
// PAIR_NP adjacent lanes share one site's list (entries sub, sub + NP, ...),
// so that the grid holds enough warps to fill every SM; the site's own force
// is reduced over its lanes with shuffles before one atomic add.
constexpr int PAIR_NP = 8;
constexpr int PAIR_T = 64;

template <int NP>
GB_D double group_sum(double v) {
#pragma unroll
  for (int o = NP / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block sums of (v, xx, yx, zx, yy, zy, zz) into an accumulator slot laid out
// as v, vir(1..3, 1..3) column-major, the symmetric entries mirrored
GB_D void block_sum_sym7(double (&vals)[7], double *sh, double *acc) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int k = 0; k < 7; ++k) {
    const double v = warp_sum(vals[k]);
    if (lane == 0) sh[warp * 7 + k] = v;
  }
  __syncthreads();
  if (warp == 0) {
    constexpr int dst0[7] = {0, 1, 2, 3, 5, 6, 9};       // v, xx, yx, zx, yy, zy, zz
    constexpr int dst1[7] = {-1, -1, 4, 7, -1, 8, -1};   // mirrored xy, xz, yz
#pragma unroll
    for (int k = 0; k < 7; ++k) {
      double s2 = lane < nw ? sh[lane * 7 + k] : 0.0;
      s2 = warp_sum(s2);
      if (lane == 0 && s2 != 0.0) {
        atomicAdd(acc + dst0[k], s2);
        if (dst1[k] >= 0) atomicAdd(acc + dst1[k], s2);
      }
    }
  }
}

// NC: positions in bohr in a non-cubic box (rwald_basic / rwald_cell,
// ewald_noncubic.f90:56-273): minimum image dx - L nint(dx / L) per side
template <bool NC>
__global__ void __launch_bounds__(PAIR_T) k_ewald_real(const double *__restrict__ rs, const double *__restrict__ q,
                                                       int na, const int *__restrict__ count,
                                                       const int *__restrict__ idx, int cap, double alpha,
                                                       double3 box, double3 onbox, double *g, double *acc) {
  __shared__ double sh[32 * 7];
  const double p = 3.0525860, a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741,
               a4 = -1.453152027, a5 = 1.061405429;
  const double sfac = -2.0 * alpha / sqrt(acos(-1.0));
  const int c = blockIdx.y;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(tid / PAIR_NP), sub = (int)(tid % PAIR_NP);
  const bool active = i < na;
  double vals[7] = {0, 0, 0, 0, 0, 0, 0};  // v, xx, yx, zx, yy, zy, zz
  double fx = 0, fy = 0, fz = 0;
  const double *R = rs + (long long)c * na * 3;
  double *G = g + (long long)c * na * 3;
  if (active) {
    const double xi = R[3 * i], yi = R[3 * i + 1], zi = R[3 * i + 2], qi = q[i];
    const int mi = i / 3;
    const int n = min(count[(long long)c * na + i], cap);
    const int *L = idx + ((long long)c * na + i) * cap;
    for (int t = sub; t < n; t += PAIR_NP) {
      const int j = L[t];
      double dx = xi - R[3 * j], dy = yi - R[3 * j + 1], dz = zi - R[3 * j + 2];
      if (NC) {
        dx -= box.x * rint(dx * onbox.x);
        dy -= box.y * rint(dy * onbox.y);
        dz -= box.z * rint(dz * onbox.z);
      } else {
        dx -= rint(dx);
        dy -= rint(dy);
        dz -= rint(dz);
      }
      const double drsq = dx * dx + dy * dy + dz * dz;
      const double inv = rsqrt(drsq);
      const double x = alpha * (drsq * inv);
      const double e = exp(-x * x);
      const double tt = p / (p + x);
      double erfc = e * tt * (a1 + tt * (a2 + tt * (a3 + tt * (a4 + tt * a5))));
      if (mi == j / 3) erfc -= 1.0;
      const double du = erfc * inv;
      const double dur = (sfac * e - du) * (inv * inv);
      const double qij = qi * q[j];
      const double dv = qij * du, dvr = qij * dur;
      const double dvx = dvr * dx, dvy = dvr * dy, dvz = dvr * dz;
      fx += dvx;
      fy += dvy;
      fz += dvz;
      atomicAdd(G + 3 * j, -dvx);
      atomicAdd(G + 3 * j + 1, -dvy);
      atomicAdd(G + 3 * j + 2, -dvz);
      vals[0] += dv;
      vals[1] += dx * dvx;
      vals[2] += dy * dvx;
      vals[3] += dz * dvx;
      vals[4] += dy * dvy;
      vals[5] += dz * dvy;
      vals[6] += dz * dvz;
    }
  }
  fx = group_sum<PAIR_NP>(fx);
  fy = group_sum<PAIR_NP>(fy);
  fz = group_sum<PAIR_NP>(fz);
  if (active && sub == 0) {
    atomicAdd(G + 3 * i, fx);
    atomicAdd(G + 3 * i + 1, fy);
    atomicAdd(G + 3 * i + 2, fz);
  }
  block_sum_sym7(vals, sh, acc);
}

// ---- Lennard-Jones O-O (lj_list / lj_basic / lj_cell, ljones.f90) ----
// points are the oxygens; bead test with the same rounding as the reference
constexpr int LJ_NP = 4;

__global__ void __launch_bounds__(PAIR_T) k_lj(const double *r, int na, int npt, int nconf_list,
                                               const int *count, const int *idx, int cap,
                                               double sigsq, double rcutsq, double3 box, double3 onbox,
                                               double dscale, double *out, double *acc) {
  __shared__ double sh[32 * 10];
  const int c = blockIdx.y;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int o = (int)(tid / LJ_NP), sub = (int)(tid % LJ_NP);
  const bool active = o < npt;
  double vals[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  double fx = 0, fy = 0, fz = 0;
  const double *R = r + (long long)c * na * 3;
  double *F = out + (long long)c * na * 3;
  if (active) {
    const int lc = nconf_list == 1 ? 0 : c;
    const int n = min(count[(long long)lc * npt + o], cap);
    const int *L = idx + ((long long)lc * npt + o) * cap;
    const double xo = R[9 * o], yo = R[9 * o + 1], zo = R[9 * o + 2];
    for (int t = sub; t < n; t += LJ_NP) {
      const int j = L[t];
      double dx = __dsub_rn(R[9 * j], xo), dy = __dsub_rn(R[9 * j + 1], yo), dz = __dsub_rn(R[9 * j + 2], zo);
      dx = __dsub_rn(dx, __dmul_rn(box.x, nint_d(__dmul_rn(onbox.x, dx))));
      dy = __dsub_rn(dy, __dmul_rn(box.y, nint_d(__dmul_rn(onbox.y, dy))));
      dz = __dsub_rn(dz, __dmul_rn(box.z, nint_d(__dmul_rn(onbox.z, dz))));
      const double drsq = dsq3(dx, dy, dz);
      if (drsq < rcutsq) {
        const double onr2 = 1.0 / drsq;
        const double sr2 = sigsq * onr2;
        const double sr6 = sr2 * sr2 * sr2;
        const double vij = sr6 * (sr6 - 1.0);
        const double wij = sr6 * (sr6 - 0.5);
        const double fij = wij * onr2;
        const double dfx = fij * dx, dfy = fij * dy, dfz = fij * dz;
        atomicAdd(F + 9 * j, -dscale * dfx);
        atomicAdd(F + 9 * j + 1, -dscale * dfy);
        atomicAdd(F + 9 * j + 2, -dscale * dfz);
        fx += dfx;
        fy += dfy;
        fz += dfz;
        vals[0] += vij;
        vals[1] -= dx * dfx; vals[2] -= dy * dfx; vals[3] -= dz * dfx;
        vals[4] -= dx * dfy; vals[5] -= dy * dfy; vals[6] -= dz * dfy;
        vals[7] -= dx * dfz; vals[8] -= dy * dfz; vals[9] -= dz * dfz;
      }
    }
  }
  fx = group_sum<LJ_NP>(fx);
  fy = group_sum<LJ_NP>(fy);
  fz = group_sum<LJ_NP>(fz);
  if (active && sub == 0) {
    atomicAdd(F + 9 * o, dscale * fx);
    atomicAdd(F + 9 * o + 1, dscale * fy);
    atomicAdd(F + 9 * o + 2, dscale * fz);
  }
  block_sum_atomic<10>(vals, sh, acc);
}

// ---- TEM-switched correction (ewc_basic_tem / ewc_list_tem, correct_tem.f90) ----
__global__ void __launch_bounds__(128) k_tem(const double *rs, const double *q, int na,
                                             int nconf_list, const int *count, const int *idx,
                                             int cap, double rcutsq, double ta1, double ta2,
                                             double ta3, double3 box, double3 onbox, double *g,
                                             double *acc) {
  __shared__ double sh[32 * 10];
  const int c = blockIdx.y;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double vals[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (i < na) {
    const double *R = rs + (long long)c * na * 3;
    double *G = g + (long long)c * na * 3;
    const int lc = nconf_list == 1 ? 0 : c;
    const int n = min(count[(long long)lc * na + i], cap);
    const int *L = idx + ((long long)lc * na + i) * cap;
    const double xo = R[3 * i], yo = R[3 * i + 1], zo = R[3 * i + 2], qo = q[i];
    double fx = 0, fy = 0, fz = 0;
    for (int t = 0; t < n; ++t) {
      const int j = L[t];
      double dx = __dsub_rn(R[3 * j], xo), dy = __dsub_rn(R[3 * j + 1], yo), dz = __dsub_rn(R[3 * j + 2], zo);
      dx = __dsub_rn(dx, __dmul_rn(box.x, nint_d(__dmul_rn(onbox.x, dx))));
      dy = __dsub_rn(dy, __dmul_rn(box.y, nint_d(__dmul_rn(onbox.y, dy))));
      dz = __dsub_rn(dz, __dmul_rn(box.z, nint_d(__dmul_rn(onbox.z, dz))));
      const double drsq = dsq3(dx, dy, dz);
      if (drsq < rcutsq) {
        const double dr = sqrt(drsq);
        const double onr = 1.0 / dr;
        const double zij = q[j] * qo;
        const double vc = zij * onr;
        const double dvc = -vc * onr;
        const double dr3 = drsq * dr, dr4 = dr3 * dr;
        const double f = 1.0 - ta1 * dr + ta2 * dr3 - ta3 * dr4;
        const double df = -ta1 + 3.0 * ta2 * drsq - 4.0 * ta3 * dr3;
        const double dv = vc * f;
        const double dvr = vc * df + dvc * f;
        const double dvx = dvr * dx * onr, dvy = dvr * dy * onr, dvz = dvr * dz * onr;
        atomicAdd(G + 3 * j, dvx);
        atomicAdd(G + 3 * j + 1, dvy);
        atomicAdd(G + 3 * j + 2, dvz);
        fx -= dvx;
        fy -= dvy;
        fz -= dvz;
        vals[0] += dv;
        vals[1] += dx * dvx; vals[2] += dy * dvx; vals[3] += dz * dvx;
        vals[4] += dx * dvy; vals[5] += dy * dvy; vals[6] += dz * dvy;
        vals[7] += dx * dvz; vals[8] += dy * dvz; vals[9] += dz * dvz;
      }
    }
    atomicAdd(G + 3 * i, fx);
    atomicAdd(G + 3 * i + 1, fy);
    atomicAdd(G + 3 * i + 2, fz);
  }
  block_sum_atomic<10>(vals, sh, acc);
}

// centroid rc = (sum_b r_b) / B per coordinate row, beads summed in order
__global__ void k_centroid(const double *r, double *rc, int na, int B) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long S = 3LL * na;
  if (t >= S) return;
  double s = 0.0;
  for (int b = 0; b < B; ++b) s = s + r[t + S * b];
  rc[t] = s / (double)B;
}

// Shared list of B configurations (ListSpread): each site's centroid over the
// configurations (as k_centroid), and the largest squared distance of a
// configuration's site from its centroid, max-reduced into sp.w[0].  A site
// beyond the list's margin (sp.w[1]) asks for a rebuild (moved); one beyond
// the stencil's cap (the largest margin the list can take) is an error.
__global__ void k_site_centroid(const double *r, double *cen, int na, int B, ListSpread sp, unsigned *moved,
                                unsigned *status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  float d2 = 0.0f;
  if (i < na) {
    const long long S = 3LL * na;
    double c[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      double s = 0.0;
      for (int b = 0; b < B; ++b) s = s + r[S * b + 3 * i + d];
      c[d] = s / (double)B;
      cen[3 * i + d] = c[d];
    }
    for (int b = 0; b < B; ++b) {
      const double *x = r + S * b + 3 * i;
      const float dx = (float)(x[0] - c[0]), dy = (float)(x[1] - c[1]), dz = (float)(x[2] - c[2]);
      d2 = fmaxf(d2, dx * dx + dy * dy + dz * dz);
    }
    if (!(d2 <= sp.dcap * sp.dcap)) atomicOr(status, ST_LIST_OVERFLOW);  // NaN too
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) d2 = fmaxf(d2, __shfl_xor_sync(0xffffffffu, d2, o));
  if ((threadIdx.x & 31) == 0) {
    if (d2 > 0.0f) atomicMax(reinterpret_cast<int *>(sp.w), __float_as_int(d2));  // non-negative: int order
    if (d2 > *(volatile float *)(sp.w + 1)) atomicOr(moved, 1u);
  }
}

// the margin of a shared list at a rebuild (the all-pairs build; the
// cell-sorted one takes it in k_cell_count), and the next step's spread word
__global__ void k_spread_update(const unsigned *flag, ListSpread sp) {
  volatile float *w = sp.w;
  if (*flag) {
    const float dres = fminf(sp.dcap, 1.25f * sqrtf(w[0]) + sp.dmin);
    const float rl = sp.base + 2.0f * dres;
    w[1] = dres * dres;
    w[2] = rl * rl * (1.0f + 1e-5f);
  }
  w[0] = 0.0f;
}

// fixed-point coordinates of B configurations (fx [B][npt]) and, with slot_of
// (the shared list's cell-order slots), the same in slot order (fxs)
__global__ void k_fx_slots(PairGeom g, int B, const double *q, const int *slot_of, int4 *fx, int4 *fxs) {
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= (long long)B * g.npt) return;
  const int c = (int)(t / g.npt), i = (int)(t % g.npt);
  const int4 v = fixed_point(g, c, i, q);
  fx[t] = v;
  if (fxs) fxs[(long long)c * g.npt + slot_of[i]] = v;
}

__global__ void k_sum_counts(const int *count, long long n, unsigned long long *out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long v = t < n ? (unsigned long long)count[t] : 0ull;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(out, v);
}

__global__ void k_max_count(const int *count, long long n, int *out) {
  long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  int v = t < n ? count[t] : 0;
  for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
  if ((threadIdx.x & 31) == 0 && v) atomicMax(out, v);
}

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// longest list (diagnostics only: synchronises the stream)
int list_max(cudaStream_t s, const PairList &pl) {
  if (!pl.count || pl.nconf <= 0 || pl.npt <= 0) return 0;
  int *d = nullptr, h = 0;
  if (cudaMalloc(&d, sizeof(int)) != cudaSuccess) return -1;
  cudaMemsetAsync(d, 0, sizeof(int), s);
  long long n = (long long)pl.nconf * pl.npt;
  k_max_count<<<nblk(n, 256), 256, 0, s>>>(pl.count, n, d);
  cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  cudaFree(d);
  return h;
}

// total entries of a pair list (profiling only: synchronises the stream)
double list_total(cudaStream_t s, const PairList &pl) {
  unsigned long long *d = nullptr, h = 0;
  if (cudaMalloc(&d, sizeof(unsigned long long)) != cudaSuccess) return 0.0;
  cudaMemsetAsync(d, 0, sizeof(unsigned long long), s);
  long long n = (long long)pl.nconf * pl.npt;
  k_sum_counts<<<nblk(n, 256), 256, 0, s>>>(pl.count, n, d);
  cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  cudaFree(d);
  return (double)h;
}

void launch_frac32(cudaStream_t s, const PairGeom &g, int nconf, float4 *frac, float4 *lo, const double *q,
                   int4 *fx) {
  long long n = (long long)nconf * g.npt;
  k_frac32<<<nblk(n, 256), 256, 0, s>>>(g, nconf, frac, lo, q, fx);
}

// FP32 thresholds around rcutsq: below lo accept, at or above hi reject,
// between: exact FP64 test
void list_thresholds(const PairGeom &g, float3 *len, float *lo, float *hi) {
  double lmax;
  if (g.unit) {
    *len = make_float3(1.f, 1.f, 1.f);
    lmax = 1.0;
  } else {
    *len = make_float3((float)g.box[0], (float)g.box[1], (float)g.box[2]);
    lmax = fmax(g.box[0], fmax(g.box[1], g.box[2]));
  }
  // FP32 error of d^2 is below 1e-6 * lmax^2 for wrapped fractional coordinates;
  // pairs within 4e-6 * lmax^2 of the cut-off go to the exact FP64 test
  const double band = 4e-6 * lmax * lmax;
  *lo = (float)(g.rcutsq - band);
  *hi = (float)(g.rcutsq + band);
}

void launch_build_list(cudaStream_t s, const PairGeom &g, int nconf, const float4 *frac,
                       PairList &pl, unsigned *status, const unsigned *gate, const float *thr_dev) {
  float3 len;
  float thr_lo, thr_hi;
  list_thresholds(g, &len, &thr_lo, &thr_hi);
  const long long ncount = (long long)nconf * g.npt;
  if (gate) k_skin_zero<<<nblk(ncount, 256), 256, 0, s>>>(pl.count, ncount, gate);
  else cudaMemsetAsync(pl.count, 0, sizeof(int) * (size_t)ncount, s);
  // partner chunks of 1024 points, halved until the grid has ~4 blocks per SM
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  int jchunk = 1024;
  const long long bi = (long long)nblk(g.npt, LB_T) * nconf;
  while (jchunk > LB_T && bi * (long long)nblk(g.npt, jchunk) < 4LL * nsm) jchunk /= 2;
  dim3 grid(nblk(g.npt, LB_T), nblk(g.npt, jchunk), nconf);
  auto go = [&](auto kern) {
    kern<<<grid, LB_T, 0, s>>>(g, frac, pl.count, pl.idx, pl.cap, len, thr_lo, thr_hi, status, gate, jchunk,
                               thr_dev);
  };
  if (g.full) {
    if (g.excl_mol) go(k_build_list2<true, true>);
    else go(k_build_list2<true, false>);
  } else {
    if (g.excl_mol) go(k_build_list2<false, true>);
    else go(k_build_list2<false, false>);
  }
}

void launch_skin_check(cudaStream_t s, const PairGeom &g, int nconf, const double *ref, double lim2,
                       unsigned *flag) {
  const long long n = (long long)nconf * g.npt;
  k_skin_check<<<nblk(n, 256), 256, 0, s>>>(g, nconf, ref, lim2, flag);
}

void launch_skin_save(cudaStream_t s, const PairGeom &g, int nconf, double *ref, const unsigned *flag,
                      unsigned *rebuilds) {
  const long long n = (long long)nconf * g.npt;
  k_skin_save<<<nblk(n, 256), 256, 0, s>>>(g, nconf, ref, flag, rebuilds);
}

// The cell grid of a superset build: cells of side >= 1/R of the largest
// accepted distance (R = 1..CELL_RMAX, 2R + 1 cells per axis at least), the
// stencil pruned to the cells that can hold a pair within that distance (with
// a margin for the FP32 cell index), and the R of the lowest estimated scan
// cost (stencil points plus a fixed cost per stencil row); false when even
// that exceeds 60 % of an all-pairs scan (the all-pairs build is used).
bool list_cell_grid(const PairGeom &g, int nc[3], int *R, signed char *reach) {
  float3 len;
  float thr_lo, thr_hi;
  list_thresholds(g, &len, &thr_lo, &thr_hi);
  const double cut = std::sqrt((double)thr_hi) * (1.0 + 1e-5);
  const double cut2 = cut * cut * (1.0 + 1e-4);
  const double L[3] = {len.x, len.y, len.z};
  double best = 0.6;  // estimated cost per point, in all-pairs scans
  bool found = false;
  for (int r = 1; r <= CELL_RMAX; ++r) {
    int n[3];
    bool ok = true;
    double side[3];
    for (int d = 0; d < 3; ++d) {
      n[d] = (int)std::min(std::floor(L[d] * r / cut), 128.0);
      ok = ok && n[d] >= 2 * r + 1;
      side[d] = L[d] / std::max(n[d], 1) * (1.0 - 1e-5);
    }
    if (!ok) continue;
    const double ncell = (double)n[0] * n[1] * n[2];
    auto gap = [](int o, double s) {
      const double q = std::max(0, std::abs(o) - 1) * s;
      return q * q;
    };
    signed char rr[(2 * CELL_RMAX + 1) * (2 * CELL_RMAX + 1)];
    double cells = 0.0, rows = 0.0;
    for (int oz = -r; oz <= r; ++oz)
      for (int oy = -r; oy <= r; ++oy) {
        const double dyz = gap(oy, side[1]) + gap(oz, side[2]);
        int rx = -1;
        for (int ox = 0; ox <= r; ++ox)
          if (dyz + gap(ox, side[0]) < cut2) rx = ox;
        rr[(oz + r) * (2 * r + 1) + (oy + r)] = (signed char)rx;
        if (rx >= 0) {
          cells += 2 * rx + 1;
          rows += 1.0;
        }
      }
    const double cost = cells / ncell + rows * 24.0 / std::max(1, g.npt);
    if (cost < best) {
      best = cost;
      found = true;
      *R = r;
      for (int d = 0; d < 3; ++d) nc[d] = n[d];
      std::memcpy(reach, rr, sizeof rr);
    }
  }
  return found;
}

static_assert(sizeof(CellSort::reach) == sizeof(CellSortDev::reach), "stencil table sizes");

CellSortDev dev_cells(const CellSort &cs) {
  CellSortDev d{};
  d.nx = cs.nc[0];
  d.ny = cs.nc[1];
  d.nz = cs.nc[2];
  d.R = cs.R;
  std::memcpy(d.reach, cs.reach, sizeof d.reach);
  d.ccount = cs.ccount;
  d.cstart = cs.cstart;
  d.cellid = cs.cellid;
  d.crank = cs.crank;
  d.spos = cs.spos;
  d.sidx = cs.sidx;
  d.slot_of = cs.slot_of;
  d.fxs = cs.fxs;
  d.ticket = cs.ticket;
  return d;
}

// skin test and cell counts (every step), then, gated by flag, the cell-order
// scatter (which also zeroes the list counts) and the build
void launch_cell_count(cudaStream_t s, const PairGeom &g, int nconf, float4 *frac, float4 *lo, const double *q,
                       const CellSort &cs, const double *ref, double lim2, int check, unsigned *flag, int4 *fx,
                       const ListSpread &sp) {
  CellSortDev d = dev_cells(cs);
  const long long n = (long long)nconf * g.npt;
  k_cell_count<<<nblk(n, 256), 256, 0, s>>>(g, nconf, frac, lo, q, d, ref, lim2, check, flag, fx, sp);
}

void launch_site_centroid(cudaStream_t s, const double *r, double *cen, int na, int B, const ListSpread &sp,
                          unsigned *moved, unsigned *status) {
  k_site_centroid<<<nblk(na, 128), 128, 0, s>>>(r, cen, na, B, sp, moved, status);
}

void launch_spread_update(cudaStream_t s, const unsigned *flag, const ListSpread &sp) {
  k_spread_update<<<1, 1, 0, s>>>(flag, sp);
}

void launch_fx_slots(cudaStream_t s, const PairGeom &g, int B, const double *q, const int *slot_of, int4 *fx,
                     int4 *fxs) {
  k_fx_slots<<<nblk((long long)B * g.npt, 256), 256, 0, s>>>(g, B, q, slot_of, fx, fxs);
}

void launch_build_sorted(cudaStream_t s, const PairGeom &g, int nconf, const float4 *frac, PairList &pl,
                         unsigned *status, const unsigned *gate, const CellSort &cs, double *ref,
                         unsigned *rebuilds, const int4 *fx, const float *thr_dev) {
  float3 len;
  float thr_lo, thr_hi;
  list_thresholds(g, &len, &thr_lo, &thr_hi);
  CellSortDev d = dev_cells(cs);
  const long long n = (long long)nconf * g.npt;
  k_cell_scatter<<<nblk(n, 256), 256, 0, s>>>(g, nconf, frac, d, pl.count, gate, ref, rebuilds, fx);
  auto go = [&](auto kern, auto *idx) {
    kern<<<nblk(32 * n, LB_T), LB_T, 0, s>>>(g, nconf, d, pl.count, idx, pl.cap, len, thr_lo, thr_hi, status,
                                             gate, thr_dev);
  };
  unsigned short *i16 = reinterpret_cast<unsigned short *>(pl.idx);
  if (pl.slots) {  // never with exclusions
    if (g.full) go(k_build_sorted<true, false, unsigned short, true>, i16);
    else go(k_build_sorted<false, false, unsigned short, true>, i16);
  } else if (g.full) {
    if (g.excl_mol) pl.i16 ? go(k_build_sorted<true, true, unsigned short>, i16) : go(k_build_sorted<true, true, int>, pl.idx);
    else pl.i16 ? go(k_build_sorted<true, false, unsigned short>, i16) : go(k_build_sorted<true, false, int>, pl.idx);
  } else {
    if (g.excl_mol) pl.i16 ? go(k_build_sorted<false, true, unsigned short>, i16) : go(k_build_sorted<false, true, int>, pl.idx);
    else pl.i16 ? go(k_build_sorted<false, false, unsigned short>, i16) : go(k_build_sorted<false, false, int>, pl.idx);
  }
}

void launch_list_filter(cudaStream_t s, const PairGeom &g, int nconf, const float4 *frac,
                        const PairList &skin, PairList &pl, unsigned *status) {
  float3 len;
  float thr_lo, thr_hi;
  list_thresholds(g, &len, &thr_lo, &thr_hi);
  const long long nw = (long long)nconf * g.npt;
  if (skin.i16)
    k_list_filter<unsigned short><<<nblk(nw * 32, 128), 128, 0, s>>>(
        g, nconf, frac, skin.count, reinterpret_cast<const unsigned short *>(skin.idx), skin.cap, pl.count, pl.idx,
        pl.cap, len, thr_lo, thr_hi, status);
  else
    k_list_filter<int><<<nblk(nw * 32, 128), 128, 0, s>>>(g, nconf, frac, skin.count, skin.idx, skin.cap, pl.count,
                                                        pl.idx, pl.cap, len, thr_lo, thr_hi, status);
}

void launch_msite(cudaStream_t s, const double *r, double *rs, int na, int B, double alpha,
                  double scale, double *gz) {
  int nm = na / 3;
  long long n = (long long)nm * B * 3;
  k_msite<<<nblk(n, 256), 256, 0, s>>>(r, rs, nm, B, alpha, 0.5 * (1.0 - alpha), scale, gz);
}

void launch_msite_chain(cudaStream_t s, const double *g, double *out, int na, int B, double alpha,
                        double scale, double sign, int accumulate, const double *g2, unsigned *status) {
  int nm = na / 3;
  long long n = (long long)nm * B * 3;
  k_msite_chain<<<nblk(n, 256), 256, 0, s>>>(g, g2, out, nm, B, alpha, 0.5 * (1.0 - alpha), scale, sign,
                                             accumulate, status);
}

void launch_ewald_real(cudaStream_t s, const double *rs, const double *q, int na, int B,
                       const PairList &pl, double alpha, const double *box, double *g, double *acc) {
  dim3 grid(nblk((long long)na * PAIR_NP, PAIR_T), B);
  if (box) {
    const double3 bx = make_double3(box[0], box[1], box[2]);
    const double3 ob = make_double3(1.0 / box[0], 1.0 / box[1], 1.0 / box[2]);
    k_ewald_real<true><<<grid, PAIR_T, 0, s>>>(rs, q, na, pl.count, pl.idx, pl.cap, alpha, bx, ob, g, acc);
  } else {
    const double3 one = make_double3(1.0, 1.0, 1.0);
    k_ewald_real<false><<<grid, PAIR_T, 0, s>>>(rs, q, na, pl.count, pl.idx, pl.cap, alpha, one, one, g, acc);
  }
}

void launch_lj(cudaStream_t s, const double *r, int na, int B, const PairList &pl, double sigsq,
               double rcutsq, const double *box, double dscale, double *out, double *acc) {
  int npt = na / 3;
  dim3 grid(nblk((long long)npt * LJ_NP, PAIR_T), B);
  double3 bx = make_double3(box[0], box[1], box[2]);
  double3 ob = make_double3(1.0 / box[0], 1.0 / box[1], 1.0 / box[2]);
  k_lj<<<grid, PAIR_T, 0, s>>>(r, na, npt, pl.nconf, pl.count, pl.idx, pl.cap, sigsq, rcutsq, bx, ob,
                            dscale, out, acc);
}

void launch_tem(cudaStream_t s, const double *rs, const double *q, int na, int B,
                const PairList &pl, double sig, const double *box, double *g, double *acc) {
  dim3 grid(nblk(na, 128), B);
  double3 bx = make_double3(box[0], box[1], box[2]);
  double3 ob = make_double3(1.0 / box[0], 1.0 / box[1], 1.0 / box[2]);
  const double a1 = 2.0 / sig, a2 = 2.0 / (sig * sig * sig), a3 = 1.0 / (sig * sig * sig * sig);
  k_tem<<<grid, 128, 0, s>>>(rs, q, na, pl.nconf, pl.count, pl.idx, pl.cap, sig * sig, a1, a2, a3,
                             bx, ob, g, acc);
}

void launch_centroid(cudaStream_t s, const double *r, double *rc, int na, int B) {
  long long n = 3LL * na;
  k_centroid<<<nblk(n, 256), 256, 0, s>>>(r, rc, na, B);
}
