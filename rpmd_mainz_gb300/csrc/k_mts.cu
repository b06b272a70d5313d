// k_mts.cu -- the multiple-time-step block of evolve_pi in one kernel (FP64).
//
// evolve_pi.f90:82-161 and 222-228: the opening kicks, the forward normal-mode
// transforms of p and r, mts substeps of {free ring-polymer rotation, back
// transform of r, intramolecular forces on every bead, virial kinetic-energy
// partial sums, forward transform of the forces and the momentum kick}, and the
// closing back transform of p with the last half kick.  None of these couples
// different molecules, so one block owns whole ring polymers of MPB molecules:
// each of its 9*MPB threads holds one coordinate row (atom, xyz) of p and r in
// registers and runs the transforms in registers (gb_fft.cuh); the bead
// positions and intramolecular forces of a substep pass between the row view
// and the (molecule, bead) view through shared memory.  HBM traffic per step is
// one read of p, r, dvdr, dvdr2 (dvdr once more per substep for the estimator)
// and one write of p, r, rnm, dvdr2.
#include "gb_common.cuh"
#include "gb_df.cuh"
#include "gb_fft.cuh"
#include "gb_intra.cuh"
#include "gb_kernels.h"

#include <algorithm>
#include <cmath>

namespace {

// A block owns mpb molecules (chosen at launch so that the grid is one wave
// over the SMs, at most MPB_MAX) and runs 9 * mpb threads, one per coordinate
// row, rounded up to whole warps; the extra lanes of the last warp carry rows
// of no molecule and store nothing.
// At most 8 warps (28 molecules, 252 rows) keep two warps per SM sub-partition,
// which leaves 255 registers per thread for the register-resident rows.
template <int NB>
struct MtsCfg {
  static constexpr int MPB_MAX = NB <= 32 ? 28 : 14;
  static constexpr int T_MAX = (9 * MPB_MAX + 31) / 32 * 32;
  static constexpr int LD = NB + 1;  // padded bead stride in shared memory
};

struct MtsArgs {
  double *p, *r, *rnm, *dvdr2;
  const double *dvdr;
  const double *monod;  // monod(ic, c, k) at ic + 3*(c + 4*k)
  const double *tw;     // twiddles of length nb
  double *acc_int, *acc_ke;
  unsigned *status;  // ST_NONFINITE when a force or momentum written is not finite
  int na, nm, mts, model, mpb;
  double halfdt, dtsmall, halfdtsmall;
  float hdt_h, hdt_l, hds_h, hds_l;  // halfdt and halfdtsmall as FP32 pairs (mixed kernel)
  double sc;                          // sqrt(1/nb)
  // mixed kernel: ring_contract (evolve_pi.f90:405-431) of the new positions
  // into rb1 / rb2 (nullptr: not fused) with nbc1 / nbc2 <= MTS_NBC beads,
  // twiddles tw_c1 / tw_c2, scale s12 = sqrt(1/nbc) sqrt(nbc/nb)
  double *rb1, *rb2;
  int nbc1, nbc2;
  const double *tw_c1, *tw_c2;
  double s12_1, s12_2;
  IntraPar ip;
};
constexpr int MTS_NBC = 9;  // longest contracted ring written by the mixed kernel

template <int NB>
__global__ void __launch_bounds__(MtsCfg<NB>::T_MAX, 1) k_mts_fused(MtsArgs a) {
  using C = MtsCfg<NB>;
  extern __shared__ double sm[];
  const int T = blockDim.x;
  const int nrow = (T + 8) / 9 * 9;                // rows with shared-memory slots
  double *s_rst = sm;                              // [nrow][LD]
  double *s_f2 = s_rst + nrow * C::LD;             // [nrow][LD]
  double *s_mono = s_f2 + nrow * C::LD;            // [12*NB]
  double *s_tw = s_mono + 12 * NB;                 // [2*NB] cos, sin
  double *s_twf = s_tw + 2 * NB;                   // [2*NB] scaled by sqrt(1/nb) / 2 (forward)
  double *s_twi = s_twf + 2 * NB;                  // [2*NB] scaled by sqrt(1/nb) (inverse)
  double *s_red = s_twi + 2 * NB;                  // [32 warps][18]
  const int t = threadIdx.x;
  const double sc = a.sc;
  for (int i = t; i < 12 * NB; i += T) s_mono[i] = a.monod[i];
  for (int i = t; i < 2 * NB; i += T) {
    const double w = a.tw[i];
    s_tw[i] = w;
    s_twf[i] = (0.5 * sc) * w;
    s_twi[i] = sc * w;
  }

  // Every thread runs the same instruction stream between barriers: rows past
  // the last molecule (or past the block's mpb) work on a copy of the last
  // molecule and store nothing.
  const int mpb = a.mpb;
  const int m0 = blockIdx.x * mpb;
  const int ml = t / 9, lr = t % 9;           // local molecule, row within molecule
  const int m = m0 + ml;
  const bool valid = ml < mpb && m < a.nm;
  const int mc = valid ? m : a.nm - 1;        // molecule whose data this row reads
  const long long S = 3LL * a.na;             // stride between beads
  const long long row = 9LL * mc + lr;        // global coordinate row
  const int ic = lr / 3;                      // atom type O, H, H
  const int xyz = lr % 3;

  double p[NB], x[NB];
#pragma unroll
  for (int j = 0; j < NB; ++j) {
    const double pj = a.p[row + S * j] - a.halfdt * a.dvdr[row + S * j];
    p[j] = pj - a.halfdtsmall * a.dvdr2[row + S * j];
    x[j] = a.r[row + S * j];
  }
  __syncthreads();
  gb_r2hc_s<NB>([&](int j) { return p[j]; }, [&](int k, double v) { p[k] = v; }, s_tw, s_twf);
  gb_r2hc_s<NB>([&](int j) { return x[j]; }, [&](int k, double v) { x[k] = v; }, s_tw, s_twf);

  double e_last = 0.0, vir[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  double q1 = 0.0, q2 = 0.0;
  for (int im = 1; im <= a.mts; ++im) {
    {
      // free ring-polymer rotation (evolve_pi.f90:109-125)
#pragma unroll
      for (int k = 0; k < NB; ++k) {
        const double *mo = s_mono + ic + 12 * k;
        const double pp = p[k] * mo[0] + x[k] * mo[3];
        x[k] = p[k] * mo[6] + x[k] * mo[9];
        p[k] = pp;
      }
      // bead positions rst = HC2R(r) (evolve_pi.f90:141-145)
      double *dst = s_rst + (ml * 9 + lr) * C::LD;
      gb_hc2r_s<NB>([&](int j) { return x[j]; }, [&](int k, double v) { dst[k] = v; }, s_tw, s_twi);
    }
    __syncthreads();
    // intramolecular forces per (molecule, bead) (forces(rst, ..., 4)); rows of
    // molecules past the end hold copies and are left out of the sums
    double e_sub = 0.0;
    for (int idx = t; idx < mpb * NB; idx += T) {
      const int mm = idx / NB, j = idx % NB;
      const double w = (m0 + mm < a.nm) ? 1.0 : 0.0;
      double xm[9], fm[9], vm[9];
#pragma unroll
      for (int d = 0; d < 9; ++d) xm[d] = s_rst[(mm * 9 + d) * C::LD + j];
      e_sub += w * intra_molecule(a.model, xm, fm, vm, a.ip);
#pragma unroll
      for (int d = 0; d < 9; ++d) {
        s_f2[(mm * 9 + d) * C::LD + j] = fm[d];
        vir[d] += w * vm[d];
      }
    }
    if (im == a.mts) e_last = e_sub;
    __syncthreads();
    {
      // virial_ke partial sums (kinetic.f90:23-40)
      const double *rs_row = s_rst + (ml * 9 + lr) * C::LD;
      const double *f2_row = s_f2 + (ml * 9 + lr) * C::LD;
      double rc = 0.0;
#pragma unroll
      for (int j = 0; j < NB; ++j) rc = rc + rs_row[j];
      rc = rc / (double)NB;
      if (valid) {  // rows of no molecule have no intramolecular forces in s_f2
#pragma unroll
        for (int j = 0; j < NB; ++j) {
          const double dr = rs_row[j] - rc;
          q1 += dr * a.dvdr[row + S * j];
          q2 += dr * f2_row[j];
        }
      }
      if (im != a.mts) {  // FT(dvdr2) and p -= dtsmall dvdr2 (evolve_pi.f90:156-159)
        const double dts = a.dtsmall;
        gb_r2hc_s<NB>([&](int j) { return f2_row[j]; }, [&](int k, double v) { p[k] = p[k] - dts * v; },
                      s_tw, s_twf);
      }
    }
    if (im != a.mts) __syncthreads();
  }
  {
    // back to beads: p = HC2R(p); r = rst; p -= halfdtsmall dvdr2 (evolve_pi.f90:222-228)
    const double *rs_row = s_rst + (ml * 9 + lr) * C::LD;
    const double *f2_row = s_f2 + (ml * 9 + lr) * C::LD;
    const double hds = a.halfdtsmall;
    double *gp = a.p + row;
    bool bad = false;
    gb_hc2r_s<NB>([&](int j) { return p[j]; },
                  [&](int k, double v) {
                    const double pk = v - hds * f2_row[k];
                    bad |= gb_nonfinite(pk);
                    if (valid) gp[S * k] = pk;
                  }, s_tw, s_twi);
    if (valid) {
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        a.r[row + S * j] = rs_row[j];
        a.rnm[row + S * j] = x[j];
        a.dvdr2[row + S * j] = f2_row[j];
        bad |= gb_nonfinite(f2_row[j]);
      }
    }
    gb_flag_nonfinite(a.status, bad && valid);
  }
  // block sums: [0] last-substep intra energy, [1..9] intra virial summed over
  // substeps, [10] tq1, [11] tq2, [12..14] tq1 per xyz, [15..17] tq2 per xyz
  double red[18];
  red[0] = e_last;
#pragma unroll
  for (int d = 0; d < 9; ++d) red[1 + d] = vir[d];
  red[10] = q1;
  red[11] = q2;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    red[12 + d] = d == xyz ? q1 : 0.0;
    red[15 + d] = d == xyz ? q2 : 0.0;
  }
  const int lane = t & 31, warp = t >> 5, nw = (T + 31) / 32;
#pragma unroll
  for (int i = 0; i < 18; ++i) {
    double v = warp_sum(red[i]);
    if (lane == 0) s_red[warp * 18 + i] = v;
  }
  __syncthreads();
  if (t < 18) {
    double s = 0.0;
    for (int w = 0; w < nw; ++w) s += s_red[w * 18 + t];
    if (s != 0.0) {
      if (t < 10) atomicAdd(a.acc_int + t, s);
      else if (t < 12) atomicAdd(a.acc_ke + (t - 10), s);
      else atomicAdd(a.acc_ke + 2 + (t - 12), s);
    }
  }
}

// Mixed precision (same structure as k_mts_fused).  The centroid mode of p and
// r stays FP64 (its bead sums, its free step and its kicks); the other normal
// modes live in FP32 registers.  Their free ring-polymer rotation uses each
// FP64 coefficient split into FP32 hi + lo, so that the rotation keeps its
// unit determinant to ~1e-14 (a coefficient rounded to FP32 alone would make
// the mode amplitudes grow or shrink steadily); the products and the states
// round to FP32, which is noise.  Every transform runs in FP32 on deviations:
// the centroid mode is the FP64 bead sum, the other modes come from an FP32
// transform of x_j - x_0.  The intramolecular forces run in FP32 on positions
// taken relative to the molecule's oxygen centroid, so that FP32 holds them to
// ~1e-7 bohr.
template <int NB>
// Two blocks per SM: the FP32 modes need about half the registers of the FP64
// kernel, so 128 per thread (a few spilled at nb = 64) give twice the warps.
__global__ void __launch_bounds__(MtsCfg<NB>::T_MAX, 2) k_mts_mixed(MtsArgs a) {
  using C = MtsCfg<NB>;
  extern __shared__ double sm[];
  const int T = blockDim.x;
  const int nrow = (T + 8) / 9 * 9;
  const int nf = (3 * nrow * C::LD + 1) & ~1;      // float slots, rounded to whole doubles
  float *s_dev = reinterpret_cast<float *>(sm);    // [nrow][LD] x_j - (oxygen centroid)
  float *s_f2 = s_dev + nrow * C::LD;              // [nrow][LD] intramolecular forces
  float *s_dvf = s_f2 + nrow * C::LD;              // [nrow][LD] dvdr for the estimator
  double *s_cen = sm + nf / 2;                     // [nrow] row centroids
  double *s_mono = s_cen + nrow;                   // [12] monodromy of the centroid mode
  double *s_red = s_mono + 12;                     // [32 warps][18]
  float *s_mh = reinterpret_cast<float *>(s_red + 32 * 18);  // [12*NB] coefficients, hi
  float *s_ml = s_mh + 12 * NB;                    // [12*NB] and lo parts
  float *s_tw = s_ml + 12 * NB;                    // [2*NB] cos, sin
  float *s_twf = s_tw + 2 * NB;                    // scaled by sqrt(1/nb) / 2
  float *s_twi = s_twf + 2 * NB;                   // scaled by sqrt(1/nb)
  float *s_tw_l = s_twi + 2 * NB;                  // lo parts of the three tables
  float *s_twf_l = s_tw_l + 2 * NB;
  float *s_twi_l = s_twf_l + 2 * NB;
  float *s_ct = s_twi_l + 2 * NB;                  // [2][2*MTS_NBC] contraction cos, sin
  const int t = threadIdx.x;
  const double sc = a.sc;
  // FP32 hi + lo splits of the tables (d2df: integer operations, no FP64
  // conversions)
  for (int i = t; i < 12 * NB; i += T) {
    const double w = a.monod[i];
    d2df(w, s_mh[i], s_ml[i]);
    if (i < 12) s_mono[i] = w;
  }
  for (int i = t; i < 2 * NB; i += T) {
    const double w = a.tw[i], wf = (0.5 * sc) * w, wi = sc * w;
    d2df(w, s_tw[i], s_tw_l[i]);
    d2df(wf, s_twf[i], s_twf_l[i]);
    d2df(wi, s_twi[i], s_twi_l[i]);
  }
  for (int i = t; i < 4 * MTS_NBC; i += T) {
    const int q = i / (2 * MTS_NBC), e = i % (2 * MTS_NBC);
    const double *tw = q ? a.tw_c2 : a.tw_c1;
    const int nbc = q ? a.nbc2 : a.nbc1;
    const double *rb = q ? a.rb2 : a.rb1;
    s_ct[i] = rb && e < 2 * nbc ? d2f(tw[e]) : 0.f;
  }
  const int mpb = a.mpb;
  const int m0 = blockIdx.x * mpb;
  const int ml = t / 9, lr = t % 9;
  const int m = m0 + ml;
  const bool valid = ml < mpb && m < a.nm;
  const int mc = valid ? m : a.nm - 1;
  const long long S = 3LL * a.na;
  const long long row = 9LL * mc + lr;
  const int ic = lr / 3;
  const int xyz = lr % 3;
  const int orow = ml * 9 + xyz;                   // oxygen row of the same coordinate
  float *dv_row = s_dvf + t * C::LD;

  // The opening kicks and the forward transforms without per-element FP64
  // instructions.  Momenta: the forces become FP32 (integer-built rounding) and
  // the kick p - halfdt dvdr - halfdtsmall dvdr2 (evolve_pi.f90:82-83) is
  // formed in FP32 with hi + lo coefficients; the bead momenta of a ring are
  // independent draws, so FP32 holds them to the precision of their spread.
  // Positions: each bead's deviation from bead 0, (hi_j - hi_0) + (lo_j - lo_0)
  // from integer-built hi + lo splits, so that FP32 keeps ~2^-24 of the
  // deviation rather than of the coordinate.  The centroid modes take
  // compensated (Kahan) FP32 bead sums and one FP64 product each; modes k >= 1
  // come from the FP32 transform with split twiddles (the state's round trip:
  // no systematic gain per step).
  double p0, x0;
  float pf[NB], xf[NB];
  {
    float d[NB];
    float ch = 0.f, cc = 0.f;  // Kahan sum and its running compensation
    auto kahan = [&](float v) {
      const float y = v - cc;
      const float t2 = ch + y;
      cc = (t2 - ch) - y;
      ch = t2;
    };
#pragma unroll
    for (int j = 0; j < NB; ++j) {
      const float dv = d2f(a.dvdr[row + S * j]), dv2 = d2f(a.dvdr2[row + S * j]);
      dv_row[j] = dv;
      const float kick = fmaf(a.hdt_h, dv, fmaf(a.hdt_l, dv, fmaf(a.hds_h, dv2, a.hds_l * dv2)));
      d[j] = d2f(a.p[row + S * j]) - kick;
      kahan(d[j]);
    }
    __syncthreads();  // the shared tables are written
    p0 = sc * (f2d(ch) - f2d(cc));
    gb_r2hc_s<NB, float, true>([&](int j) { return d[j]; }, [&](int k, float val) { pf[k] = val; }, s_tw, s_twf,
                               s_tw_l, s_twf_l);
    const double r0 = a.r[row];
    float h0, l0;
    d2df(r0, h0, l0);
    ch = 0.f;
    cc = 0.f;
    d[0] = 0.f;
#pragma unroll
    for (int j = 1; j < NB; ++j) {
      float h, l;
      d2df(a.r[row + S * j], h, l);
      d[j] = (h - h0) + (l - l0);
      kahan(d[j]);
    }
    x0 = sc * ((double)NB * r0 + (f2d(ch) - f2d(cc)));
    gb_r2hc_s<NB, float, true>([&](int j) { return d[j]; }, [&](int k, float val) { xf[k] = val; }, s_tw, s_twf,
                               s_tw_l, s_twf_l);
  }

  float e_lh = 0.f, e_ll = 0.f, q1h = 0.f, q1l = 0.f, q2h = 0.f, q2l = 0.f;  // df sums
  float vir[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float off = 0.f;  // this row's centroid minus its oxygen's centroid
  for (int im = 1; im <= a.mts; ++im) {
    {  // free ring-polymer rotation (evolve_pi.f90:109-125)
      const double *mo = s_mono + ic;
      const double pp = p0 * mo[0] + x0 * mo[3];
      x0 = p0 * mo[6] + x0 * mo[9];
      p0 = pp;
#pragma unroll
      for (int k = 1; k < NB; ++k) {
        const float *h = s_mh + ic + 12 * k, *l = s_ml + ic + 12 * k;
        const float pk = pf[k], xk = xf[k];
        pf[k] = fmaf(pk, h[0], fmaf(xk, h[3], fmaf(pk, l[0], xk * l[3])));
        xf[k] = fmaf(pk, h[6], fmaf(xk, h[9], fmaf(pk, l[6], xk * l[9])));
      }
    }
    const double cen = sc * x0;
    s_cen[t] = cen;
    __syncthreads();
    {
      float oh, ol;
      d2df(cen - s_cen[orow], oh, ol);
      off = oh + ol;
    }
    {  // bead positions relative to the oxygen centroid (evolve_pi.f90:141-145)
      float *dst = s_dev + t * C::LD;
      // split tables in every substep (one copy of the transform's code: the
      // kernel is large enough to stall on the instruction cache); the last
      // substep's positions are the new state, r = centroid + deviation
      // without the offset's rounding
      const bool last = im == a.mts && valid;
      double *gr = a.r + row;
      gb_hc2r_s<NB, float, true>([&](int j) { return j ? xf[j] : 0.f; },
                                 [&](int k, float v) {
                                   dst[k] = off + v;
                                   if (last) gr[S * k] = cen + f2d(v);
                                 },
                                 s_tw, s_twi, s_tw_l, s_twi_l);
    }
    __syncthreads();
    float esh = 0.f, esl = 0.f;
    for (int idx = t; idx < mpb * NB; idx += T) {
      const int mm = idx / NB, j = idx % NB;
      const bool w = m0 + mm < a.nm;
      float xr[9], fm[9], vm[9];
#pragma unroll
      for (int d = 0; d < 9; ++d) xr[d] = s_dev[(mm * 9 + d) * C::LD + j];
      const float e = intra_molecule_t<float>(a.model, xr, fm, vm, a.ip);
#pragma unroll
      for (int d = 0; d < 9; ++d) s_f2[(mm * 9 + d) * C::LD + j] = fm[d];
      if (w) {
        df_acc(esh, esl, e);
#pragma unroll
        for (int d = 0; d < 9; ++d) vir[d] += vm[d];
      }
    }
    if (im == a.mts) e_lh = esh, e_ll = esl;
    __syncthreads();
    {
      const float *dev_row = s_dev + t * C::LD;
      const float *f2_row = s_f2 + t * C::LD;
      if (valid) {  // virial_ke partial sums (kinetic.f90:23-40) about the bead centroid
        float a1 = 0.f, a2 = 0.f;
#pragma unroll
        for (int j = 0; j < NB; ++j) {
          const float dr = dev_row[j] - off;
          a1 += dr * dv_row[j];
          a2 += dr * f2_row[j];
        }
        df_acc(q1h, q1l, a1);
        df_acc(q2h, q2l, a2);
      }
      if (im != a.mts) {  // FT(dvdr2) and p -= dtsmall dvdr2 (evolve_pi.f90:156-159)
        const float dtsf = (float)a.dtsmall;
        float f0 = 0.f;
        gb_r2hc_s<NB, float>([&](int j) { return f2_row[j]; },
                             [&](int k, float v) {
                               if (k) pf[k] = fmaf(-dtsf, v, pf[k]);
                               else f0 = v;
                             },
                             s_tw, s_twf);
        p0 = p0 - a.dtsmall * f2d(f0);
      }
    }
    if (im != a.mts) __syncthreads();
  }
  {
    // back to beads: p = HC2R(p); r = rst (written in the last substep);
    // p -= halfdtsmall dvdr2 (evolve_pi.f90:222-228)
    const float *f2_row = s_f2 + t * C::LD;
    const float hds = (float)a.halfdtsmall;
    const double pc = sc * p0;
    double *gp = a.p + row;
    bool bad = gb_nonfinite(pc);
    gb_hc2r_s<NB, float, true>([&](int j) { return j ? pf[j] : 0.f; },
                               [&](int k, float v) {
                                 const float dp = fmaf(-hds, f2_row[k], v);
                                 bad |= gb_nonfinite(dp);
                                 if (valid) gp[S * k] = pc + f2d(dp);
                               },
                               s_tw, s_twi, s_tw_l, s_twi_l);
    if (valid) {
#pragma unroll
      for (int j = 0; j < NB; ++j) {
        a.rnm[row + S * j] = j ? f2d(xf[j]) : x0;
        a.dvdr2[row + S * j] = f2d(f2_row[j]);
        bad |= gb_nonfinite(f2_row[j]);
      }
      gb_flag_nonfinite(a.status, bad);
      // contracted rings of the new positions (gb_hc2r_direct over modes 0..h,
      // the FP32 modes summed in FP32): rb_j = s12 x0 + s12 y_j
      auto contract = [&](double *rb, int nbc, const float *ct, double s12) {
        if (!rb) return;
        const int h = (nbc - 1) / 2;
        const double base = s12 * x0;
        const float sf = d2f(s12);
        for (int j = 0; j < nbc; ++j) {
          float y = 0.f;
          int mm = 0;
#pragma unroll
          for (int k = 1; k <= (MTS_NBC - 1) / 2; ++k) {
            if (k <= h && k < NB) {
              mm += j;
              if (mm >= nbc) mm -= nbc;
              y += 2.f * (xf[k] * ct[mm] - xf[NB - k] * ct[nbc + mm]);
            }
          }
          rb[row + S * j] = base + f2d(sf * y);
        }
      };
      contract(a.rb1, a.nbc1, s_ct, a.s12_1);
      contract(a.rb2, a.nbc2, s_ct + 2 * MTS_NBC, a.s12_2);
    }
  }
  // block totals: df / FP32 warp sums, FP64 across warps (threads 0..17)
  float rh[9], rl[9];  // energy, q1, q2, q1 by axis, q2 by axis
  rh[0] = e_lh, rl[0] = e_ll;
  rh[1] = q1h, rl[1] = q1l;
  rh[2] = q2h, rl[2] = q2l;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    rh[3 + d] = d == xyz ? q1h : 0.f, rl[3 + d] = d == xyz ? q1l : 0.f;
    rh[6 + d] = d == xyz ? q2h : 0.f, rl[6 + d] = d == xyz ? q2l : 0.f;
  }
  const int lane = t & 31, warp = t >> 5, nw = (T + 31) / 32;
  float *s_rf = reinterpret_cast<float *>(s_red);  // [32 warps][36] floats in the [32][18] doubles
#pragma unroll
  for (int i = 0; i < 9; ++i) warp_sum_df(rh[i], rl[i]);
#pragma unroll
  for (int d = 0; d < 9; ++d) vir[d] = warp_sum_f32(vir[d]);
  if (lane == 0) {
    float *o = s_rf + warp * 36;
    // slots 2i, 2i+1: df values in the order of the 18 totals below
    o[0] = rh[0], o[1] = rl[0];
#pragma unroll
    for (int d = 0; d < 9; ++d) o[2 + 2 * d] = vir[d], o[3 + 2 * d] = 0.f;
    o[20] = rh[1], o[21] = rl[1];
    o[22] = rh[2], o[23] = rl[2];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      o[24 + 2 * d] = rh[3 + d], o[25 + 2 * d] = rl[3 + d];
      o[30 + 2 * d] = rh[6 + d], o[31 + 2 * d] = rl[6 + d];
    }
  }
  __syncthreads();
  if (t < 18) {  // 0 energy, 1..9 virial, 10, 11 q1, q2, 12..14 q1 by axis, 15..17 q2 by axis
    double s2 = 0.0;
    for (int w = 0; w < nw; ++w) s2 += df2d(s_rf[w * 36 + 2 * t], s_rf[w * 36 + 2 * t + 1]);
    if (s2 != 0.0) {
      if (t < 10) atomicAdd(a.acc_int + t, s2);
      else if (t < 12) atomicAdd(a.acc_ke + (t - 10), s2);
      else atomicAdd(a.acc_ke + 2 + (t - 12), s2);
    }
  }
}

// Mixed precision with two lanes per coordinate row (nb >= 8).  The same
// step as k_mts_mixed, but a row's beads and normal modes are split over a
// lane pair (gb_r2hc_pair / gb_hc2r_pair: lane q holds the beads 2i + q and
// the half-complex elements qM + i, M = nb / 2), so that the grid has twice
// the warps (one thread per row left the SMs latency-bound at ~8 warps each)
// and each lane runs M-point transforms (half the code).  The centroid mode
// (FP64) is kept by both lanes of a pair with the same operations, so the two
// copies stay equal; lane 0's element 0 (the FP32 centroid slot) stays zero.
template <int NB>
struct MtsPairCfg {
  static constexpr int M = NB / 2;
  static constexpr int MPB_MAX = NB <= 32 ? 28 : 14;
  static constexpr int T_MAX = (18 * MPB_MAX + 31) / 32 * 32;
  static constexpr int LD = NB + 2;  // bead stride in shared memory: lanes (row r, q) hit banks 2r + q
};

template <int NB>
__global__ void __launch_bounds__(MtsPairCfg<NB>::T_MAX, 1) k_mts_mixed_pair(MtsArgs a) {
  using C = MtsPairCfg<NB>;
  constexpr int M = C::M;
  extern __shared__ double sm[];
  const int T = blockDim.x;
  const int nrow = (T / 2 + 8) / 9 * 9;
  const int nf = (3 * nrow * C::LD + 1) & ~1;
  float *s_dev = reinterpret_cast<float *>(sm);    // [nrow][LD] x_j - (oxygen centroid)
  float *s_f2 = s_dev + nrow * C::LD;              // [nrow][LD] intramolecular forces
  float *s_dvf = s_f2 + nrow * C::LD;              // [nrow][LD] dvdr for the estimator
  double *s_cen = sm + nf / 2;                     // [nrow] row centroids
  double *s_mono = s_cen + nrow;                   // [12] monodromy of the centroid mode
  double *s_red = s_mono + 12;                     // [32 warps][18]
  float *s_mh = reinterpret_cast<float *>(s_red + 32 * 18);  // [12*NB] coefficients, hi
  float *s_ml = s_mh + 12 * NB;                    // [12*NB] lo
  float *s_twm = s_ml + 12 * NB;                   // [2M] cos, sin of 2 pi m / M
  float *s_twm_l = s_twm + 2 * M;
  float *s_twfm = s_twm_l + 2 * M;                 // [2M] half of s_twm
  float *s_twfm_l = s_twfm + 2 * M;
  float *s_twi = s_twfm_l + 2 * M;                 // [2NB] sc cos, sc sin of 2 pi m / nb
  float *s_twi_l = s_twi + 2 * NB;
  float *s_ct = s_twi_l + 2 * NB;                  // [2][2*MTS_NBC] contraction cos, sin
  const int t = threadIdx.x;
  const double sc = a.sc;
  for (int i = t; i < 12 * NB; i += T) {
    const double w = a.monod[i];
    d2df(w, s_mh[i], s_ml[i]);
    if (i < 12) s_mono[i] = w;
  }
  for (int i = t; i < 2 * M; i += T) {  // length-M tables: every other entry of length nb
    const int mm = i < M ? 2 * i : NB + 2 * (i - M);
    float h, l;
    d2df(a.tw[mm], h, l);
    s_twm[i] = h, s_twm_l[i] = l;
    s_twfm[i] = 0.5f * h, s_twfm_l[i] = 0.5f * l;
  }
  for (int i = t; i < 2 * NB; i += T) d2df(sc * a.tw[i], s_twi[i], s_twi_l[i]);
  for (int i = t; i < 4 * MTS_NBC; i += T) {
    const int qq = i / (2 * MTS_NBC), e = i % (2 * MTS_NBC);
    const double *tw = qq ? a.tw_c2 : a.tw_c1;
    const int nbc = qq ? a.nbc2 : a.nbc1;
    const double *rb = qq ? a.rb2 : a.rb1;
    s_ct[i] = rb && e < 2 * nbc ? d2f(tw[e]) : 0.f;
  }
  const int q = t & 1;   // beads 2i + q, half-complex elements qM + i
  const int rl = t >> 1; // row of the block
  const int mpb = a.mpb;
  const int m0 = blockIdx.x * mpb;
  const int ml = rl / 9, lr = rl % 9;
  const int m = m0 + ml;
  const bool valid = ml < mpb && m < a.nm;
  const int mc = valid ? m : a.nm - 1;
  const long long S = 3LL * a.na;
  const long long row = 9LL * mc + lr;
  const int ic = lr / 3;
  const int xyz = lr % 3;
  const int orow = ml * 9 + xyz;
  float *dv_row = s_dvf + rl * C::LD;
  auto bead = [&](int i) { return 2 * i + q; };

  // opening kicks and forward transforms without per-element FP64 (as in
  // k_mts_mixed); each lane's compensated bead sums are combined over the pair
  double p0, x0;
  float pf[M], xf[M];
  {
    float d[M];
    float ch = 0.f, cc = 0.f;
    auto kahan = [&](float v) {
      const float y = v - cc;
      const float t2 = ch + y;
      cc = (t2 - ch) - y;
      ch = t2;
    };
    auto pair_sum = [&]() {  // the same FP64 value on both lanes (addition commutes)
      const float oh = __shfl_xor_sync(0xffffffffu, ch, 1), oc = __shfl_xor_sync(0xffffffffu, cc, 1);
      return (f2d(ch) - f2d(cc)) + (f2d(oh) - f2d(oc));
    };
#pragma unroll
    for (int i = 0; i < M; ++i) {
      const long long o = row + S * bead(i);
      const float dv = d2f(a.dvdr[o]), dv2 = d2f(a.dvdr2[o]);
      dv_row[bead(i)] = dv;
      const float kick = fmaf(a.hdt_h, dv, fmaf(a.hdt_l, dv, fmaf(a.hds_h, dv2, a.hds_l * dv2)));
      d[i] = d2f(a.p[o]) - kick;
      kahan(d[i]);
    }
    __syncthreads();  // the shared tables are written
    p0 = sc * pair_sum();
    gb_r2hc_pair<NB, true>(q, [&](int i) { return d[i]; }, [&](int i, float v) { pf[i] = v; }, s_twm, s_twfm,
                           s_twi, s_twm_l, s_twfm_l, s_twi_l);
    const double r0 = a.r[row];
    float h0, l0;
    d2df(r0, h0, l0);
    ch = 0.f;
    cc = 0.f;
#pragma unroll
    for (int i = 0; i < M; ++i) {
      float h, l;
      d2df(a.r[row + S * bead(i)], h, l);
      d[i] = (h - h0) + (l - l0);
      kahan(d[i]);
    }
    x0 = sc * ((double)NB * r0 + pair_sum());
    gb_r2hc_pair<NB, true>(q, [&](int i) { return d[i]; }, [&](int i, float v) { xf[i] = v; }, s_twm, s_twfm,
                           s_twi, s_twm_l, s_twfm_l, s_twi_l);
    if (q == 0) pf[0] = xf[0] = 0.f;  // the centroid is p0, x0
  }

  float e_lh = 0.f, e_ll = 0.f, q1h = 0.f, q1l = 0.f, q2h = 0.f, q2l = 0.f;  // df sums
  float vir[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  float off = 0.f;
  for (int im = 1; im <= a.mts; ++im) {
    {  // free ring-polymer rotation (evolve_pi.f90:109-125)
      const double *mo = s_mono + ic;
      const double pp = p0 * mo[0] + x0 * mo[3];
      x0 = p0 * mo[6] + x0 * mo[9];
      p0 = pp;
#pragma unroll
      for (int i = 0; i < M; ++i) {
        const int h = q * M + i;
        const float *hh = s_mh + ic + 12 * h, *ll = s_ml + ic + 12 * h;
        const float pk = pf[i], xk = xf[i];
        pf[i] = fmaf(pk, hh[0], fmaf(xk, hh[3], fmaf(pk, ll[0], xk * ll[3])));
        xf[i] = fmaf(pk, hh[6], fmaf(xk, hh[9], fmaf(pk, ll[6], xk * ll[9])));
      }
    }
    const double cen = sc * x0;
    if (q == 0) s_cen[rl] = cen;
    __syncthreads();
    {
      float oh, ol;
      d2df(cen - s_cen[orow], oh, ol);
      off = oh + ol;
    }
    {  // bead positions relative to the oxygen centroid (evolve_pi.f90:141-145)
      float *dst = s_dev + rl * C::LD;
      const bool last = im == a.mts && valid;
      double *gr = a.r + row;
      gb_hc2r_pair<NB, true>(q, [&](int i) { return xf[i]; },
                             [&](int i, float v) {
                               dst[bead(i)] = off + v;
                               if (last) gr[S * bead(i)] = cen + f2d(v);
                             },
                             s_twm, s_twi, s_twm_l, s_twi_l);
    }
    __syncthreads();
    float esh = 0.f, esl = 0.f;
    for (int idx = t; idx < mpb * NB; idx += T) {
      const int mm = idx / NB, j = idx % NB;
      const bool w = m0 + mm < a.nm;
      float xr[9], fm[9], vm[9];
#pragma unroll
      for (int d = 0; d < 9; ++d) xr[d] = s_dev[(mm * 9 + d) * C::LD + j];
      const float e = intra_molecule_t<float>(a.model, xr, fm, vm, a.ip);
#pragma unroll
      for (int d = 0; d < 9; ++d) s_f2[(mm * 9 + d) * C::LD + j] = fm[d];
      if (w) {
        df_acc(esh, esl, e);
#pragma unroll
        for (int d = 0; d < 9; ++d) vir[d] += vm[d];
      }
    }
    if (im == a.mts) e_lh = esh, e_ll = esl;
    __syncthreads();
    {
      const float *dev_row = s_dev + rl * C::LD;
      const float *f2_row = s_f2 + rl * C::LD;
      if (valid) {  // virial_ke partial sums (kinetic.f90:23-40) over this lane's beads
        float a1 = 0.f, a2 = 0.f;
#pragma unroll
        for (int i = 0; i < M; ++i) {
          const float dr = dev_row[bead(i)] - off;
          a1 += dr * dv_row[bead(i)];
          a2 += dr * f2_row[bead(i)];
        }
        df_acc(q1h, q1l, a1);
        df_acc(q2h, q2l, a2);
      }
      if (im != a.mts) {  // FT(dvdr2) and p -= dtsmall dvdr2 (evolve_pi.f90:156-159)
        const float dtsf = (float)a.dtsmall;
        float f0 = 0.f;
        gb_r2hc_pair<NB, false>(q, [&](int i) { return f2_row[bead(i)]; },
                                [&](int i, float v) {
                                  if (q == 0 && i == 0) f0 = v;
                                  else pf[i] = fmaf(-dtsf, v, pf[i]);
                                },
                                s_twm, s_twfm, s_twi);
        f0 = __shfl_sync(0xffffffffu, f0, (t & 31) & ~1);  // lane 0's centroid force
        p0 = p0 - a.dtsmall * f2d(f0);
      }
    }
    if (im != a.mts) __syncthreads();
  }
  {
    // back to beads: p = HC2R(p); r = rst (written in the last substep);
    // p -= halfdtsmall dvdr2 (evolve_pi.f90:222-228)
    const float *f2_row = s_f2 + rl * C::LD;
    const float hds = (float)a.halfdtsmall;
    const double pc = sc * p0;
    double *gp = a.p + row;
    bool bad = gb_nonfinite(pc);
    gb_hc2r_pair<NB, true>(q, [&](int i) { return pf[i]; },
                           [&](int i, float v) {
                             const float dp = fmaf(-hds, f2_row[bead(i)], v);
                             bad |= gb_nonfinite(dp);
                             if (valid) gp[S * bead(i)] = pc + f2d(dp);
                           },
                           s_twm, s_twi, s_twm_l, s_twi_l);
    if (valid) {
#pragma unroll
      for (int i = 0; i < M; ++i) {
        const int h = q * M + i;
        a.rnm[row + S * h] = h ? f2d(xf[i]) : x0;
        a.dvdr2[row + S * bead(i)] = f2d(f2_row[bead(i)]);
        bad |= gb_nonfinite(f2_row[bead(i)]);
      }
      gb_flag_nonfinite(a.status, bad);
    }
    // contracted rings of the new positions: rb_j = s12 x0 + s12 y_j, y_j =
    // sum_k 2 (Re X_k cos - Im X_k sin); lane 0 sums the real parts, lane 1 the
    // imaginary ones, and the lane of the bead's parity stores
    auto contract = [&](double *rb, int nbc, const float *ct, double s12) {
      const int h = (nbc - 1) / 2;
      const double base = s12 * x0;
      const float sf = d2f(s12);
      for (int j = 0; j < nbc; ++j) {
        float y = 0.f;
        int mm = 0;
#pragma unroll
        for (int k = 1; k <= (MTS_NBC - 1) / 2; ++k) {
          if (k <= h && k < M) {
            mm += j;
            if (mm >= nbc) mm -= nbc;
            y += q ? -2.f * xf[M - k] * ct[nbc + mm] : 2.f * xf[k] * ct[mm];
          }
        }
        y += __shfl_xor_sync(0xffffffffu, y, 1);
        if (valid && (j & 1) == q) rb[row + S * j] = base + f2d(sf * y);
      }
    };
    if (a.rb1) contract(a.rb1, a.nbc1, s_ct, a.s12_1);
    if (a.rb2) contract(a.rb2, a.nbc2, s_ct + 2 * MTS_NBC, a.s12_2);
  }
  // block totals: df / FP32 warp sums, FP64 across warps (threads 0..17)
  float rh[9], rl9[9];  // energy, q1, q2, q1 by axis, q2 by axis
  rh[0] = e_lh, rl9[0] = e_ll;
  rh[1] = q1h, rl9[1] = q1l;
  rh[2] = q2h, rl9[2] = q2l;
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    rh[3 + d] = d == xyz ? q1h : 0.f, rl9[3 + d] = d == xyz ? q1l : 0.f;
    rh[6 + d] = d == xyz ? q2h : 0.f, rl9[6 + d] = d == xyz ? q2l : 0.f;
  }
  const int lane = t & 31, warp = t >> 5, nw = (T + 31) / 32;
  float *s_rf = reinterpret_cast<float *>(s_red);
#pragma unroll
  for (int i = 0; i < 9; ++i) warp_sum_df(rh[i], rl9[i]);
#pragma unroll
  for (int d = 0; d < 9; ++d) vir[d] = warp_sum_f32(vir[d]);
  if (lane == 0) {
    float *o = s_rf + warp * 36;
    o[0] = rh[0], o[1] = rl9[0];
#pragma unroll
    for (int d = 0; d < 9; ++d) o[2 + 2 * d] = vir[d], o[3 + 2 * d] = 0.f;
    o[20] = rh[1], o[21] = rl9[1];
    o[22] = rh[2], o[23] = rl9[2];
#pragma unroll
    for (int d = 0; d < 3; ++d) {
      o[24 + 2 * d] = rh[3 + d], o[25 + 2 * d] = rl9[3 + d];
      o[30 + 2 * d] = rh[6 + d], o[31 + 2 * d] = rl9[6 + d];
    }
  }
  __syncthreads();
  if (t < 18) {
    double s2 = 0.0;
    for (int w = 0; w < nw; ++w) s2 += df2d(s_rf[w * 36 + 2 * t], s_rf[w * 36 + 2 * t + 1]);
    if (s2 != 0.0) {
      if (t < 10) atomicAdd(a.acc_int + t, s2);
      else if (t < 12) atomicAdd(a.acc_ke + (t - 10), s2);
      else atomicAdd(a.acc_ke + 2 + (t - 12), s2);
    }
  }
}

template <int NB>
size_t mts_smem_pair(int T) {
  using C = MtsPairCfg<NB>;
  const int nrow = (T / 2 + 8) / 9 * 9;
  const int nf = (3 * nrow * C::LD + 1) & ~1;
  return sizeof(float) * nf + sizeof(double) * (nrow + 12 + 32 * 18) +
         sizeof(float) * (24 * NB + 8 * C::M + 4 * NB + 4 * MTS_NBC);
}

template <int NB>
size_t mts_smem_mixed(int T) {
  using C = MtsCfg<NB>;
  const int nrow = (T + 8) / 9 * 9;
  const int nf = (3 * nrow * C::LD + 1) & ~1;
  return sizeof(float) * nf + sizeof(double) * (nrow + 12 + 32 * 18) +
         sizeof(float) * (24 * NB + 12 * NB + 4 * MTS_NBC);
}

template <int NB>
size_t mts_smem(int T) {
  using C = MtsCfg<NB>;
  const int nrow = (T + 8) / 9 * 9;
  return sizeof(double) * (2 * nrow * C::LD + 12 * NB + 6 * NB + 32 * 18);
}

template <int NB>
void launch_nb(cudaStream_t s, MtsArgs a, bool mixed) {
  using C = MtsCfg<NB>;
  static bool attr = false;
  if (!attr) {  // the largest request of any launch
    cudaFuncSetAttribute(k_mts_fused<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mts_smem<NB>(C::T_MAX));
    cudaFuncSetAttribute(k_mts_mixed<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)mts_smem_mixed<NB>(C::T_MAX));
    if constexpr (NB >= 8)
      cudaFuncSetAttribute(k_mts_mixed_pair<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)mts_smem_pair<NB>(MtsPairCfg<NB>::T_MAX));
    attr = true;
  }
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  // one wave of blocks over the SMs when the molecules fit (two blocks per SM
  // for the mixed kernel), else MPB_MAX per block; a tuned count
  // (gbrpmd_ctx_autotune) overrides it
  const int wave = std::max(nsm, 1) * (mixed ? 2 : 1);
  a.mpb = a.mpb > 0 ? std::min(C::MPB_MAX, a.mpb) : std::max(1, std::min(C::MPB_MAX, (a.nm + wave - 1) / wave));
  const unsigned grid = (unsigned)((a.nm + a.mpb - 1) / a.mpb);
  if constexpr (NB >= 8) {
    if (mixed) {  // two lanes per coordinate row
      const int T2 = (18 * a.mpb + 31) / 32 * 32;
      k_mts_mixed_pair<NB><<<grid, T2, mts_smem_pair<NB>(T2), s>>>(a);
      return;
    }
  }
  const int T = (9 * a.mpb + 31) / 32 * 32;
  if (mixed) k_mts_mixed<NB><<<grid, T, mts_smem_mixed<NB>(T), s>>>(a);
  else k_mts_fused<NB><<<grid, T, mts_smem<NB>(T), s>>>(a);
}

int intra_model_of(const gb_params &P) {
  if (P.intra_model == GB_INTRA_SPCFW) return 1;
  return P.alp == 0.0 ? 0 : 2;
}

}  // namespace

// Runs the fused block when nb is a power of two up to 64; *used = 0 otherwise.
void launch_fused_mts(cudaStream_t s, gb_context *c, double dt, int *used) {
  *used = 0;
  const int nb = c->nb;
  if (nb != 2 && nb != 4 && nb != 8 && nb != 16 && nb != 32 && nb != 64) return;
  MtsArgs a;
  a.mpb = c->tune.mts_mpb;  // 0: chosen in launch_nb
  a.p = c->p;
  a.r = c->r;
  a.rnm = c->rnm;
  a.dvdr2 = c->dvdr2;
  a.dvdr = c->dvdr;
  a.monod = c->monod;
  a.tw = c->tw_nb;
  a.acc_int = c->acc + (size_t)ACC_INT * ACC_STRIDE;
  a.acc_ke = c->acc + (size_t)ACC_KE * ACC_STRIDE;
  a.status = c->status;
  a.na = c->na;
  a.nm = c->nm;
  a.mts = c->P.mts;
  a.model = intra_model_of(c->P);
  a.halfdt = 0.5 * dt;
  a.dtsmall = dt / (double)c->P.mts;
  a.halfdtsmall = 0.5 * a.dtsmall;
  auto split = [](double v, float &h, float &l) {
    h = (float)v;
    l = (float)(v - (double)h);
  };
  split(a.halfdt, a.hdt_h, a.hdt_l);
  split(a.halfdtsmall, a.hds_h, a.hds_l);
  a.sc = std::sqrt(1.0 / (double)nb);
  // the mixed kernel writes the contracted rings when the forces follow the
  // propagation directly (no barostat shift in between)
  a.rb1 = a.rb2 = nullptr;
  a.nbc1 = a.nbc2 = 0;
  a.tw_c1 = c->tw_c1;
  a.tw_c2 = c->tw_c2;
  a.s12_1 = a.s12_2 = 0.0;
  c->rb1_ready = c->rb2_ready = false;
  const bool mixed_k = c->P.precision == GB_PREC_MIXED;
  auto fuse = [&](int nbc) { return mixed_k && !c->nbaro && nb > 1 && nbc > 0 && nbc <= MTS_NBC && nbc <= nb && (nbc & 1); };
  if (fuse(c->P.nbdf1)) {
    a.rb1 = c->rb1;
    a.nbc1 = c->P.nbdf1;
    a.s12_1 = std::sqrt((double)a.nbc1 / (double)nb) * std::sqrt(1.0 / (double)a.nbc1);
    c->rb1_ready = true;
  }
  if (fuse(c->P.nbdf2)) {
    a.rb2 = c->rb2;
    a.nbc2 = c->P.nbdf2;
    a.s12_2 = std::sqrt((double)a.nbc2 / (double)nb) * std::sqrt(1.0 / (double)a.nbc2);
    c->rb2_ready = true;
  }
  a.ip.reoh = c->P.reoh;
  a.ip.theta = c->P.theta;
  a.ip.rehh = 2.0 * sin(0.5 * c->P.theta) * c->P.reoh;
  a.ip.apot = c->P.apot;
  a.ip.bpot = c->P.bpot;
  a.ip.alp = c->P.alp;
  const bool mixed = c->P.precision == GB_PREC_MIXED;
  switch (nb) {
    case 2: launch_nb<2>(s, a, mixed); break;
    case 4: launch_nb<4>(s, a, mixed); break;
    case 8: launch_nb<8>(s, a, mixed); break;
    case 16: launch_nb<16>(s, a, mixed); break;
    case 32: launch_nb<32>(s, a, mixed); break;
    case 64: launch_nb<64>(s, a, mixed); break;
  }
  *used = 1;
}
