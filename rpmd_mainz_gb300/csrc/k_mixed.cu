// k_mixed.cu -- FP32 force kernels of the mixed-precision path.
//
// Same pair sets and formulas as the FP64 kernels (k_pairs.cu, k_recip.cu),
// with the per-pair and per-(k, site) arithmetic in FP32:
//  * LJ positions enter as two FP32 numbers per wrapped fractional coordinate
//    (hi + lo, k_frac32), so a minimum-image displacement
//    (hi_i - hi_j - rint(hi_i - hi_j)) + (lo_i - lo_j) keeps ~1e-14 of the box;
//    real-space Ewald positions as 32-bit fixed-point fractions (frac_point);
//  * pair kernels walk full lists (each pair from both ends), so every point's
//    force is summed by its own lanes and no atomics are needed; the
//    real-space kernel walks the skin list itself and drops pairs beyond the
//    cut-off with its FP32 distance (no per-step exact filter), two entries at
//    a time in paired FP32 arithmetic (FFMA2 / FADD2 / FMUL2);
//  * force and energy sums are compensated (Kahan) FP32 per thread, virials
//    plain FP32 per thread; energies df (two-float) and virials FP32 within a
//    warp, FP64 across warps (block_sum_df: no per-thread FP64 instruction);
//  * the reciprocal-space power tables are FP32 sines and cosines of phases
//    reduced in two-float arithmetic; structure-factor partials are FP32 over
//    a chunk of sites and df over chunks; energy, virial and the k-space
//    totals stay FP64.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <type_traits>

#include "gb_common.cuh"
#include "gb_df.cuh"
#include "gb_f2.cuh"
#include "gb_kernels.h"

namespace {

constexpr int MX_T = 64;     // threads per block of the pair kernels
// resident blocks per SM asked of the real-space kernel: a register bound of
// 80 per thread (fewer spill)
constexpr int MX_MINB = 12;
// lanes per site (real-space Ewald: 8, 16 or 32, default 16) and per oxygen
// (LJ: 2, 4 or 8, default 4) are template parameters; the launchers take them
// from the context's tuning (gbrpmd_ctx_autotune)

GB_D void kadd(float &s, float &c, float v) {  // Kahan-compensated s += v
  const float y = v - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

template <int NP>
GB_D float group_sum_f(float v) {
#pragma unroll
  for (int o = NP / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// minimum-image difference of two hi/lo fractional coordinates
GB_D float dmin(float hi_a, float lo_a, float hi_b, float lo_b) {
  const float d = hi_a - hi_b;
  return (d - rintf(d)) + (lo_a - lo_b);
}

// rwald (ewald_cubic.f90:78-233) in FP32 over a full list; g += gradient
// (single writer per site), energy and virial halved for the double count.
// Positions are 32-bit fixed-point fractional coordinates (frac_point): the
// wrapping difference of two, read as a signed integer, is the minimum-image
// difference in units of 2^-32, and its conversion rounds it to FP32 relative
// to its own size (the precision of a hi + lo pair of floats, with one 16-byte
// gather per partner and no rint per component); the charge's bits ride in w.
// IT: the list entry type (unsigned short for up to 65535 sites halves the
// list's bytes).  SLOTS: the entries are cell-order slots of the last list
// rebuild (bit 15: same molecule) and the partners' positions come from fxs,
// the same coordinates in slot order, so that consecutive entries of a list,
// mostly runs of the same cells, gather from neighbouring addresses.
// Each lane takes every NP-th quad of consecutive entries and evaluates two
// entries at a time in paired FP32 arithmetic (gb_f2.cuh: one instruction, two
// correctly rounded operations); entries beyond the cut-off (and the missing
// partners of the list's tail) get a zero charge product instead of a branch.
// exp(-x^2) is the fast exponential (__expf): its error, a few ulp, is below
// that of the erfc polynomial it multiplies.  A quad's terms are summed plainly
// and added to the lane's compensated (Kahan) force and energy sums.
// npair (profiling only): in-cut entries counted.  bx: side lengths that turn
// fractional differences into distances, times 2^-32 (1 * 2^-32 in the unit
// box of the cubic sum; the box in bohr for the non-cubic one, rwald_basic /
// rwald_cell of ewald_noncubic.f90)
template <int NP, typename IT, bool SLOTS>
__global__ void __launch_bounds__(MX_T, MX_MINB) k_ewald_real_mx(const int4 *__restrict__ fx,
                                                              const int4 *__restrict__ fxs, int na,
                                                              const int *__restrict__ count,
                                                              const IT *__restrict__ idx, int cap, float alpha,
                                                              float sfac, float rcutsq, float3 bx, double *g,
                                                              double *acc, int add, unsigned long long *npair,
                                                              int lconf) {
  __shared__ float sh[32 * 8];
  const float p = 3.0525860f, a1 = 0.254829592f, a2 = -0.284496736f, a3 = 1.421413741f,
              a4 = -1.453152027f, a5 = 1.061405429f;
  const int c = blockIdx.y;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int i = (int)(tid / NP), sub = (int)(tid % NP);
  const bool active = i < na;
  const int4 *X = fx + (long long)c * na;
  const int4 *XJ = SLOTS ? fxs + (long long)c * na : X;
  int nin = 0;
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, ev = 0.f, evc = 0.f;
  const float2 z2 = f2s(0.f);
  float2 vxx = z2, vyx = z2, vzx = z2, vyy = z2, vzy = z2, vzz = z2;
  if (active) {
    const int4 xi = X[i];
    const float mqi = -__int_as_float(xi.w);  // the pair terms carry -q_i q_j
    const int m3 = (i / 3) * 3;  // first site of i's molecule
    // the list of i: its configuration's, or with lconf = 0 the one list the
    // configurations share (built on their centroids)
    const long long row = (long long)(lconf ? c : 0) * na + i;
    const int n = min(count[row], cap);
    const IT *L = idx + row * cap;
    auto same = [&](int e) { return SLOTS ? (e & 0x8000) != 0 : (unsigned)(e - m3) < 3u; };
    auto slot = [&](int e) { return SLOTS ? (e & 0x7fff) : e; };
    const float2 bxx = f2s(bx.x), bxy = f2s(bx.y), bxz = f2s(bx.z), al2 = f2s(alpha), p2 = f2s(p);
    const float2 msf = f2s(-sfac);
    // two entries ea, eb (va, vb false: no partner, the tail of the list);
    // returns the gradient terms and -q_i q_j du, adds the virial terms
    auto pair2 = [&](int ea, int eb, const int4 &xa, const int4 &xb, bool va, bool vb, float2 &fxv, float2 &fyv,
                     float2 &fzv, float2 &eu) {
      const float2 dx = mul2(f2((float)(int)((unsigned)xi.x - (unsigned)xa.x), (float)(int)((unsigned)xi.x - (unsigned)xb.x)), bxx);
      const float2 dy = mul2(f2((float)(int)((unsigned)xi.y - (unsigned)xa.y), (float)(int)((unsigned)xi.y - (unsigned)xb.y)), bxy);
      const float2 dz = mul2(f2((float)(int)((unsigned)xi.z - (unsigned)xa.z), (float)(int)((unsigned)xi.z - (unsigned)xb.z)), bxz);
      const float2 drsq = fma2(dz, dz, fma2(dy, dy, mul2(dx, dx)));
      const bool ina = va && drsq.x < rcutsq, inb = vb && drsq.y < rcutsq;
      if (npair) nin += (int)ina + (int)inb;
      // -q_i q_j, zero for an entry beyond the cut-off
      const float2 mq = f2(ina ? mqi * __int_as_float(xa.w) : 0.f, inb ? mqi * __int_as_float(xb.w) : 0.f);
      // an entry beyond the cut-off may be far: keep its arithmetic finite
      const float2 d2 = f2(ina ? drsq.x : 1.f, inb ? drsq.y : 1.f);
      const float2 inv = f2(rsqrtf(d2.x), rsqrtf(d2.y));
      const float2 x = mul2(al2, mul2(d2, inv));
      const float2 xx = mul2(x, x);
      const float2 e = f2(__expf(-xx.x), __expf(-xx.y));
      const float2 den = add2(p2, x);
      const float2 tt = f2(__fdividef(p, den.x), __fdividef(p, den.y));
      const float2 poly = fma2(tt, fma2(tt, fma2(tt, fma2(tt, f2s(a5), f2s(a4)), f2s(a3)), f2s(a2)), f2s(a1));
      float2 erfc = mul2(mul2(e, tt), poly);
      erfc = add2(erfc, f2(same(ea) ? -1.f : 0.f, same(eb) ? -1.f : 0.f));  // same molecule
      const float2 du = mul2(erfc, inv);
      const float2 w = fma2(msf, e, du);                    // du - sfac e = -dur r^2
      const float2 dvr = mul2(mq, mul2(w, mul2(inv, inv)));  // q_i q_j dur
      fxv = mul2(dvr, dx);
      fyv = mul2(dvr, dy);
      fzv = mul2(dvr, dz);
      eu = mul2(mq, du);
      vxx = fma2(dx, fxv, vxx);
      vyx = fma2(dy, fxv, vyx);
      vzx = fma2(dz, fxv, vzx);
      vyy = fma2(dy, fyv, vyy);
      vzy = fma2(dz, fyv, vzy);
      vzz = fma2(dz, fzv, vzz);
    };
    // lane sub takes the quads of consecutive entries sub, sub + NP, ...: one
    // 8-byte (16-byte for int entries) load per quad, loaded two quads ahead
    // of their arithmetic; entries past n (the list rows hold a multiple of
    // four) are read but not used
    using Q = typename std::conditional<sizeof(IT) == 2, uint2, uint4>::type;
    const Q *LQ = reinterpret_cast<const Q *>(L);
    auto ent = [&](const Q &w, int k) -> int {
      if constexpr (sizeof(IT) == 2) {
        const unsigned h = k < 2 ? w.x : w.y;
        return (k & 1) ? (int)(h >> 16) : (int)(h & 0xffffu);
      } else {
        return (int)(k == 0 ? w.x : k == 1 ? w.y : k == 2 ? w.z : w.w);
      }
    };
    const int nq = (n + 3) >> 2;
    int qd = sub;
    Q w0{}, w1{};
    if (qd < nq) w0 = LQ[qd];
    if (qd + NP < nq) w1 = LQ[qd + NP];
    for (; qd < nq; qd += NP) {
      const int b = 4 * qd;
      const bool v1 = b + 1 < n, v2 = b + 2 < n, v3 = b + 3 < n;
      const int e0 = ent(w0, 0), e1 = v1 ? ent(w0, 1) : e0, e2 = v2 ? ent(w0, 2) : e0, e3 = v3 ? ent(w0, 3) : e0;
      const int4 x0 = XJ[slot(e0)], x1 = XJ[slot(e1)], x2 = XJ[slot(e2)], x3 = XJ[slot(e3)];
      w0 = w1;
      if (qd + 2 * NP < nq) w1 = LQ[qd + 2 * NP];
      float2 fa, fb, fc, fd, ga, gb, gc, gd;
      pair2(e0, e1, x0, x1, true, v1, fa, fb, fc, fd);
      pair2(e2, e3, x2, x3, v2, v3, ga, gb, gc, gd);
      // the quad's four terms summed plainly, then one compensated add
      const float2 qx = add2(fa, ga), qy = add2(fb, gb), qz = add2(fc, gc), qe = add2(fd, gd);
      kadd(sx, cx, qx.x + qx.y);
      kadd(sy, cy, qy.x + qy.y);
      kadd(sz, cz, qz.x + qz.y);
      kadd(ev, evc, qe.x + qe.y);
    }
  }
  if (npair) {  // one atomic per warp
    const int tot = __reduce_add_sync(0xffffffffu, nin);
    if ((threadIdx.x & 31) == 0 && tot) atomicAdd(npair, (unsigned long long)tot);
  }
  // each lane's compensated sum, then FP32 across the site's lanes
  const float fx0 = group_sum_f<NP>(sx - cx);
  const float fy0 = group_sum_f<NP>(sy - cy);
  const float fz0 = group_sum_f<NP>(sz - cz);
  if (active && sub == 0) {
    double *G = g + ((long long)c * na + i) * 3;
    G[0] = (add ? G[0] : 0.0) + f2d(fx0);
    G[1] = (add ? G[1] : 0.0) + f2d(fy0);
    G[2] = (add ? G[2] : 0.0) + f2d(fz0);
  }
  const float vir6[6] = {vxx.x + vxx.y, vyx.x + vyx.y, vzx.x + vzx.y, vyy.x + vyy.y, vzy.x + vzy.y, vzz.x + vzz.y};
  constexpr int dst[7] = {0, 1, 2, 3, 5, 6, 9};       // v, xx, yx, zx, yy, zy, zz
  constexpr int dst2[7] = {-1, -1, 4, 7, -1, 8, -1};  // mirrored xy, xz, yz
  // energy: the sum holds -q_i q_j du; halved: each pair from both ends
  block_sum_df<7>(-ev, evc, vir6, sh, acc, dst, dst2, 0.5, 0.5);
}

// lj_list / lj_basic (ljones.f90) in FP32 over a full oxygen list; bead pairs
// beyond rcut are skipped as in the reference; out += dscale * gradient
template <int NP>
__global__ void __launch_bounds__(MX_T) k_lj_mx(const float4 *__restrict__ hi, const float4 *__restrict__ lo, int na,
                                                int npt, int nconf_list, const int *__restrict__ count,
                                                const int *__restrict__ idx, int cap, float sigsq, float rcutsq,
                                                float3 box, double dscale, double *out, double *acc) {
  __shared__ float sh[32 * 11];
  const int c = blockIdx.y;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int o = (int)(tid / NP), sub = (int)(tid % NP);
  const bool active = o < npt;
  const float4 *H = hi + (long long)c * npt, *Lo = lo + (long long)c * npt;
  float sx = 0.f, sy = 0.f, sz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  float vsum = 0.f, vcmp = 0.f, w[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (active) {
    const int lc = nconf_list == 1 ? 0 : c;
    const int n = min(count[(long long)lc * npt + o], cap);
    const int *L = idx + ((long long)lc * npt + o) * cap;
    const float4 hi_o = H[o], lo_o = Lo[o];
    auto pair = [&](const float4 &hj, const float4 &lj) {
      // j - o, as the reference orients it
      const float dx = dmin(hj.x, lj.x, hi_o.x, lo_o.x) * box.x;
      const float dy = dmin(hj.y, lj.y, hi_o.y, lo_o.y) * box.y;
      const float dz = dmin(hj.z, lj.z, hi_o.z, lo_o.z) * box.z;
      const float drsq = dx * dx + dy * dy + dz * dz;
      if (drsq < rcutsq) {
        const float onr2 = __fdividef(1.0f, drsq);
        const float sr2 = sigsq * onr2;
        const float sr6 = sr2 * sr2 * sr2;
        const float fij = sr6 * (sr6 - 0.5f) * onr2;
        const float fx = fij * dx, fy = fij * dy, fz = fij * dz;
        kadd(sx, cx, fx);
        kadd(sy, cy, fy);
        kadd(sz, cz, fz);
        kadd(vsum, vcmp, sr6 * (sr6 - 1.0f));
        w[0] -= dx * fx; w[1] -= dy * fx; w[2] -= dz * fx;
        w[3] -= dx * fy; w[4] -= dy * fy; w[5] -= dz * fy;
        w[6] -= dx * fz; w[7] -= dy * fz; w[8] -= dz * fz;
      }
    };
    int t = sub;
    for (; t + 3 * NP < n; t += 4 * NP) {
      const int j0 = L[t], j1 = L[t + NP], j2 = L[t + 2 * NP], j3 = L[t + 3 * NP];
      const float4 h0 = H[j0], h1 = H[j1], h2 = H[j2], h3 = H[j3];
      const float4 l0 = Lo[j0], l1 = Lo[j1], l2 = Lo[j2], l3 = Lo[j3];
      pair(h0, l0);
      pair(h1, l1);
      pair(h2, l2);
      pair(h3, l3);
    }
    for (; t < n; t += NP) {
      const int j = L[t];
      pair(H[j], Lo[j]);
    }
  }
  const float fx = group_sum_f<NP>(sx - cx);
  const float fy = group_sum_f<NP>(sy - cy);
  const float fz = group_sum_f<NP>(sz - cz);
  if (active && sub == 0) {
    double *F = out + (long long)c * na * 3 + 9LL * o;
    F[0] += dscale * f2d(fx);
    F[1] += dscale * f2d(fy);
    F[2] += dscale * f2d(fz);
  }
  constexpr int dst[10] = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9};
  constexpr int dst2[10] = {-1, -1, -1, -1, -1, -1, -1, -1, -1, -1};
  block_sum_df<10>(vsum, -vcmp, w, sh, acc, dst, dst2, 0.5, 0.5);  // halved: each pair from both ends
}

// ---- reciprocal space (kwald, ewald_cubic.f90:235-533), FP32 ----
constexpr int MSK_CHUNK = 64;  // sites per structure-factor block (FP32 partial sums)
constexpr int MSK_G = 8;   // m values per work item (the k tables' group length)
constexpr int MSK_SP = 2;  // threads per work item
constexpr int MSK_T = 128;
constexpr int MF_S = 32;  // sites per lane group of the force block (one warp's lanes; the kernel assumes 32)
constexpr int MF_GMAX = 16;  // column shares (warps) per force block: 8 or 16 (tuned)
constexpr int MF_KZ = 16;    // z powers held in registers when kmax < MF_KZ
constexpr int SIGN32 = (int)0x80000000u;

GB_D float flipf(float v, int mask) { return __int_as_float(__float_as_int(v) ^ mask); }

// The power tables of ewald_cubic.f90:254-286 / ewald_noncubic.f90:296-336,
// q e^{i k lat x} (x component) and e^{i k lat y}, e^{i k lat z}: for each
// entry the phase in periods, t = k x lat / (2 pi), is reduced modulo 1 in
// two-float arithmetic (exact product k * hi by FMA) and the entry is
// sincospif(2 t) in FP32 (one thread per site axis and its K1 entries: one
// thread per entry, repeating the FP64 product, measured 10 % slower).  The reference's recurrence over k in FP64 rounded
// to FP32 and this direct form differ by a few FP32 ulps.  per = lat / (2 pi).
__global__ void k_recip_tables_mx(const double *rs, const double *q, int na, int B, int kmax, double3 per,
                                  float2 *tab) {
  // one thread per (configuration, site, axis): the FP64 product and its
  // two-float split once, then the K1 powers (the same FP32 operations per m
  // as one thread per entry, without repeating the FP64 work K1 times)
  const int K1 = kmax + 1;
  const long long w = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (w >= 3LL * na * B) return;
  const int ax = (int)(w % 3);
  const int s = (int)((w / 3) % na);
  float fh, fl;
  d2df((ax == 0 ? per.x : ax == 1 ? per.y : per.z) * rs[w], fh, fl);
  const float a = ax == 0 ? __double2float_rn(q[s]) : 1.0f;
  float2 *o = tab + w * K1;
  o[0] = make_float2(a, 0.f);
  for (int k = 1; k < K1; ++k) {
    const float kf = (float)k;
    const float pr = kf * fh;
    const float pe = fmaf(kf, fh, -pr);  // k fh = pr + pe exactly
    const float t = (pr - rintf(pr)) + fmaf(kf, fl, pe);
    float sn, cs;
    sincospif(2.0f * t, &sn, &cs);
    o[k] = make_float2(a * cs, a * sn);
  }
}

// SP threads share a work item, each taking MSK_G / SP of its m values (more
// warps for the same work: the site loop is latency-bound at one thread per item)
template <int SP>
__global__ void __launch_bounds__(MSK_T) k_recip_sk_mx(const float2 *tab, int na, int kmax, int ngrp,
                                                       const int4 *grp, int nkp, int nchunk, float4 *sk_part) {
  constexpr int GP = MSK_G / SP;  // m values per thread
  extern __shared__ float2 stf[];  // [MSK_CHUNK][3][K1]
  const int K1 = kmax + 1, K3 = 3 * K1;
  const int c = blockIdx.z, chunk = blockIdx.y;
  const int s0 = chunk * MSK_CHUNK, ns = min(MSK_CHUNK, na - s0);
  const float2 *src = tab + ((long long)c * na + s0) * K3;
  for (int w = threadIdx.x; w < ns * K3; w += MSK_T) stf[w] = src[w];
  __syncthreads();
  const int tg = blockIdx.x * MSK_T + threadIdx.x;
  const int gi = tg / SP, part = tg % SP;
  if (gi >= ngrp) return;
  const int4 gr = __ldg(grp + gi);
  const int kx = gr.x & 0xffff, ky = gr.y;
  const int len = min(GP, (gr.x >> 16) - part * GP), m0 = gr.z + part * GP;
  if (len <= 0) return;
  const int aky = abs(ky);
  const int ymask = ky < 0 ? SIGN32 : 0;
  // paired sums: (P_r, Q_r) and (P_i, Q_i) of each m, the (cos, sin) of m z
  // times the real or imaginary part of the column's factor
  float2 rq[GP], iq[GP];
#pragma unroll
  for (int g = 0; g < GP; ++g) rq[g] = iq[g] = make_float2(0.f, 0.f);
  for (int s = 0; s < ns; ++s) {
    const float2 *S = stf + s * K3;
    const float2 X = S[kx], Y = S[K1 + aky];
    const float yi = flipf(Y.y, ymask);
    const float cr = fmaf(X.x, Y.x, -X.y * yi);
    const float ci = fmaf(X.x, yi, X.y * Y.x);
    const float2 cr2 = make_float2(cr, cr), ci2 = make_float2(ci, ci);
    const float2 *Z = S + 2 * K1 + m0;
#pragma unroll
    for (int g = 0; g < GP; ++g) {
      if (g < len) {
        const float2 z = Z[g];
        rq[g] = fma2(cr2, z, rq[g]);
        iq[g] = fma2(ci2, z, iq[g]);
      }
    }
  }
  float4 *out = sk_part + ((long long)c * nchunk + chunk) * nkp + gr.w + part * GP;
#pragma unroll
  for (int g = 0; g < GP; ++g)
    if (g < len) out[g] = make_float4(rq[g].x, iq[g].x, rq[g].y, iq[g].y);
}

// df (two-float) sums of the chunk partials; energy, virial and force tables
// per k pair in FP32 (one warp per block), energy and virial summed as df
// across the warp and in FP64 across blocks
// chunk slices per k pair in the weights kernel (SL warps per block): 16 for
// many chunks, fewer when the configuration has few sites (idle warps otherwise)

template <int MW_SL>
__global__ void __launch_bounds__(32 * MW_SL) k_recip_weights_mx(const float4 *sk_part, int nchunk, int nkp,
                                                                const int4 *kpair, const double *kw, const double *kvir,
                                                                float4 *sk, double *acc) {
  __shared__ float part[8][MW_SL][32];  // df (hi, lo) of the four sums per slice
  const int lane = threadIdx.x & 31, slice = threadIdx.x >> 5;
  const int c = blockIdx.y;
  const int k = blockIdx.x * 32 + lane;
  float h[4] = {0.f, 0.f, 0.f, 0.f}, l[4] = {0.f, 0.f, 0.f, 0.f};
  if (k < nkp) {
#pragma unroll 4
    for (int ch = slice; ch < nchunk; ch += MW_SL) {
      const float4 p = sk_part[((long long)c * nchunk + ch) * nkp + k];
      df_acc(h[0], l[0], p.x);
      df_acc(h[1], l[1], p.y);
      df_acc(h[2], l[2], p.z);
      df_acc(h[3], l[3], p.w);
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    part[2 * q][slice][lane] = h[q];
    part[2 * q + 1][slice][lane] = l[q];
  }
  __syncthreads();
  if (slice != 0) return;  // warp 0 finishes, in FP32: energy and virial terms per k pair
  float vals[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (k < nkp) {
    float P[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      float H = part[2 * q][0][lane], L = part[2 * q + 1][0][lane];
      for (int j = 1; j < MW_SL; ++j) df_add(H, L, part[2 * q][j][lane], part[2 * q + 1][j][lane]);
      P[q] = H + L;
    }
    const float Pr = P[0], Pi = P[1], Qr = P[2], Qi = P[3];
    const int4 kv = kpair[k];
    const float w = d2f(kw[k]);
    float et, ed = 0.f, Ar, Ai, Dr, Di;  // ed: et(+m) - et(-m)
    if (kv.w == 1) {
      et = 2.f * w * (Pr * Pr + Pi * Pi + Qr * Qr + Qi * Qi);
      ed = 4.f * w * (Pi * Qr - Pr * Qi);
      Ar = 4.f * w * Pr;
      Ai = 4.f * w * Pi;
      Dr = -4.f * w * Qi;
      Di = 4.f * w * Qr;
    } else if (kv.w == 2) {
      const float sr = Pr - Qi, si = Pi + Qr;
      et = w * (sr * sr + si * si);
      Ar = Dr = 2.f * w * sr;
      Ai = Di = 2.f * w * si;
    } else {
      et = w * (Pr * Pr + Pi * Pi);
      Ar = 2.f * w * Pr;
      Ai = 2.f * w * Pi;
      Dr = Di = 0.f;
    }
    vals[0] = et;
    // virial factors (gb_kvec.h): [0..8] on the summed energy, [9], [10] on
    // the difference for xz, yz (non-cubic sum only)
    const double *kf = kvir + (long long)GB_KVIR * k;
#pragma unroll
    for (int e = 0; e < 9; ++e) vals[1 + e] = et * d2f(kf[e]);
    const float f9 = d2f(kf[9]), f10 = d2f(kf[10]);
    vals[1 + 6] += ed * f9;
    vals[1 + 2] += ed * f9;
    vals[1 + 7] += ed * f10;
    vals[1 + 5] += ed * f10;
    const float m = (float)kv.z;
    // ordered for the force pass's paired products: (Ar, Di) and (-Ai, Dr)
    // multiply (cos, sin) of m z into the real and imaginary parts of the x, y
    // term, (m Dr, m Ai) and (-m Di, m Ar) into those of the z term
    float4 *o = sk + ((long long)c * nkp + k) * 2;
    o[0] = make_float4(Ar, Di, -Ai, Dr);
    o[1] = make_float4(m * Dr, m * Ai, -m * Di, m * Ar);
  }
#pragma unroll
  for (int e = 0; e < 10; ++e) {  // df across the warp, FP64 atomics
    float h = vals[e], l = 0.f;
    warp_sum_df(h, l);
    if (lane == 0 && h != 0.f) atomicAdd(acc + e, df2d(h, l));
  }
}

// one block per 32 sites: its site tables are loaded into shared memory once,
// and each of its MF_G warps takes a share of the columns (by k-pair count);
// the warps' per-site sums are added as df pairs in a fixed order
// STAGED: the whole k-pair table (8 floats per pair) is copied to shared
// memory first, so that the inner loop reads it with shared-memory broadcasts
// NS sites per lane (block of 32 NS sites): every k-pair table entry loaded
// from shared memory serves NS sites.  KZ > 0 (kmax < KZ): each lane keeps its
// sites' z powers (m = 0..KZ-1) in registers, so that the inner loop over m,
// unrolled with a uniform branch per m, loads only the k-pair table entries
// (shared-memory broadcasts) and is FMA-bound; KZ = 0 reads them from shared
// memory in a plain loop.
// gridDim.z splits the k pairs into that many ranges of whole columns (equal
// k-pair counts), one per block of a site tile, so that the grid fills the SMs
// in about even waves; each block stages only its range, and with more than
// one range the blocks of a tile add their sums with FP64 atomics.
template <bool STAGED, int MF_G, int NS, int KZ>
__global__ void __launch_bounds__(32 * MF_G) k_recip_force_mx(const float2 *__restrict__ tab, int na,
                                                                       int kmax, int ncol,
                                                                       const KCol *__restrict__ cols, int nkp,
                                                                       const float4 *__restrict__ sk, double3 lat,
                                                                       double *g) {
  constexpr int BS = MF_S * NS;  // sites per block
  // [3][K1][BS] float2 site tables, [MF_G][BS][3] df sums, then
  // (STAGED) the k-pair table [nkp][2] float4
  extern __shared__ float4 smf[];
  float2 *stf = reinterpret_cast<float2 *>(smf);
  const int K1 = kmax + 1, K3 = 3 * K1;
  const int c = blockIdx.y;
  const int t = threadIdx.x, sl = t % 32, wg = t / 32;
  const int i0 = blockIdx.x * BS;
  for (int w = t; w < K3 * BS; w += 32 * MF_G) {
    const int e = w / BS, s2 = w % BS;
    const int si = min(i0 + s2, na - 1);
    stf[w] = tab[((long long)c * na + si) * K3 + e];
  }
  const int tab_f4 = (K3 * BS + 1) / 2;                       // float4 slots of the site tables
  float2 *red = reinterpret_cast<float2 *>(smf + tab_f4);     // MF_G * BS * 3 df pairs
  int4 *scol = reinterpret_cast<int4 *>(smf + tab_f4 + (MF_G * BS * 3 + 1) / 2);  // [ncol] column records
  float4 *sT = reinterpret_cast<float4 *>(scol + ncol);       // [k pairs of the block][2]
  // the column records in shared memory: the range searches and the loop read
  // them there instead of through dependent global loads
  for (int w = t; w < ncol; w += 32 * MF_G) scol[w] = __ldg(reinterpret_cast<const int4 *>(cols + w));
  __syncthreads();
  auto first_col = [&](long long kp) {
    int lo = 0, hi = ncol;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (scol[mid].z < kp) lo = mid + 1;
      else hi = mid;
    }
    return lo;
  };
  // this block's whole columns and their k pairs [kb_lo, kb_hi)
  const int KS = gridDim.z, ks = blockIdx.z;
  const int bc0 = first_col((long long)ks * nkp / KS), bc1 = first_col((long long)(ks + 1) * nkp / KS);
  const int kb_lo = bc0 < ncol ? scol[bc0].z : nkp;
  const int kb_hi = bc1 < ncol ? scol[bc1].z : nkp;
  if (STAGED) {
    const float4 *src = sk + ((long long)c * nkp + kb_lo) * 2;
    for (int w = t; w < 2 * (kb_hi - kb_lo); w += 32 * MF_G) sT[w] = src[w];
  }
  const long long kp_lo = kb_lo + (long long)wg * (kb_hi - kb_lo) / MF_G;
  const long long kp_hi = kb_lo + (long long)(wg + 1) * (kb_hi - kb_lo) / MF_G;
  const int col0 = max(first_col(kp_lo), bc0), col1 = min(first_col(kp_hi), bc1);
  __syncthreads();
  // k pair kp at T + 2 kp (staged: the block's range starts at sT)
  const float4 *T = STAGED ? sT - 2LL * kb_lo : sk + (long long)c * nkp * 2;
  float2 zr[KZ > 0 ? KZ : 1][NS];
  if constexpr (KZ > 0) {
#pragma unroll
    for (int m = 0; m < KZ; ++m)
#pragma unroll
      for (int u = 0; u < NS; ++u) zr[m][u] = m < K1 ? stf[(2 * K1 + m) * BS + sl + 32 * u] : make_float2(0.f, 0.f);
  }
  float sx[NS], sy[NS], sz[NS], ex[NS], ey[NS], ez[NS];
#pragma unroll
  for (int u = 0; u < NS; ++u) sx[u] = sy[u] = sz[u] = ex[u] = ey[u] = ez[u] = 0.f;
  for (int col = col0; col < col1; ++col) {
    const int4 ci4 = scol[col];
    const int kx = ci4.x, ky = ci4.y, koff = ci4.z, mlo = ci4.w & 0xffff, mhi = ci4.w >> 16;
    // paired sums over m: the two components of each are the cos and sin
    // halves of one sum (added at the column's end)
    float cr[NS], ci[NS];
    float2 ur[NS], ui[NS], vr[NS], vi[NS];
#pragma unroll
    for (int u = 0; u < NS; ++u) {
      const int so = sl + 32 * u;
      const float2 X = stf[kx * BS + so], Y = stf[(K1 + abs(ky)) * BS + so];
      const float yi = flipf(Y.y, ky < 0 ? SIGN32 : 0);
      cr[u] = fmaf(X.x, Y.x, -X.y * yi);
      ci[u] = fmaf(X.x, yi, X.y * Y.x);
      ur[u] = ui[u] = vr[u] = vi[u] = make_float2(0.f, 0.f);
    }
    const float4 *Tp = T + 2LL * (koff - mlo);
    auto step = [&](int m, const float2 (&z)[NS]) {
      float4 t0, t1;
      if (STAGED) {
        t0 = Tp[2 * m];
        t1 = Tp[2 * m + 1];
      } else {
        t0 = __ldg(Tp + 2 * m);
        t1 = __ldg(Tp + 2 * m + 1);
      }
#pragma unroll
      for (int u = 0; u < NS; ++u) {
        ur[u] = fma2(z[u], make_float2(t0.x, t0.y), ur[u]);
        ui[u] = fma2(z[u], make_float2(t0.z, t0.w), ui[u]);
        vr[u] = fma2(z[u], make_float2(t1.x, t1.y), vr[u]);
        vi[u] = fma2(z[u], make_float2(t1.z, t1.w), vi[u]);
      }
    };
    if constexpr (KZ > 0) {
      static_assert(KZ == 16, "the jump below covers m = 0..15");
      // enter at m = mhi and fall through to m = 1 (m = 0 when mlo = 0): one
      // uniform indirect jump per column, no predicated-off steps
      switch (mhi) {
#define GB_ZSTEP(M) \
  case M:           \
    step(M, zr[M]); \
    [[fallthrough]];
        GB_ZSTEP(15) GB_ZSTEP(14) GB_ZSTEP(13) GB_ZSTEP(12) GB_ZSTEP(11) GB_ZSTEP(10) GB_ZSTEP(9) GB_ZSTEP(8)
        GB_ZSTEP(7) GB_ZSTEP(6) GB_ZSTEP(5) GB_ZSTEP(4) GB_ZSTEP(3) GB_ZSTEP(2) GB_ZSTEP(1)
#undef GB_ZSTEP
        case 0:
          if (mlo == 0) step(0, zr[0]);
          break;
        default:
          break;
      }
    } else {
      const float2 *Z = stf + 2 * K1 * BS + sl;
#pragma unroll 4
      for (int m = mlo; m <= mhi; ++m) {
        float2 z[NS];
#pragma unroll
        for (int u = 0; u < NS; ++u) z[u] = Z[m * BS + 32 * u];
        step(m, z);
      }
    }
#pragma unroll
    for (int u = 0; u < NS; ++u) {
      const float urs = ur[u].x + ur[u].y, uis = ui[u].x + ui[u].y;
      const float vrs = vr[u].x + vr[u].y, vis = vi[u].x + vi[u].y;
      const float ts = -fmaf(cr[u], uis, ci[u] * urs);
      kadd(sx[u], ex[u], (float)kx * ts);
      kadd(sy[u], ey[u], (float)ky * ts);
      kadd(sz[u], ez[u], -fmaf(cr[u], vis, ci[u] * vrs));
    }
  }
#pragma unroll
  for (int u = 0; u < NS; ++u) {
    const int so = sl + 32 * u;
    red[(wg * BS + so) * 3] = make_float2(sx[u], -ex[u]);
    red[(wg * BS + so) * 3 + 1] = make_float2(sy[u], -ey[u]);
    red[(wg * BS + so) * 3 + 2] = make_float2(sz[u], -ez[u]);
  }
  __syncthreads();
  for (int w2 = t; w2 < 3 * BS; w2 += 32 * MF_G) {
    const int s2 = w2 / 3, d = w2 % 3;
    float H = 0.f, L = 0.f;
    for (int w = 0; w < MF_G; ++w) {
      const float2 r = red[(w * BS + s2) * 3 + d];
      df_add(H, L, r.x, r.y);
    }
    if (i0 + s2 < na) {
      double *gd = g + ((long long)c * na + i0 + s2) * 3 + d;
      const double v = (d == 0 ? lat.x : d == 1 ? lat.y : lat.z) * df2d(H, L);
      if (KS > 1) atomicAdd(gd, v);
      else *gd += v;
    }
  }
}

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

int sm_count_mx() {
  int dev = 0, n = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) return 1;
  return n;
}

}  // namespace

void launch_ewald_real_mx(cudaStream_t s, const int4 *fx, const int4 *fxs, int na, int B, const PairList &pl,
                          double alpha, double rcutsq, const double *box, int np, double *g, double *acc, bool add,
                          unsigned long long *npair) {
  const float two32 = 2.3283064365386963e-10f;  // 2^-32: fixed-point units to fractions
  const float3 bx = make_float3((float)box[0] * two32, (float)box[1] * two32, (float)box[2] * two32);
  const float sfac = (float)(-2.0 * alpha / std::sqrt(std::acos(-1.0)));  // d erfc(alpha r) / dr factor
  const unsigned short *i16 = reinterpret_cast<const unsigned short *>(pl.idx);
  auto go = [&](auto NPc) {
    constexpr int NP = decltype(NPc)::value;
    dim3 grid(nblk((long long)na * NP, MX_T), B);
    const int lconf = pl.nconf == 1 ? 0 : 1;  // one list shared by the B configurations
    if (pl.slots)
      k_ewald_real_mx<NP, unsigned short, true><<<grid, MX_T, 0, s>>>(
          fx, fxs, na, pl.count, i16, pl.cap, (float)alpha, sfac, (float)rcutsq, bx, g, acc, add ? 1 : 0, npair,
          lconf);
    else if (pl.i16)
      k_ewald_real_mx<NP, unsigned short, false><<<grid, MX_T, 0, s>>>(
          fx, fx, na, pl.count, i16, pl.cap, (float)alpha, sfac, (float)rcutsq, bx, g, acc, add ? 1 : 0, npair,
          lconf);
    else
      k_ewald_real_mx<NP, int, false><<<grid, MX_T, 0, s>>>(fx, fx, na, pl.count, pl.idx, pl.cap, (float)alpha, sfac,
                                                            (float)rcutsq, bx, g, acc, add ? 1 : 0, npair, lconf);
  };
  if (const char *e = std::getenv("GBRPMD_EW_NP")) np = std::atoi(e);  // fixed lanes per site (measurements)
  if (np == 8) go(std::integral_constant<int, 8>());
  else if (np == 32) go(std::integral_constant<int, 32>());
  else go(std::integral_constant<int, 16>());
}

void launch_lj_mx(cudaStream_t s, const float4 *hi, const float4 *lo, int na, int B, const PairList &pl,
                  double sigsq, double rcutsq, const double *box, double dscale, int np, double *out, double *acc) {
  const int npt = na / 3;
  const float3 bx = make_float3((float)box[0], (float)box[1], (float)box[2]);
  auto go = [&](auto NPc) {
    constexpr int NP = decltype(NPc)::value;
    dim3 grid(nblk((long long)npt * NP, MX_T), B);
    k_lj_mx<NP><<<grid, MX_T, 0, s>>>(hi, lo, na, npt, pl.nconf, pl.count, pl.idx, pl.cap, (float)sigsq,
                                      (float)rcutsq, bx, dscale, out, acc);
  };
  if (np == 2) go(std::integral_constant<int, 2>());
  else if (np == 8) go(std::integral_constant<int, 8>());
  else go(std::integral_constant<int, 4>());
}

size_t recip_sk_smem_mx(int kmax) { return sizeof(float2) * MSK_CHUNK * 3 * (kmax + 1); }
// dynamic shared memory of k_recip_force_mx<., g, ns>
size_t recip_force_smem_mx(int kmax, int nkp_staged, int g, int ns, int ncol) {
  const int bs = MF_S * ns;
  return sizeof(float4) * ((3 * (kmax + 1) * bs + 1) / 2 + (g * bs * 3 + 1) / 2 + (size_t)ncol +
                           2 * (size_t)nkp_staged);
}

// partial sums need nconf * nchunk * nkp float4 (half of the FP64 layout)
void launch_recip_sk_mx(cudaStream_t s, gb_context *c, const double *rs, const double *q, int B) {
  if (c->nkp == 0) return;
  const int kmax = c->P.kmax;
  const long long nw = 3LL * c->na * B;
  float2 *tab = reinterpret_cast<float2 *>(c->ktab);
  const double3 lat = recip_lat(c);
  const double ot = 0.5 / std::acos(-1.0);
  k_recip_tables_mx<<<nblk(nw, 128), 128, 0, s>>>(rs, q, c->na, B, kmax,
                                                 make_double3(lat.x * ot, lat.y * ot, lat.z * ot), tab);
  const int nchunk = (c->na + MSK_CHUNK - 1) / MSK_CHUNK;
  // GBRPMD_SK_TC=1 puts the structure factors on the tensor cores (k_recip_tc.cu;
  // kmax < 16): measured at 4096 H2O, nb = 32 it takes 24-34 us per launch
  // against 17 us for the CUDA-core kernel below, so it is not the default
  const char *tc = std::getenv("GBRPMD_SK_TC");
  if (tc && tc[0] == '1' && recip_sk_tc_chunk() == MSK_CHUNK && launch_recip_sk_tc(s, c, B, nchunk)) return;
  static_assert(MSK_G % MSK_SP == 0, "work item split");
  dim3 grid(nblk((long long)c->ngrp * MSK_SP, MSK_T), nchunk, B);
  k_recip_sk_mx<MSK_SP><<<grid, MSK_T, recip_sk_smem_mx(kmax), s>>>(tab, c->na, kmax, c->ngrp, c->kgrp, c->nkp,
                                                                   nchunk, reinterpret_cast<float4 *>(c->sk_part));
}

void launch_recip_weights_mx(cudaStream_t s, gb_context *c, int B, double *acc) {
  if (c->nkp == 0) return;
  const int nchunk = (c->na + MSK_CHUNK - 1) / MSK_CHUNK;
  dim3 grid(nblk(c->nkp, 32), B);
  auto go = [&](auto SLc) {
    constexpr int SL = decltype(SLc)::value;
    k_recip_weights_mx<SL><<<grid, 32 * SL, 0, s>>>(reinterpret_cast<const float4 *>(c->sk_part), nchunk, c->nkp,
                                                    c->kpair, c->kw, c->kvir, reinterpret_cast<float4 *>(c->sk), acc);
  };
  if (nchunk <= 4) go(std::integral_constant<int, 4>());
  else if (nchunk <= 8) go(std::integral_constant<int, 8>());
  else go(std::integral_constant<int, 16>());  // (32 slices measured 3 % slower on 192 chunks)
}

template <bool STAGED, int G, int NS, int KZ>
void force_attr() {
  cudaFuncSetAttribute(k_recip_force_mx<STAGED, G, NS, KZ>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
}

template <int G, int NS, int KZ>
void force_launch(cudaStream_t s, gb_context *c, int B, double *g) {
  static_assert(G <= MF_GMAX, "column shares");
  const int kmax = c->P.kmax;
  int ks = c->tune.rf_ks;
  if (const char *e = std::getenv("GBRPMD_RF_KS")) ks = std::atoi(e);  // fixed k-pair ranges (measurements)
  ks = std::max(1, std::min(ks, std::max(1, c->nkp / 64)));
  // a block stages its share of the k pairs and at most one column more
  const size_t staged = recip_force_smem_mx(kmax, (c->nkp + ks - 1) / ks + 2 * (kmax + 1) + 2, G, NS, c->ncol);
  dim3 grid(nblk(c->na, MF_S * NS), B, ks);
  if (staged <= 160 * 1024)
    k_recip_force_mx<true, G, NS, KZ><<<grid, 32 * G, staged, s>>>(
        reinterpret_cast<const float2 *>(c->ktab), c->na, kmax, c->ncol, c->kcol, c->nkp,
        reinterpret_cast<const float4 *>(c->sk), recip_lat(c), g);
  else
    k_recip_force_mx<false, G, NS, KZ><<<grid, 32 * G, recip_force_smem_mx(kmax, 0, G, NS, c->ncol), s>>>(
        reinterpret_cast<const float2 *>(c->ktab), c->na, kmax, c->ncol, c->kcol, c->nkp,
        reinterpret_cast<const float4 *>(c->sk), recip_lat(c), g);
}

bool recip_force_tc_on(const gb_context *c) {
  const char *v = std::getenv("GBRPMD_RF_TC");
  return !(v && v[0] == '0') && c->P.kmax + 1 <= 16;
}

void launch_recip_force_mx(cudaStream_t s, gb_context *c, int B, double *g) {
  if (c->nkp == 0) return;
  // the force pass on the tensor cores (k_recip_tc.cu) unless GBRPMD_RF_TC=0
  // asks for the CUDA-core pass below (also taken when kmax + 1 > 16)
  const char *tcv = std::getenv("GBRPMD_RF_TC");
  if (!(tcv && tcv[0] == '0') && launch_recip_force_tc(s, c, B, g)) return;
  const bool zr = c->P.kmax < MF_KZ;  // z powers in registers
  const int v = (c->tune.rf_g == 16 ? 4 : 0) + (c->tune.rf_ns == 2 ? 2 : 0) + (zr ? 1 : 0);
  switch (v) {
    case 0: force_launch<8, 1, 0>(s, c, B, g); break;
    case 1: force_launch<8, 1, MF_KZ>(s, c, B, g); break;
    case 2: force_launch<8, 2, 0>(s, c, B, g); break;
    case 3: force_launch<8, 2, MF_KZ>(s, c, B, g); break;
    case 4: force_launch<16, 1, 0>(s, c, B, g); break;
    case 5: force_launch<16, 1, MF_KZ>(s, c, B, g); break;
    case 6: force_launch<16, 2, 0>(s, c, B, g); break;
    default: force_launch<16, 2, MF_KZ>(s, c, B, g); break;
  }
}

void recip_set_attributes_mx() {
  static bool done = false;
  if (done) return;
  cudaFuncSetAttribute(k_recip_sk_mx<MSK_SP>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);

  force_attr<true, 8, 1, 0>();
  force_attr<false, 8, 1, 0>();
  force_attr<true, 8, 1, MF_KZ>();
  force_attr<false, 8, 1, MF_KZ>();
  force_attr<true, 8, 2, 0>();
  force_attr<false, 8, 2, 0>();
  force_attr<true, 8, 2, MF_KZ>();
  force_attr<false, 8, 2, MF_KZ>();
  force_attr<true, 16, 1, 0>();
  force_attr<false, 16, 1, 0>();
  force_attr<true, 16, 1, MF_KZ>();
  force_attr<false, 16, 1, MF_KZ>();
  force_attr<true, 16, 2, 0>();
  force_attr<false, 16, 2, 0>();
  force_attr<true, 16, 2, MF_KZ>();
  force_attr<false, 16, 2, MF_KZ>();
  done = true;
}
