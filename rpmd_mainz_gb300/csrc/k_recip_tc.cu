// k_recip_tc.cu -- the structure factors of the mixed k-space sum (kwald,
// ewald_cubic.f90:235-533; kwald_nc, ewald_noncubic.f90) as a product on the
// tensor cores.
//
// For one configuration and a chunk of sites, with C_s = q_s e^{i kx x_s}
// e^{i ky y_s} per (kx, ky) column and Z_s[m] = e^{i m z_s}:
//   P_m = sum_s C_s Re Z_s[m],  Q_m = sum_s C_s Im Z_s[m]
// (S(kx, ky, +-m) = P_m +- i Q_m), i.e. the real product D = A B of
//   A [(column, re / im)][site] = (Re C_s, Im C_s),
//   B [site][(m, cos / sin)]    = (Re Z_s[m], Im Z_s[m]),
// 2 x (#columns) by 2 (kmax + 1) over the chunk's sites.  A warp takes 8
// columns (A rows: the real parts of the 8 columns, then their imaginary
// parts) and all m: per step of 8 sites each lane forms the two C_s its
// operand registers hold from the power tables in shared memory, and mma.sync
// m16n8k8 TF32 products accumulate D in FP32, every operand split into two
// TF32 terms (hi * hi + hi * lo + lo * hi: ~2^-22 per product).  In the
// accumulator layout lane (g, t) of n-tile j holds, for column g and
// m = 4 j + t, exactly (Re P_m, Re Q_m, Im P_m, Im Q_m), which it stores as the
// k pair's chunk partial (the same [chunk][k pair] float4 (Pr, Pi, Qr, Qi)
// layout that the CUDA-core kernel writes and k_recip_weights_mx reduces in
// two-float arithmetic).  Chunks of 64 sites keep each accumulator to 8 steps.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>

#include "gb_common.cuh"
#include "gb_df.cuh"
#include "gb_context.h"
#include "gb_kernels.h"

namespace {

constexpr int TC_CHUNK = 64;  // sites per chunk: the partials' layout of the weights kernel
constexpr int TC_WARPS = 8;   // column tiles (8 columns each) per block
constexpr int SIGN32 = (int)0x80000000u;

GB_D unsigned tf32_rna(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

GB_D void mma_tf32(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3, unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

GB_D void split_tf32(float v, unsigned &h, unsigned &l) {
  h = tf32_rna(v);
  l = tf32_rna(v - __uint_as_float(h));
}

// NT n-tiles of 8: m = 0 .. 4 NT - 1 (kmax < 4 NT)
template <int NT>
__global__ void __launch_bounds__(32 * TC_WARPS) k_recip_sk_tc(const float2 *__restrict__ tab, int na, int kmax,
                                                               int ncol, const KCol *__restrict__ cols, int nkp,
                                                               int nchunk, float4 *__restrict__ sk_part) {
  extern __shared__ float2 stf[];  // [TC_CHUNK][3][K1]
  const int K1 = kmax + 1, K3 = 3 * K1;
  const int c = blockIdx.z, chunk = blockIdx.y;
  const int s0 = chunk * TC_CHUNK, ns = min(TC_CHUNK, na - s0);
  const float2 *src = tab + ((long long)c * na + s0) * K3;
  for (int w = threadIdx.x; w < TC_CHUNK * K3; w += blockDim.x) stf[w] = w < ns * K3 ? src[w] : make_float2(0.f, 0.f);
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  const int ctile = blockIdx.x * TC_WARPS + (threadIdx.x >> 5);
  if (ctile * 8 >= ncol) return;  // the whole warp
  const int col = ctile * 8 + g;
  int kx = 0, ky = 0, koff = 0, mlo = 1, mhi = 0;  // columns past the end store nothing
  if (col < ncol) {
    const int4 ci4 = __ldg(reinterpret_cast<const int4 *>(cols + col));
    kx = ci4.x, ky = ci4.y, koff = ci4.z, mlo = ci4.w & 0xffff, mhi = ci4.w >> 16;
  }
  const int aky = ky < 0 ? -ky : ky;
  const int ymask = ky < 0 ? SIGN32 : 0;
  // the three products in separate accumulators (independent MMA chains)
  float acc[NT][4], accl[NT][4], accm[NT][4];
#pragma unroll
  for (int j = 0; j < NT; ++j)
#pragma unroll
    for (int e = 0; e < 4; ++e) acc[j][e] = accl[j][e] = accm[j][e] = 0.f;
  // B columns of this lane: n = 8 j + g -> m = 4 j + g / 2, cos (g even) or sin
  const int mb = g >> 1, part = g & 1;
#pragma unroll 2
  for (int k8 = 0; k8 < TC_CHUNK; k8 += 8) {
    // A: Re / Im C of column g at sites k8 + t (a0, a1) and k8 + t + 4 (a2, a3)
    unsigned ah[4], al[4];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const float2 *S = stf + (k8 + t + 4 * h) * K3;
      const float2 X = S[kx], Y = S[K1 + aky];
      const float yi = __int_as_float(__float_as_int(Y.y) ^ ymask);
      const float cr = fmaf(X.x, Y.x, -X.y * yi);
      const float cim = fmaf(X.x, yi, X.y * Y.x);
      split_tf32(cr, ah[2 * h], al[2 * h]);        // a0 / a2: row g (real part)
      split_tf32(cim, ah[2 * h + 1], al[2 * h + 1]);  // a1 / a3: row g + 8 (imaginary part)
    }
#pragma unroll
    for (int j = 0; j < NT; ++j) {
      const int m = 4 * j + mb;
      unsigned bh[2], bl[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        float v = 0.f;
        if (m < K1) {
          const float2 z = stf[(k8 + t + 4 * h) * K3 + 2 * K1 + m];
          v = part ? z.y : z.x;
        }
        split_tf32(v, bh[h], bl[h]);
      }
      // operand order (a0, a1, a2, a3) = (row g, k t), (row g+8, k t), (row g, k t+4), (row g+8, k t+4)
      mma_tf32(accl[j], al[0], al[1], al[2], al[3], bh[0], bh[1]);
      mma_tf32(accm[j], ah[0], ah[1], ah[2], ah[3], bl[0], bl[1]);
      mma_tf32(acc[j], ah[0], ah[1], ah[2], ah[3], bh[0], bh[1]);
    }
  }
  // (c0, c1, c2, c3) = (Re P_m, Re Q_m, Im P_m, Im Q_m) for column g, m = 4 j + t
  float4 *out = sk_part + ((long long)c * nchunk + chunk) * nkp;
#pragma unroll
  for (int j = 0; j < NT; ++j) {
    const int m = 4 * j + t;
    if (m >= mlo && m <= mhi)
      out[koff + (m - mlo)] = make_float4(acc[j][0] + (accl[j][0] + accm[j][0]), acc[j][2] + (accl[j][2] + accm[j][2]),
                                          acc[j][1] + (accl[j][1] + accm[j][1]), acc[j][3] + (accl[j][3] + accm[j][3]));
  }
}

// The k-space force pass as a product on the tensor cores.  For a column
// (kx, ky) and a site, the four sums of the force pass over the column's m
// range are U_o = sum_m (cos m z, sin m z) . T_o[m] (o = ur, ui, vr, vi; T the
// force table of the k pair, stored as the (cos, sin) coefficient pairs of
// each o), i.e. the real product U = A B with
//   A [site][2 m + s] = (cos m z, sin m z)[s]        (the site's z powers),
//   B [2 m + s][4 col + o] = T_o[m][s]               (zero outside the m range),
// K = 2 (kmax + 1) <= 32, and the site's column factor c = X[kx] Y[ky]
// enters only afterwards: ts = -(c_r ui + c_i ur) gives the x and y terms
// (kx ts, ky ts) and -(c_r vi + c_i vr) the z term, as in k_recip_force_mx.
// A block takes 64 sites (four warps of 16 rows) and a share of the column
// tiles (8 columns, N = 32); a warp keeps its A fragments (split into two
// TF32 terms) in registers for all its tiles, the block stages each tile's B
// (split) in shared memory, and mma.sync m16n8k8 TF32 forms hi hi + hi lo +
// lo hi.  In the accumulator layout lane (g, t) of n-tile j holds, for rows g
// and g + 8, outputs 2t and 2t + 1 of column 2j + t / 2: (ur, ui) for even t,
// (vr, vi) for odd t, so that even lanes sum the x and y terms and odd lanes
// the z term (compensated), combined across the lanes of a row at the end.
constexpr int RF_SPB = 64;    // sites per block
constexpr int RF_BLD = 40;    // row stride of the staged B tile (conflict-free fragment loads)
constexpr int SIGN32F = (int)0x80000000u;

__global__ void __launch_bounds__(128) k_recip_force_tc(const float2 *__restrict__ tab, int na, int kmax, int ncol,
                                                        const KCol *__restrict__ cols, int nkp,
                                                        const float4 *__restrict__ sk, double3 lat, double *g) {
  extern __shared__ float smr[];
  const int K1 = kmax + 1, K3 = 3 * K1;
  float2 *stf = reinterpret_cast<float2 *>(smr);        // [RF_SPB][3][K1]
  float *sbh = smr + 2 * RF_SPB * K3;                   // [32][RF_BLD] B tile, hi
  float *sbl = sbh + 32 * RF_BLD;                       // lo
  int4 *scol = reinterpret_cast<int4 *>(sbl + 32 * RF_BLD);  // [8] the tile's column records
  const int c = blockIdx.y;
  const int s0 = blockIdx.x * RF_SPB, ns = min(RF_SPB, na - s0);
  const int tid = threadIdx.x;
  const float2 *src = tab + ((long long)c * na + s0) * K3;
  for (int w = tid; w < RF_SPB * K3; w += 128) stf[w] = w < ns * K3 ? src[w] : make_float2(0.f, 0.f);
  __syncthreads();
  const int warp = tid >> 5, lane = tid & 31, gq = lane >> 2, tq = lane & 3;
  const int r0 = warp * 16 + gq, r1 = r0 + 8;  // the lane's two site rows
  // A fragments: a0 = A[r0][8 ks + tq], a1 = A[r1][.], a2 = A[r0][8 ks + tq + 4], a3 = A[r1][.]
  unsigned ah[4][4], al[4][4];
#pragma unroll
  for (int ks = 0; ks < 4; ++ks)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const int r = (e & 1) ? r1 : r0;
      const int kk = 8 * ks + tq + ((e & 2) ? 4 : 0);
      const int m = kk >> 1;
      float v = 0.f;
      if (m < K1) {
        const float2 z = stf[r * K3 + 2 * K1 + m];
        v = (kk & 1) ? z.y : z.x;
      }
      split_tf32(v, ah[ks][e], al[ks][e]);
    }
  // this block's column tiles
  const int ntile = (ncol + 7) / 8;
  const int t_lo = (int)((long long)blockIdx.z * ntile / gridDim.z);
  const int t_hi = (int)((long long)(blockIdx.z + 1) * ntile / gridDim.z);
  float sa = 0.f, ca = 0.f, sb = 0.f, cb = 0.f;  // row r0: x (even lanes) or z (odd); y (even lanes)
  float sa1 = 0.f, ca1 = 0.f, sb1 = 0.f, cb1 = 0.f;  // row r1
  auto kadd = [](float &s, float &cc, float v) {
    const float y = v - cc;
    const float t = s + y;
    cc = (t - s) - y;
    s = t;
  };
  const float4 *T = sk + (long long)c * nkp * 2;
  for (int tile = t_lo; tile < t_hi; ++tile) {
    const int col0 = 8 * tile;
    __syncthreads();  // the previous tile's B is consumed
    if (tid < 8) {
      const int col = col0 + tid;
      scol[tid] = col < ncol ? __ldg(reinterpret_cast<const int4 *>(cols + col)) : make_int4(0, 0, 0, 1);  // mlo 1 > mhi 0
    }
    __syncthreads();
    // B: 16 m x 8 columns x 2 halves of the k pair's table (t0: ur, ui; t1: vr, vi)
    for (int w = tid; w < 256; w += 128) {
      const int m = w >> 4, cl = (w >> 1) & 7, half = w & 1;
      const int4 ci = scol[cl];
      const int mlo = ci.w & 0xffff, mhi = ci.w >> 16;
      float4 t = make_float4(0.f, 0.f, 0.f, 0.f);
      if (m >= mlo && m <= mhi) t = T[2LL * (ci.z + m - mlo) + half];
      const int n0 = 4 * cl + 2 * half;  // outputs (ur, ui) or (vr, vi)
      unsigned h, l;
      split_tf32(t.x, h, l); sbh[(2 * m) * RF_BLD + n0] = __uint_as_float(h); sbl[(2 * m) * RF_BLD + n0] = __uint_as_float(l);
      split_tf32(t.y, h, l); sbh[(2 * m + 1) * RF_BLD + n0] = __uint_as_float(h); sbl[(2 * m + 1) * RF_BLD + n0] = __uint_as_float(l);
      split_tf32(t.z, h, l); sbh[(2 * m) * RF_BLD + n0 + 1] = __uint_as_float(h); sbl[(2 * m) * RF_BLD + n0 + 1] = __uint_as_float(l);
      split_tf32(t.w, h, l); sbh[(2 * m + 1) * RF_BLD + n0 + 1] = __uint_as_float(h); sbl[(2 * m + 1) * RF_BLD + n0 + 1] = __uint_as_float(l);
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
      for (int ks = 0; ks < 4; ++ks) {
        const int rb = (8 * ks + tq) * RF_BLD + 8 * j + gq;
        const unsigned bh0 = __float_as_uint(sbh[rb]), bh1 = __float_as_uint(sbh[rb + 4 * RF_BLD]);
        const unsigned bl0 = __float_as_uint(sbl[rb]), bl1 = __float_as_uint(sbl[rb + 4 * RF_BLD]);
        mma_tf32(acc, al[ks][0], al[ks][1], al[ks][2], al[ks][3], bh0, bh1);
        mma_tf32(acc, ah[ks][0], ah[ks][1], ah[ks][2], ah[ks][3], bl0, bl1);
        mma_tf32(acc, ah[ks][0], ah[ks][1], ah[ks][2], ah[ks][3], bh0, bh1);
      }
      // column 2j + tq / 2 of the tile; (acc0, acc1) row r0, (acc2, acc3) row r1
      const int4 ci = scol[2 * j + (tq >> 1)];
      const int kx = ci.x, ky = ci.y;
      const int aky = ky < 0 ? -ky : ky, ymask = ky < 0 ? SIGN32F : 0;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = h ? r1 : r0;
        const float2 X = stf[r * K3 + kx], Y = stf[r * K3 + K1 + aky];
        const float yi = __int_as_float(__float_as_int(Y.y) ^ ymask);
        const float cr = fmaf(X.x, Y.x, -X.y * yi);
        const float cim = fmaf(X.x, yi, X.y * Y.x);
        const float u0 = acc[2 * h], u1 = acc[2 * h + 1];  // (ur, ui) or (vr, vi)
        const float v = -fmaf(cr, u1, cim * u0);
        float &s_a = h ? sa1 : sa, &c_a = h ? ca1 : ca, &s_b = h ? sb1 : sb, &c_b = h ? cb1 : cb;
        if ((tq & 1) == 0) {
          kadd(s_a, c_a, (float)kx * v);
          kadd(s_b, c_b, (float)ky * v);
        } else {
          kadd(s_a, c_a, v);  // z term
        }
      }
    }
  }
  // per row: x, y from the even lanes (tq 0, 2), z from the odd (1, 3)
  float hx0 = sa, lx0 = -ca, hy0 = sb, ly0 = -cb, hx1 = sa1, lx1 = -ca1, hy1 = sb1, ly1 = -cb1;
  auto pair_add = [](float &h, float &l) {
    const float oh = __shfl_xor_sync(0xffffffffu, h, 2), ol = __shfl_xor_sync(0xffffffffu, l, 2);
    df_add(h, l, oh, ol);
  };
  pair_add(hx0, lx0);
  pair_add(hy0, ly0);
  pair_add(hx1, lx1);
  pair_add(hy1, ly1);
  // lane tq = 0 holds x, y of its rows; tq = 1 holds z (in its x slot)
  const bool multi = gridDim.z > 1;
  auto put = [&](int r, int d, float h, float l) {
    if (s0 + r >= na) return;
    double *gd = g + ((long long)c * na + s0 + r) * 3 + d;
    const double v = (d == 0 ? lat.x : d == 1 ? lat.y : lat.z) * df2d(h, l);
    if (multi) atomicAdd(gd, v);
    else *gd += v;
  };
  if (tq == 0) {
    put(r0, 0, hx0, lx0);
    put(r0, 1, hy0, ly0);
    put(r1, 0, hx1, lx1);
    put(r1, 1, hy1, ly1);
  } else if (tq == 1) {
    put(r0, 2, hx0, lx0);
    put(r1, 2, hx1, lx1);
  }
}

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

// false when kmax is beyond the kernel's K = 32 (kmax + 1 > 16)
bool launch_recip_force_tc(cudaStream_t s, gb_context *c, int B, double *g) {
  const int kmax = c->P.kmax;
  if (kmax + 1 > 16 || c->nkp == 0) return false;
  const size_t smem = sizeof(float) * (2 * RF_SPB * 3 * (kmax + 1) + 2 * 32 * RF_BLD) + sizeof(int4) * 8;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_recip_force_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, 64 * 1024);
    attr = true;
  }
  // column-tile ranges per block (grid.z, forces added by FP64 atomics when
  // more than one): enough blocks for every SM
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const int nsb = (int)nblk(c->na, RF_SPB) * B;
  const int ntile = (c->ncol + 7) / 8;
  int ksp = 1;
  while (ksp < ntile && nsb * ksp < 4 * nsm) ksp *= 2;
  if (const char *e = std::getenv("GBRPMD_RF_TC_KS")) ksp = std::max(1, std::atoi(e));
  ksp = std::min(ksp, ntile);
  dim3 grid(nblk(c->na, RF_SPB), B, ksp);
  k_recip_force_tc<<<grid, 128, smem, s>>>(reinterpret_cast<const float2 *>(c->ktab), c->na, kmax, c->ncol,
                                           c->kcol, c->nkp, reinterpret_cast<const float4 *>(c->sk),
                                           recip_lat(c), g);
  return true;
}

int recip_sk_tc_chunk() { return TC_CHUNK; }

// false when kmax is beyond the tensor-core kernel's tiles (kmax + 1 > 16)
bool launch_recip_sk_tc(cudaStream_t s, gb_context *c, int B, int nchunk) {
  const int kmax = c->P.kmax;
  if (kmax + 1 > 16 || c->nkp == 0) return false;
  const size_t smem = sizeof(float2) * TC_CHUNK * 3 * (kmax + 1);
  dim3 grid(nblk(c->ncol, 8 * TC_WARPS), nchunk, B);
  const float2 *tab = reinterpret_cast<const float2 *>(c->ktab);
  float4 *part = reinterpret_cast<float4 *>(c->sk_part);
  const int nt = (kmax + 4) / 4;  // n-tiles covering m = 0 .. kmax
  switch (nt) {
    case 1: k_recip_sk_tc<1><<<grid, 32 * TC_WARPS, smem, s>>>(tab, c->na, kmax, c->ncol, c->kcol, c->nkp, nchunk, part); break;
    case 2: k_recip_sk_tc<2><<<grid, 32 * TC_WARPS, smem, s>>>(tab, c->na, kmax, c->ncol, c->kcol, c->nkp, nchunk, part); break;
    case 3: k_recip_sk_tc<3><<<grid, 32 * TC_WARPS, smem, s>>>(tab, c->na, kmax, c->ncol, c->kcol, c->nkp, nchunk, part); break;
    default: k_recip_sk_tc<4><<<grid, 32 * TC_WARPS, smem, s>>>(tab, c->na, kmax, c->ncol, c->kcol, c->nkp, nchunk, part); break;
  }
  return true;
}
