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

#include "gb_common.cuh"
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

inline unsigned nblk(long long n, int t) { return (unsigned)((n + t - 1) / t); }

}  // namespace

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
