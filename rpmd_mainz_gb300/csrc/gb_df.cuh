// gb_df.cuh -- FP64-free helpers of the mixed-precision kernels.
//
// On GB300 the FP64 pipe issues about 2 lanes per clock per SM, and the
// FP32 <-> FP64 conversion instructions run on it at the same rate (measured:
// DFMA 1.6, cvt.f64.f32 and cvt.f32.f64 1.9 lanes/clk/SM, against 86 for a
// dependent FFMA chain and 37 for cvt.f32.s32).  A per-element FP64 operation
// therefore costs as much as ~50 FP32 ones.  The mixed kernels keep FP64 for
// stored state and totals only and do the per-element work with:
//  * exact FP32 -> FP64 and FP64 -> (hi, lo) FP32 splits built from integer
//    bit operations (no FP64 instruction);
//  * two-float ("df") sums from the error-free TwoSum of Knuth (TAOCP vol. 2,
//    4.2.2) and the FMA-based exact product, about 48 significant bits.
#pragma once

#include "gb_common.cuh"

// exact float -> double for normal floats and zero; FP32 subnormals flush to
// a signed zero, infinities and NaNs stay infinities and NaNs
GB_D double f2d(float f) {
  const unsigned u = __float_as_uint(f);
  const unsigned s = u & 0x80000000u, e = (u >> 23) & 0xffu, m = u & 0x7fffffu;
  const unsigned E = e == 0xffu ? 0x7ffu : e + 896u;  // 1023 - 127
  const unsigned hi = e == 0u ? s : (s | (E << 20) | (m >> 3));
  const unsigned lo = e == 0u ? 0u : (m << 29);
  return __hiloint2double((int)hi, (int)lo);
}

// d = hi + lo to ~2^-47 relative: hi = d truncated to 24 significant bits, lo =
// the remaining 29 bits rounded to FP32 (same sign).  |d| below 2^-126 (FP32
// normal range) splits to a signed zero, beyond the FP32 range (and NaN) to
// an infinity; below 2^-75 lo is zero (its weight leaves the FP32 range).
// Branch-free: the mixed kernels inline it many times.
GB_D void d2df(double d, float &hi, float &lo) {
  const unsigned H = (unsigned)__double2hiint(d), L = (unsigned)__double2loint(d);
  const unsigned s = H & 0x80000000u;
  const int E = (int)((H >> 20) & 0x7ffu);
  const int e = E - 896;  // biased FP32 exponent
  const unsigned mh = ((H & 0xfffffu) << 3) | (L >> 29);
  const bool nrm = (unsigned)(e - 1) < 254u;
  const int es = E - 948;  // biased FP32 exponent of 2^(E-1075), the weight of L's bit 0
  const float w = es > 0 ? __uint_as_float((unsigned)es << 23) : 0.f;
  const float l = __uint_as_float(__float_as_uint(__uint2float_rn(L & 0x1fffffffu) * w) | s);
  hi = __uint_as_float(nrm ? (s | ((unsigned)e << 23) | mh) : (e >= 255 ? (s | 0x7f800000u) : s));
  lo = nrm ? l : 0.f;
}

// d rounded to the nearest FP32 (ties to even, as the conversion instruction
// rounds: differences of FP32 values meet exact ties often, and rounding them
// away from zero drifts) by integer operations; outside the FP32 normal range
// as d2df
GB_D float d2f(double d) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(d);
  const unsigned long long u = b + 0x0fffffffull + ((b >> 29) & 1ull);  // half an FP32 ulp, less one on even
  const unsigned H = (unsigned)(u >> 32), L = (unsigned)u;
  const unsigned s = H & 0x80000000u;
  const int e = (int)((H >> 20) & 0x7ffu) - 896;
  const unsigned mh = ((H & 0xfffffu) << 3) | (L >> 29);
  const bool nrm = (unsigned)(e - 1) < 254u;
  return __uint_as_float(nrm ? (s | ((unsigned)e << 23) | mh) : (e >= 255 ? (s | 0x7f800000u) : s));
}

// s + e = a + b exactly (TwoSum)
GB_D void two_sum(float a, float b, float &s, float &e) {
  s = a + b;
  const float v = s - a;
  e = (a - (s - v)) + (b - v);
}

// (h, l) += b, with the rounding error carried in l (l is not renormalised:
// for sums of many terms; df_norm before use)
GB_D void df_acc(float &h, float &l, float b) {
  float s, e;
  two_sum(h, b, s, e);
  h = s;
  l += e;
}

// (h, l) += (bh, bl), renormalised
GB_D void df_add(float &h, float &l, float bh, float bl) {
  float s, e;
  two_sum(h, bh, s, e);
  e += l + bl;
  h = s + e;
  l = e - (h - s);
}

GB_D void df_norm(float &h, float &l) {
  const float s = h + l;
  l = l - (s - h);
  h = s;
}

// (h, l) * c for an FP32 c, renormalised
GB_D void df_mulf(float &h, float &l, float c) {
  const float p = h * c;
  const float e = fmaf(h, c, -p);
  const float t = fmaf(l, c, e);
  h = p + t;
  l = t - (h - p);
}

// one FP64 addition of two exact conversions
GB_D double df2d(float h, float l) { return f2d(h) + f2d(l); }

// df sum over the 32 lanes of a warp (every lane gets the total)
GB_D void warp_sum_df(float &h, float &l) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float bh = __shfl_xor_sync(0xffffffffu, h, o), bl = __shfl_xor_sync(0xffffffffu, l, o);
    df_add(h, l, bh, bl);
  }
}

GB_D float warp_sum_f32(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Block sums of NV values per thread into acc[dst[k]] (and acc[dst2[k]] when
// dst2[k] >= 0) with FP64 atomics.  Value 0 is a df pair (h0, l0) scaled by
// `s0` (an energy); values 1..NV-1 are FP32 (virial entries), scaled by `sv`.
// Warps reduce in FP32 / df; lane 0 of each warp stores its partials as
// floats; threads 0..NV-1 then add the warps' partials in FP64 (exact
// conversions, one FP64 addition per warp).  `sh` holds 32 * (NV + 1) floats.
// Every thread of the block must call it.
template <int NV>
GB_D void block_sum_df(float h0, float l0, const float (&v)[NV - 1], float *sh, double *acc, const int (&dst)[NV],
                       const int (&dst2)[NV], double s0, double sv) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  warp_sum_df(h0, l0);
  float w[NV - 1];
#pragma unroll
  for (int k = 0; k < NV - 1; ++k) w[k] = warp_sum_f32(v[k]);
  if (lane == 0) {
    float *o = sh + warp * (NV + 1);
    o[0] = h0;
    o[1] = l0;
#pragma unroll
    for (int k = 0; k < NV - 1; ++k) o[2 + k] = w[k];
  }
  __syncthreads();
  const int t = threadIdx.x;
  if (t < NV) {
    double s2 = 0.0;
    for (int q = 0; q < nw; ++q) {
      const float *o = sh + q * (NV + 1);
      s2 += t == 0 ? df2d(o[0], o[1]) : f2d(o[1 + t]);
    }
    s2 *= t == 0 ? s0 : sv;
    int d = dst[0], d2 = dst2[0];
#pragma unroll
    for (int k = 1; k < NV; ++k)
      if (t == k) d = dst[k], d2 = dst2[k];
    if (s2 != 0.0) {
      atomicAdd(acc + d, s2);
      if (d2 >= 0) atomicAdd(acc + d2, s2);
    }
  }
}
