// gb_f2.cuh -- paired FP32 arithmetic of sm_100 and later (FADD2 / FMUL2 /
// FFMA2: two IEEE single-precision operations, each rounded to nearest, in one
// instruction on a register pair).  The mixed pair and k-space kernels are
// issue-bound, so evaluating two independent items per lane through these
// halves the floating-point instructions of their inner loops without
// changing any result: each component is the same correctly rounded operation
// as its scalar form.
#pragma once
#include <cuda_runtime.h>

#include "gb_common.cuh"

GB_D float2 f2(float a, float b) { return make_float2(a, b); }
GB_D float2 f2s(float a) { return make_float2(a, a); }
GB_D float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
GB_D float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
GB_D float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
GB_D float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }

// Kahan-compensated s += v per component, the compensation kept negated
// (s + n is the compensated sum): the same steps as the scalar form
GB_D void kadd2(float2 &s, float2 &n, float2 v) {
  const float2 y = __fadd2_rn(v, n);
  const float2 t = __fadd2_rn(s, y);
  n = __fadd2_rn(__ffma2_rn(t, make_float2(-1.f, -1.f), s), y);  // y - (t - s)
  s = t;
}
