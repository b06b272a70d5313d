// gb_common.cuh -- shared device helpers of the GB300 RPMD library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gb_common.h"

#define GB_HD __host__ __device__ __forceinline__
#define GB_D __device__ __forceinline__

// Fortran NINT: round half away from zero
GB_HD double nint_d(double x) { return round(x); }

// products and sums with no FMA contraction, for quantities whose exact
// rounding decides list membership (cut-off tests must agree with the
// reference's separately rounded dx*dx + dy*dy + dz*dz)
GB_D double dsq3(double dx, double dy, double dz) {
  return __dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz));
}

// non-finite test on the exponent bits (integer instructions: no FP64
// comparison, which runs on the slow FP64 pipe)
GB_D bool gb_nonfinite(double v) { return (__double2hiint(v) & 0x7ff00000) == 0x7ff00000; }
GB_D bool gb_nonfinite(float v) { return (__float_as_uint(v) & 0x7f800000u) == 0x7f800000u; }
// sets ST_NONFINITE in the status word when `bad` (status may be null)
GB_D void gb_flag_nonfinite(unsigned *status, bool bad) {
  if (bad && status) atomicOr(status, ST_NONFINITE);
}

GB_D double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// block-wide sum of `n` doubles per thread into `out` (atomically added);
// `sh` must hold 32*n doubles
template <int NV>
GB_D void block_sum_atomic(double (&v)[NV], double *sh, double *out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) v[i] = warp_sum(v[i]);
  if (lane == 0)
#pragma unroll
    for (int i = 0; i < NV; ++i) sh[warp * NV + i] = v[i];
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int i = 0; i < NV; ++i) {
      double s = lane < nw ? sh[lane * NV + i] : 0.0;
      s = warp_sum(s);
      if (lane == 0 && s != 0.0) atomicAdd(out + i, s);
    }
  }
  __syncthreads();
}

