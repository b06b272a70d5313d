// selftest.cu -- device self-check of the integer-built conversions that the
// mixed-precision kernels use in place of FP64 instructions (gb_df.cuh).
// No counterpart in the reference: a caller (the tests) compares the results
// with the IEEE conversions of its own host.
#include <cuda_runtime.h>

#include <string>

#include "gb_df.cuh"

int ctx_set_error(int code, const std::string &msg);
int ctx_check_cuda(cudaError_t e, const char *what);

namespace {

__global__ void k_conv(const double *in, int n, float *f32, float *hi, float *lo, double *back) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double x = in[t];
  const float f = d2f(x);
  float h, l;
  d2df(x, h, l);
  f32[t] = f;
  hi[t] = h;
  lo[t] = l;
  back[t] = f2d(f);
}

}  // namespace

extern "C" int gbrpmd_selftest_conversions(const double *in, int n, float *f32, float *hi, float *lo,
                                           double *back) {
  if (n < 0 || (n > 0 && (!in || !f32 || !hi || !lo || !back))) return ctx_set_error(GB_E_ARG, "bad argument");
  if (n == 0) return GB_OK;
  double *d_in = nullptr, *d_back = nullptr;
  float *d_f = nullptr;
  cudaError_t e = cudaMalloc(&d_in, sizeof(double) * 2 * n);
  if (e == cudaSuccess) e = cudaMalloc(&d_f, sizeof(float) * 3 * n);
  if (e == cudaSuccess) {
    d_back = d_in + n;
    e = cudaMemcpy(d_in, in, sizeof(double) * n, cudaMemcpyHostToDevice);
  }
  if (e == cudaSuccess) {
    k_conv<<<(n + 255) / 256, 256>>>(d_in, n, d_f, d_f + n, d_f + 2 * (size_t)n, d_back);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(f32, d_f, sizeof(float) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(hi, d_f + n, sizeof(float) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(lo, d_f + 2 * (size_t)n, sizeof(float) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(back, d_back, sizeof(double) * n, cudaMemcpyDeviceToHost);
  cudaFree(d_in);
  cudaFree(d_f);
  return e == cudaSuccess ? GB_OK : ctx_check_cuda(e, "conversion self-test");
}
