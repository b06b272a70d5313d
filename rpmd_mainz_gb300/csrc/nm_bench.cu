// nm_bench.cu -- the normal-mode transform (realft, fourier.f90:16-63, scaled by
// 1/sqrt(nb)) of many coordinate rows, timed two ways on the device:
//
//  * as the propagator runs it: the lane-pair real FFT in FP32 registers with
//    split (hi + lo) twiddles (gb_r2hc_pair / gb_hc2r_pair, k_mts.cu), two
//    lanes per row;
//  * as a dense product on the tensor cores: a warp takes 16 rows and forms
//    Y = X T_f and X' = Y T_i with mma.sync m16n8k8 TF32 products, the rows
//    split into two TF32 terms and the transform matrices into three (five
//    products per block: hi*hi, hi*mid, lo*hi, hi*lo, lo*mid, so that the
//    matrices hold ~33 bits and the round trip has no fixed gain of the order
//    of one TF32 rounding).  The accumulator layout of one product is used as
//    the operand layout of the next by numbering each 8-column block of the
//    intermediate in the order (0, 2, 4, 6, 1, 3, 5, 7): the rows of both
//    matrices are permuted to match, and no data moves between lanes.
//
// Both kernels run `reps` forward + inverse round trips per row in registers
// (the propagator runs about 12 transforms per row and outer step) between
// one load and one store, so that the times compare the transforms.
// gbrpmd_bench_nm_transform reports the time per transform of each form, the
// relative round-trip error and mean gain per round trip, and the forward
// transform's error against an FP64 direct sum on sample rows.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "gb_common.cuh"
#include "gb_df.cuh"
#include "gb_fft.cuh"

int ctx_set_error(int code, const std::string &msg);
int ctx_check_cuda(cudaError_t e, const char *what);

namespace {

constexpr int NB = 32;
constexpr int M = NB / 2;
constexpr int NBLK = NB / 8;  // 8-column blocks of a 16 x NB tile

#define BCK(x)                                            \
  do {                                                    \
    cudaError_t e_ = (x);                                 \
    if (e_ != cudaSuccess) return ctx_check_cuda(e_, #x); \
  } while (0)

// ---- the in-register lane-pair FFT ----
__global__ void __launch_bounds__(256) k_nm_fft(const float *in, float *out, int nrows, int reps,
                                                const float *tabs /* 12 NB floats */) {
  __shared__ float s_tab[12 * NB];
  for (int i = threadIdx.x; i < 12 * NB; i += blockDim.x) s_tab[i] = tabs[i];
  __syncthreads();
  const float *twm = s_tab, *twm_l = s_tab + 2 * M, *twfm = s_tab + 4 * M, *twfm_l = s_tab + 6 * M;
  const float *twi = s_tab + 8 * M, *twi_l = s_tab + 8 * M + 2 * NB;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int q = (int)(t & 1);
  const long long row = t >> 1;
  const bool valid = row < nrows;
  const long long rr = valid ? row : nrows - 1;
  float x[M];
#pragma unroll
  for (int i = 0; i < M; ++i) x[i] = in[rr * NB + 2 * i + q];
  for (int r = 0; r < reps; ++r) {
    float y[M];
    gb_r2hc_pair<NB, true>(q, [&](int i) { return x[i]; }, [&](int i, float v) { y[i] = v; }, twm, twfm, twi, twm_l,
                           twfm_l, twi_l);
    gb_hc2r_pair<NB, true>(q, [&](int i) { return y[i]; }, [&](int i, float v) { x[i] = v; }, twm, twi, twm_l, twi_l);
  }
  if (valid) {
#pragma unroll
    for (int i = 0; i < M; ++i) out[row * NB + 2 * i + q] = x[i];
  }
}

// forward only, for the accuracy check: out[row][h] in R2HC order
__global__ void k_nm_fft_fwd(const float *in, float *out, int nrows, const float *tabs) {
  __shared__ float s_tab[12 * NB];
  for (int i = threadIdx.x; i < 12 * NB; i += blockDim.x) s_tab[i] = tabs[i];
  __syncthreads();
  const float *twm = s_tab, *twm_l = s_tab + 2 * M, *twfm = s_tab + 4 * M, *twfm_l = s_tab + 6 * M;
  const float *twi = s_tab + 8 * M, *twi_l = s_tab + 8 * M + 2 * NB;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int q = (int)(t & 1);
  const long long row = t >> 1;
  const bool valid = row < nrows;
  const long long rr = valid ? row : nrows - 1;
  float x[M];
#pragma unroll
  for (int i = 0; i < M; ++i) x[i] = in[rr * NB + 2 * i + q];
  gb_r2hc_pair<NB, true>(q, [&](int i) { return x[i]; },
                         [&](int i, float v) {
                           if (valid) out[row * NB + q * M + i] = v;
                         },
                         twm, twfm, twi, twm_l, twfm_l, twi_l);
}

// ---- the in-register lane-quad FFT (four lanes per row, nb = 32) ----
// tabs4: tw8, tw8_l, twf8, twf8_l (16 each), twi, twi_l (64 each)
__global__ void __launch_bounds__(256) k_nm_fft4(const float *in, float *out, int nrows, int reps,
                                                 const float *tabs4, int fwd_only) {
  __shared__ float s_tab[4 * 16 + 2 * 64];
  for (int i = threadIdx.x; i < 4 * 16 + 2 * 64; i += blockDim.x) s_tab[i] = tabs4[i];
  __syncthreads();
  const float *tw8 = s_tab, *tw8_l = s_tab + 16, *twf8 = s_tab + 32, *twf8_l = s_tab + 48;
  const float *twi = s_tab + 64, *twi_l = s_tab + 128;
  const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const int q = (int)(t & 3);
  const long long row = t >> 2;
  const bool valid = row < nrows;
  const long long rr = valid ? row : nrows - 1;
  float x[8];
#pragma unroll
  for (int i = 0; i < 8; ++i) x[i] = in[rr * NB + 4 * i + q];
  if (fwd_only) {
    gb_r2hc_quad32<true>(q, [&](int i) { return x[i]; },
                         [&](int e, float v) {
                           if (valid) out[row * NB + gb_quad_hc(q, e)] = v;
                         },
                         tw8, twf8, twi, tw8_l, twf8_l, twi_l);
    return;
  }
  for (int r = 0; r < reps; ++r) {
    float y[8];
    gb_r2hc_quad32<true>(q, [&](int i) { return x[i]; }, [&](int e, float v) { y[e] = v; }, tw8, twf8, twi, tw8_l,
                         twf8_l, twi_l);
    gb_hc2r_quad32<true>(q, [&](int e) { return y[e]; }, [&](int i, float v) { x[i] = v; }, tw8, twi, tw8_l, twi_l);
  }
  if (valid) {
#pragma unroll
    for (int i = 0; i < 8; ++i) out[row * NB + 4 * i + q] = x[i];
  }
}

// ---- the tensor-core product ----
GB_D unsigned to_tf32(float x) {
  unsigned r;
  asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(r) : "f"(x));
  return r;
}

GB_D void mma_tf32(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k8.row.col.f32.tf32.tf32.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One transform of a 16-row tile held as operands: in[kb][4] (lane (g, t):
// rows g, g + 8; columns 8 kb + 2t, 8 kb + 2t + 1 as regs (0, 2), (1, 3)) ->
// out[nb][4] in the accumulator layout (rows g, g + 8; columns 8 nb + 2t,
// 8 nb + 2t + 1), which is again the operand layout of the next product.
// B: fragments [split][kb][nb][lane] as uint2, splits hi, mid, lo.
GB_D void tile_transform(const float (&in)[NBLK][4], float (&out)[NBLK][4], const uint2 *B, int lane) {
  unsigned ah[NBLK][4], al[NBLK][4];
#pragma unroll
  for (int kb = 0; kb < NBLK; ++kb)
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      // the operand register order (a0..a3) = (row g, row g+8) x (col pair first, second)
      const float v = in[kb][e == 0 ? 0 : e == 1 ? 2 : e == 2 ? 1 : 3];
      ah[kb][e] = to_tf32(v);
      al[kb][e] = to_tf32(v - __uint_as_float(ah[kb][e]));
    }
  constexpr int SP = NBLK * NBLK * 32;  // uint2 per split
#pragma unroll
  for (int nb = 0; nb < NBLK; ++nb) {
    float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll
    for (int kb = 0; kb < NBLK; ++kb) {
      const int f = (kb * NBLK + nb) * 32 + lane;
      const uint2 bh = B[f], bm = B[SP + f], bl = B[2 * SP + f];
      mma_tf32(acc, al[kb], bm.x, bm.y);
      mma_tf32(acc, ah[kb], bl.x, bl.y);
      mma_tf32(acc, al[kb], bh.x, bh.y);
      mma_tf32(acc, ah[kb], bm.x, bm.y);
      mma_tf32(acc, ah[kb], bh.x, bh.y);
    }
    // accumulator (c0, c1, c2, c3) = (row g: cols 2t, 2t+1; row g+8: cols 2t, 2t+1)
    // -> the in[] order used above: [0] (g, 2t), [1] (g, 2t+1), [2] (g+8, 2t), [3] (g+8, 2t+1)
#pragma unroll
    for (int e = 0; e < 4; ++e) out[nb][e] = acc[e];
  }
}

__global__ void __launch_bounds__(256) k_nm_mma(const float *in, float *out, int nrows, int reps, const uint2 *frags,
                                                int fwd_only) {
  extern __shared__ uint2 s_fr[];  // [2 transforms][3 splits][NBLK][NBLK][32]
  constexpr int PER = 3 * NBLK * NBLK * 32;
  for (int i = threadIdx.x; i < 2 * PER; i += blockDim.x) s_fr[i] = frags[i];
  __syncthreads();
  const int lane = threadIdx.x & 31, g = lane >> 2, tq = lane & 3;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarp = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long ntile = (nrows + 15) / 16;
  for (long long tile = warp; tile < ntile; tile += nwarp) {
    const long long r0 = tile * 16 + g, r1 = r0 + 8;
    const long long l0 = r0 < nrows ? r0 : nrows - 1, l1 = r1 < nrows ? r1 : nrows - 1;
    float x[NBLK][4], y[NBLK][4];
#pragma unroll
    for (int kb = 0; kb < NBLK; ++kb) {
      const float2 u = *reinterpret_cast<const float2 *>(in + l0 * NB + 8 * kb + 2 * tq);
      const float2 w = *reinterpret_cast<const float2 *>(in + l1 * NB + 8 * kb + 2 * tq);
      x[kb][0] = u.x, x[kb][1] = u.y, x[kb][2] = w.x, x[kb][3] = w.y;
    }
    if (fwd_only) {
      tile_transform(x, y, s_fr, lane);
#pragma unroll
      for (int nb = 0; nb < NBLK; ++nb) {
        if (r0 < nrows) *reinterpret_cast<float2 *>(out + r0 * NB + 8 * nb + 2 * tq) = make_float2(y[nb][0], y[nb][1]);
        if (r1 < nrows) *reinterpret_cast<float2 *>(out + r1 * NB + 8 * nb + 2 * tq) = make_float2(y[nb][2], y[nb][3]);
      }
      continue;
    }
    for (int r = 0; r < reps; ++r) {
      tile_transform(x, y, s_fr, lane);
      tile_transform(y, x, s_fr + PER, lane);
    }
#pragma unroll
    for (int kb = 0; kb < NBLK; ++kb) {
      if (r0 < nrows) *reinterpret_cast<float2 *>(out + r0 * NB + 8 * kb + 2 * tq) = make_float2(x[kb][0], x[kb][1]);
      if (r1 < nrows) *reinterpret_cast<float2 *>(out + r1 * NB + 8 * kb + 2 * tq) = make_float2(x[kb][2], x[kb][3]);
    }
  }
}

// TF32 rounding of the host (to nearest, ties away: cvt.rna), for the splits
float tf32_host(float x) {
  uint32_t u;
  std::memcpy(&u, &x, 4);
  if ((u & 0x7f800000u) != 0x7f800000u) u = (u + 0x1000u) & 0xffffe000u;
  float r;
  std::memcpy(&r, &u, 4);
  return r;
}

// the 8-column block order of the intermediate: slot a of a block holds
// column pi(a) (the accumulator's (2t, 2t + 1) read as the operand's (t, t + 4))
int perm(int a) { return a < 4 ? 2 * a : 2 * (a - 4) + 1; }

}  // namespace

extern "C" int gbrpmd_bench_nm_transform(int nrows, int reps, double *out12) {
  if (nrows < 16 || reps < 1 || !out12) return ctx_set_error(GB_E_ARG, "nm transform bench: nrows >= 16, reps >= 1");
  const double PI = 3.141592653589793238462643383279502884;
  const double sc = std::sqrt(1.0 / NB);
  // FFT tables as the propagator's pair kernel holds them
  std::vector<float> tabs(12 * NB);
  auto split = [](double v, float &h, float &l) {
    h = (float)v;
    l = (float)(v - (double)h);
  };
  for (int i = 0; i < M; ++i) {
    float h, l;
    split(std::cos(2.0 * PI * i / M), h, l);
    tabs[i] = h, tabs[2 * M + i] = l, tabs[4 * M + i] = 0.5f * h, tabs[6 * M + i] = 0.5f * l;
    split(std::sin(2.0 * PI * i / M), h, l);
    tabs[M + i] = h, tabs[3 * M + i] = l, tabs[5 * M + i] = 0.5f * h, tabs[7 * M + i] = 0.5f * l;
  }
  for (int i = 0; i < NB; ++i) {
    float h, l;
    split(sc * std::cos(2.0 * PI * i / NB), h, l);
    tabs[8 * M + i] = h, tabs[8 * M + 2 * NB + i] = l;
    split(sc * std::sin(2.0 * PI * i / NB), h, l);
    tabs[8 * M + NB + i] = h, tabs[8 * M + 3 * NB + i] = l;
  }
  // the quad form's tables: length 8 (hi, lo, halves) and length 32 scaled
  std::vector<float> tabs4(4 * 16 + 2 * 64);
  for (int i = 0; i < 8; ++i) {
    float h, l;
    split(std::cos(2.0 * PI * i / 8), h, l);
    tabs4[i] = h, tabs4[16 + i] = l, tabs4[32 + i] = 0.5f * h, tabs4[48 + i] = 0.5f * l;
    split(std::sin(2.0 * PI * i / 8), h, l);
    tabs4[8 + i] = h, tabs4[24 + i] = l, tabs4[40 + i] = 0.5f * h, tabs4[56 + i] = 0.5f * l;
  }
  for (int i = 0; i < NB; ++i) {
    float h, l;
    split(sc * std::cos(2.0 * PI * i / NB), h, l);
    tabs4[64 + i] = h, tabs4[128 + i] = l;
    split(sc * std::sin(2.0 * PI * i / NB), h, l);
    tabs4[64 + NB + i] = h, tabs4[128 + NB + i] = l;
  }
  // dense matrices: Y = X Tf (R2HC order, scaled), X = Y Ti (HC2R, scaled)
  std::vector<double> Tf(NB * NB), Ti(NB * NB);
  for (int j = 0; j < NB; ++j)
    for (int k = 0; k < NB; ++k) {
      Tf[j * NB + k] = k <= NB / 2 ? sc * std::cos(2.0 * PI * j * k / NB) : -sc * std::sin(2.0 * PI * j * (NB - k) / NB);
      double v;
      if (k == 0) v = sc;
      else if (k == NB / 2) v = (j & 1) ? -sc : sc;
      else if (k < NB / 2) v = 2.0 * sc * std::cos(2.0 * PI * j * k / NB);
      else v = -2.0 * sc * std::sin(2.0 * PI * j * (NB - k) / NB);
      Ti[k * NB + j] = v;  // row k (mode), column j (bead)
    }
  // fragments: [transform][split][kb][nb][lane] = (B[8kb + tq][8nb + g], B[8kb + tq + 4][8nb + g]),
  // operand row slot a of block kb = matrix row 8kb + perm(a)
  constexpr int PER = 3 * NBLK * NBLK * 32;
  std::vector<uint32_t> fr(2 * 2 * PER);
  for (int tr = 0; tr < 2; ++tr) {
    const std::vector<double> &T = tr ? Ti : Tf;
    for (int kb = 0; kb < NBLK; ++kb)
      for (int nb = 0; nb < NBLK; ++nb)
        for (int lane = 0; lane < 32; ++lane) {
          const int g = lane >> 2, tq = lane & 3;
          for (int half = 0; half < 2; ++half) {
            const double v = T[(8 * kb + perm(tq + 4 * half)) * NB + 8 * nb + g];
            const float h = tf32_host((float)v);
            const float m = tf32_host((float)(v - (double)h));
            const float l = tf32_host((float)(v - (double)h - (double)m));
            const float sp[3] = {h, m, l};
            for (int s = 0; s < 3; ++s) {
              uint32_t u;
              std::memcpy(&u, &sp[s], 4);
              fr[2 * (tr * PER + (s * NBLK * NBLK + kb * NBLK + nb) * 32 + lane) + half] = u;
            }
          }
        }
  }
  // seeded input rows (bead values of a few bohr with spread)
  const size_t n = (size_t)nrows * NB;
  std::vector<float> hx(n);
  uint64_t st = 0x9e3779b97f4a7c15ull;
  for (size_t i = 0; i < n; ++i) {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    hx[i] = (float)(((double)(st >> 11) / 9007199254740992.0 - 0.5) * 4.0);
  }
  float *dx = nullptr, *dy = nullptr, *dtab = nullptr, *dtab4 = nullptr;
  uint2 *dfr = nullptr;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  int rc = GB_OK;
  auto done = [&]() {
    cudaFree(dx), cudaFree(dy), cudaFree(dtab), cudaFree(dfr), cudaFree(dtab4);
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  };
  auto fail = [&](cudaError_t e, const char *what) {
    done();
    return ctx_check_cuda(e, what);
  };
  cudaError_t e;
  if ((e = cudaMalloc(&dx, n * 4)) || (e = cudaMalloc(&dy, n * 4)) || (e = cudaMalloc(&dtab, tabs.size() * 4)) ||
      (e = cudaMalloc(&dfr, fr.size() * 4)) || (e = cudaMalloc(&dtab4, tabs4.size() * 4)))
    return fail(e, "cudaMalloc (nm bench)");
  if ((e = cudaMemcpy(dx, hx.data(), n * 4, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(dtab, tabs.data(), tabs.size() * 4, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(dfr, fr.data(), fr.size() * 4, cudaMemcpyHostToDevice)) ||
      (e = cudaMemcpy(dtab4, tabs4.data(), tabs4.size() * 4, cudaMemcpyHostToDevice)) || (e = cudaEventCreate(&e0)) ||
      (e = cudaEventCreate(&e1)))
    return fail(e, "set-up (nm bench)");
  const size_t smem = sizeof(uint2) * 2 * PER;
  cudaFuncSetAttribute(k_nm_mma, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  const unsigned gfft = (unsigned)((2LL * nrows + 255) / 256);
  const unsigned gfft4 = (unsigned)((4LL * nrows + 255) / 256);
  const long long ntile = (nrows + 15) / 16;
  const unsigned gmma = (unsigned)std::min<long long>((ntile + 7) / 8, 8LL * nsm);
  std::vector<float> hy(n);
  auto timed = [&](int which, float *ms) -> cudaError_t {
    for (int w = 0; w < 3; ++w) {  // warm-up, then the best of three
      if (which == 0) k_nm_fft<<<gfft, 256>>>(dx, dy, nrows, reps, dtab);
      else if (which == 1) k_nm_mma<<<gmma, 256, smem>>>(dx, dy, nrows, reps, dfr, 0);
      else k_nm_fft4<<<gfft4, 256>>>(dx, dy, nrows, reps, dtab4, 0);
    }
    float best = 1e30f;
    for (int k = 0; k < 3; ++k) {
      cudaEventRecord(e0);
      if (which == 0) k_nm_fft<<<gfft, 256>>>(dx, dy, nrows, reps, dtab);
      else if (which == 1) k_nm_mma<<<gmma, 256, smem>>>(dx, dy, nrows, reps, dfr, 0);
      else k_nm_fft4<<<gfft4, 256>>>(dx, dy, nrows, reps, dtab4, 0);
      cudaEventRecord(e1);
      cudaError_t q = cudaEventSynchronize(e1);
      if (q != cudaSuccess) return q;
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      best = std::min(best, t);
    }
    *ms = best;
    return cudaGetLastError();
  };
  // round-trip error and mean gain per round trip: x' = g x + noise
  auto trip = [&](double *err, double *gain) -> cudaError_t {
    cudaError_t q = cudaMemcpy(hy.data(), dy, n * 4, cudaMemcpyDeviceToHost);
    double dd = 0.0, xx = 0.0, xy = 0.0;
    for (size_t i = 0; i < n; ++i) {
      const double a = hx[i], b = hy[i];
      dd += (b - a) * (b - a);
      xx += a * a;
      xy += a * b;
    }
    *err = std::sqrt(dd / xx);
    *gain = std::pow(xy / xx, 1.0 / reps) - 1.0;
    return q;
  };
  // forward transform against the FP64 direct sum on the first rows
  auto fwd_err = [&]() -> double {
    cudaMemcpy(hy.data(), dy, n * 4, cudaMemcpyDeviceToHost);
    double dd = 0.0, yy = 0.0;
    const int rows = std::min(nrows, 512);
    for (int r = 0; r < rows; ++r)
      for (int k = 0; k < NB; ++k) {
        double v = 0.0;
        for (int j = 0; j < NB; ++j) v += (double)hx[(size_t)r * NB + j] * Tf[j * NB + k];
        const double d = hy[(size_t)r * NB + k] - v;
        dd += d * d;
        yy += v * v;
      }
    return std::sqrt(dd / yy);
  };
  float ms_fft = 0.f, ms_mma = 0.f;
  double err_fft, gain_fft, err_mma, gain_mma;
  if ((e = timed(0, &ms_fft)) || (e = trip(&err_fft, &gain_fft))) return fail(e, "FFT transforms (nm bench)");
  k_nm_fft_fwd<<<gfft, 256>>>(dx, dy, nrows, dtab);
  if ((e = cudaDeviceSynchronize())) return fail(e, "FFT forward (nm bench)");
  const double ferr_fft = fwd_err();
  if ((e = timed(1, &ms_mma)) || (e = trip(&err_mma, &gain_mma))) return fail(e, "tensor-core transforms (nm bench)");
  k_nm_mma<<<gmma, 256, smem>>>(dx, dy, nrows, 1, dfr, 1);
  if ((e = cudaDeviceSynchronize())) return fail(e, "tensor-core forward (nm bench)");
  const double ferr_mma = fwd_err();
  float ms_q = 0.f;
  double err_q, gain_q;
  if ((e = timed(2, &ms_q)) || (e = trip(&err_q, &gain_q))) return fail(e, "lane-quad transforms (nm bench)");
  k_nm_fft4<<<gfft4, 256>>>(dx, dy, nrows, 1, dtab4, 1);
  if ((e = cudaDeviceSynchronize())) return fail(e, "lane-quad forward (nm bench)");
  const double ferr_q = fwd_err();
  // per transform (2 reps transforms per row)
  out12[0] = ms_fft / (2.0 * reps);
  out12[1] = ms_mma / (2.0 * reps);
  out12[2] = err_fft;
  out12[3] = gain_fft;
  out12[4] = err_mma;
  out12[5] = gain_mma;
  out12[6] = ferr_fft;
  out12[7] = ferr_mma;
  out12[8] = ms_q / (2.0 * reps);
  out12[9] = err_q;
  out12[10] = gain_q;
  out12[11] = ferr_q;
  done();
  return rc;
}
