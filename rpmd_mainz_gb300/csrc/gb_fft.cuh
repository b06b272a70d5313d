// gb_fft.cuh -- normal-mode transforms on the device.
//
// realft (fourier.f90:16-63) applies FFTW's r2r R2HC (mode +1) or HC2R
// (mode -1) to each coordinate row of r(3*na, nb) and scales by 1/sqrt(nb).
// R2HC stores Re X_0..Re X_{n/2} followed by Im X_{(n+1)/2-1}..Im X_1 with
// X_k = sum_j x_j exp(-2 pi i j k / n); HC2R is its unnormalised inverse.
//
// For power-of-two lengths the rows are transformed in registers: the n real
// values are packed into n/2 complex values z_j = x_{2j} + i x_{2j+1}, a radix-2
// complex FFT of length n/2 runs fully unrolled, and the even/odd split
// X_k = E_k + w^k O_k (w = exp(-2 pi i / n)) recovers the half-complex output;
// the inverse runs the same steps backwards.  Other lengths use the direct sum.
//
// Twiddles: tw[m] = cos(2 pi m / n), tw[n + m] = sin(2 pi m / n), m < n.
#pragma once

#include "gb_common.cuh"

GB_HD constexpr int gb_bitrev(int i, int h) {
  int r = 0;
  for (int b = 1; b < h; b <<= 1) {
    r = (r << 1) | (i & 1);
    i >>= 1;
  }
  return r;
}

// one radix-2 stage of butterfly span LEN (template recursion keeps every index
// a compile-time constant, so the arrays stay in registers)
template <int H, int N, bool INV, int LEN>
GB_D void gb_cfft_stage(double (&zr)[H], double (&zi)[H], const double *__restrict__ tw) {
  if constexpr (LEN <= H) {
    constexpr int half = LEN / 2;
#pragma unroll
    for (int k = 0; k < half; ++k) {
      double wr = 1.0, wi = 0.0;
      if (k > 0) {
        const int m = k * (N / LEN);
        wr = tw[m];
        wi = INV ? tw[N + m] : -tw[N + m];
      }
#pragma unroll
      for (int i = 0; i < H; i += LEN) {
        const int a = i + k, b = a + half;
        double tr, ti;
        if (k == 0) {
          tr = zr[b];
          ti = zi[b];
        } else {
          tr = zr[b] * wr - zi[b] * wi;
          ti = zr[b] * wi + zi[b] * wr;
        }
        zr[b] = zr[a] - tr;
        zi[b] = zi[a] - ti;
        zr[a] = zr[a] + tr;
        zi[a] = zi[a] + ti;
      }
    }
    gb_cfft_stage<H, N, INV, 2 * LEN>(zr, zi, tw);
  }
}

// in-place radix-2 complex FFT of length H on register arrays; N = table length
// (a multiple of H); INV selects exp(+...) twiddles
template <int H, int N, bool INV>
GB_D void gb_cfft(double (&zr)[H], double (&zi)[H], const double *__restrict__ tw) {
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const int j = gb_bitrev(i, H);
    if (i < j) {
      double t = zr[i]; zr[i] = zr[j]; zr[j] = t;
      t = zi[i]; zi[i] = zi[j]; zi[j] = t;
    }
  }
  gb_cfft_stage<H, N, INV, 2>(zr, zi, tw);
}

// unscaled R2HC of length N (power of two) in registers
template <int N>
GB_D void gb_r2hc(const double (&x)[N], double (&out)[N], const double *__restrict__ tw) {
  if constexpr (N == 1) {
    out[0] = x[0];
  } else {
    constexpr int H = N / 2;
    double zr[H], zi[H];
#pragma unroll
    for (int j = 0; j < H; ++j) {
      zr[j] = x[2 * j];
      zi[j] = x[2 * j + 1];
    }
    if constexpr (H > 1) gb_cfft<H, N, false>(zr, zi, tw);
    out[0] = zr[0] + zi[0];
    out[H] = zr[0] - zi[0];
#pragma unroll
    for (int k = 1; k < H; ++k) {
      const int b = H - k;
      const double er = 0.5 * (zr[k] + zr[b]), ei = 0.5 * (zi[k] - zi[b]);
      const double orr = 0.5 * (zi[k] + zi[b]), oi = -0.5 * (zr[k] - zr[b]);
      const double c = tw[k], s = tw[N + k];
      out[k] = er + c * orr + s * oi;
      out[N - k] = ei + c * oi - s * orr;
    }
  }
}

// unscaled HC2R of length N (power of two) in registers
template <int N>
GB_D void gb_hc2r(const double (&in)[N], double (&x)[N], const double *__restrict__ tw) {
  if constexpr (N == 1) {
    x[0] = in[0];
  } else {
    constexpr int H = N / 2;
    double zr[H], zi[H];
    zr[0] = 0.5 * (in[0] + in[H]);
    zi[0] = 0.5 * (in[0] - in[H]);
#pragma unroll
    for (int k = 1; k < H; ++k) {
      const double xr = in[k], xi = in[N - k];
      const double cr = in[H - k], ci = -in[H + k];  // conj(X_{H-k})
      const double er = 0.5 * (xr + cr), ei = 0.5 * (xi + ci);
      const double dr = xr - cr, di = xi - ci;
      const double c = tw[k], s = tw[N + k];
      const double orr = 0.5 * (c * dr - s * di), oi = 0.5 * (c * di + s * dr);
      zr[k] = er - oi;
      zi[k] = ei + orr;
    }
    if constexpr (H > 1) gb_cfft<H, N, true>(zr, zi, tw);
#pragma unroll
    for (int j = 0; j < H; ++j) {
      x[2 * j] = 2.0 * zr[j];
      x[2 * j + 1] = 2.0 * zi[j];
    }
  }
}

// direct-sum transforms for any length (unscaled); x and out must not alias
GB_D void gb_r2hc_direct(const double *x, double *out, int n, const double *__restrict__ tw) {
  for (int k = 0; k <= n / 2; ++k) {
    double re = 0.0;
    int m = 0;
    for (int j = 0; j < n; ++j) {
      re += x[j] * tw[m];
      m += k;
      if (m >= n) m -= n;
    }
    out[k] = re;
  }
  for (int k = 1; k <= (n + 1) / 2 - 1; ++k) {
    double im = 0.0;
    int m = 0;
    for (int j = 0; j < n; ++j) {
      im -= x[j] * tw[n + m];
      m += k;
      if (m >= n) m -= n;
    }
    out[n - k] = im;
  }
}

GB_D void gb_hc2r_direct(const double *in, double *x, int n, const double *__restrict__ tw) {
  for (int j = 0; j < n; ++j) {
    double s = in[0];
    int m = 0;
    for (int k = 1; k <= (n - 1) / 2; ++k) {
      m += j;
      if (m >= n) m -= n;
      s += 2.0 * (in[k] * tw[m] - in[n - k] * tw[n + m]);
    }
    if ((n & 1) == 0) s += (j & 1) ? -in[n / 2] : in[n / 2];
    x[j] = s;
  }
}

// Accessor forms of the power-of-two transforms: `in(j)` yields input element
// j, `out(k, v)` receives output element k.  All input elements are read before
// the first output element is written, so input and output may be the same
// storage (in-place in registers) and either may live in shared or global
// memory; with constant indices after unrolling, register arrays stay in
// registers.
template <int N, class In, class Out>
GB_D void gb_r2hc_io(In in, Out out, const double *__restrict__ tw) {
  if constexpr (N == 1) {
    out(0, in(0));
  } else {
    constexpr int H = N / 2;
    double zr[H], zi[H];
#pragma unroll
    for (int j = 0; j < H; ++j) {
      zr[j] = in(2 * j);
      zi[j] = in(2 * j + 1);
    }
    if constexpr (H > 1) gb_cfft<H, N, false>(zr, zi, tw);
    out(0, zr[0] + zi[0]);
    out(H, zr[0] - zi[0]);
#pragma unroll
    for (int k = 1; k < H; ++k) {
      const int b = H - k;
      const double er = 0.5 * (zr[k] + zr[b]), ei = 0.5 * (zi[k] - zi[b]);
      const double orr = 0.5 * (zi[k] + zi[b]), oi = -0.5 * (zr[k] - zr[b]);
      const double c = tw[k], s = tw[N + k];
      out(k, er + c * orr + s * oi);
      out(N - k, ei + c * oi - s * orr);
    }
  }
}

template <int N, class In, class Out>
GB_D void gb_hc2r_io(In in, Out out, const double *__restrict__ tw) {
  if constexpr (N == 1) {
    out(0, in(0));
  } else {
    constexpr int H = N / 2;
    double zr[H], zi[H];
    {
      const double i0 = in(0), ih = in(H);
      zr[0] = 0.5 * (i0 + ih);
      zi[0] = 0.5 * (i0 - ih);
    }
#pragma unroll
    for (int k = 1; k < H; ++k) {
      const double xr = in(k), xi = in(N - k);
      const double cr = in(H - k), ci = -in(H + k);
      const double er = 0.5 * (xr + cr), ei = 0.5 * (xi + ci);
      const double dr = xr - cr, di = xi - ci;
      const double c = tw[k], s = tw[N + k];
      const double orr = 0.5 * (c * dr - s * di), oi = 0.5 * (c * di + s * dr);
      zr[k] = er - oi;
      zi[k] = ei + orr;
    }
    if constexpr (H > 1) gb_cfft<H, N, true>(zr, zi, tw);
#pragma unroll
    for (int j = 0; j < H; ++j) {
      out(2 * j, 2.0 * zr[j]);
      out(2 * j + 1, 2.0 * zi[j]);
    }
  }
}
