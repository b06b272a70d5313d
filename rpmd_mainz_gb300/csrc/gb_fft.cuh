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

GB_D float gb_fma(float a, float b, float c) { return fmaf(a, b, c); }
GB_D double gb_fma(double a, double b, double c) { return fma(a, b, c); }

// Table products.  With SPLIT each table value is the pair hi + lo (hi the
// value rounded to R, lo the rounding remainder), and a product v * x is formed
// as fma(hi, x, lo * x): the table then carries ~2x the precision of R, so a
// forward and an inverse transform compose to the identity up to the rounding
// of the data alone (which is unbiased), instead of up to a fixed error of the
// rounded twiddles that repeats in every round trip.
template <bool SPLIT, typename R>
GB_D R gb_tmul(const R *__restrict__ hi, const R *__restrict__ lo, int i, R x) {
  if constexpr (SPLIT) return gb_fma(hi[i], x, lo[i] * x);
  else return hi[i] * x;
}

// one radix-2 stage of butterfly span LEN (template recursion keeps every index
// a compile-time constant, so the arrays stay in registers)
template <int H, int N, bool INV, int LEN, typename R, bool SPLIT>
GB_D void gb_cfft_stage(R (&zr)[H], R (&zi)[H], const R *__restrict__ tw, const R *__restrict__ twl) {
  if constexpr (LEN <= H) {
    constexpr int half = LEN / 2;
#pragma unroll
    for (int k = 0; k < half; ++k) {
      const int m = k * (N / LEN);
      R wr = (R)1, wi = (R)0, wrl = (R)0, wil = (R)0;
      if (k > 0 && 4 * m != N) {
        wr = tw[m];
        wi = INV ? tw[N + m] : -tw[N + m];
        if constexpr (SPLIT) {
          wrl = twl[m];
          wil = INV ? twl[N + m] : -twl[N + m];
        }
      }
#pragma unroll
      for (int i = 0; i < H; i += LEN) {
        const int a = i + k, b = a + half;
        R tr, ti;
        if (k == 0) {
          tr = zr[b];
          ti = zi[b];
        } else if (4 * m == N) {  // w = -i (forward) or +i (inverse): no multiplication
          tr = INV ? -zi[b] : zi[b];
          ti = INV ? zr[b] : -zr[b];
        } else if constexpr (SPLIT) {
          tr = gb_fma(zr[b], wr, gb_fma(-zi[b], wi, zr[b] * wrl - zi[b] * wil));
          ti = gb_fma(zr[b], wi, gb_fma(zi[b], wr, zr[b] * wil + zi[b] * wrl));
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
    gb_cfft_stage<H, N, INV, 2 * LEN, R, SPLIT>(zr, zi, tw, twl);
  }
}

// in-place radix-2 complex FFT of length H on register arrays; N = table length
// (a multiple of H); INV selects exp(+...) twiddles; twl: the lo parts (SPLIT)
template <int H, int N, bool INV, typename R, bool SPLIT = false>
GB_D void gb_cfft(R (&zr)[H], R (&zi)[H], const R *__restrict__ tw, const R *__restrict__ twl = nullptr) {
#pragma unroll
  for (int i = 0; i < H; ++i) {
    const int j = gb_bitrev(i, H);
    if (i < j) {
      R t = zr[i]; zr[i] = zr[j]; zr[j] = t;
      t = zi[i]; zi[i] = zi[j]; zi[j] = t;
    }
  }
  gb_cfft_stage<H, N, INV, 2, R, SPLIT>(zr, zi, tw, twl);
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
    if constexpr (H > 1) gb_cfft<H, N, false, double>(zr, zi, tw);
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
    if constexpr (H > 1) gb_cfft<H, N, true, double>(zr, zi, tw);
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

// Scaled accessor forms of the power-of-two transforms, as the propagator uses
// them: `in(j)` yields input element j, `out(k, v)` receives output element k
// already multiplied by the scale sc.  All inputs are read before the first
// output is written, so input and output may share storage; with constant
// indices after unrolling, register arrays stay in registers.
//
// The half-complex split treats k and H - k together (their twiddles are
// (c, s) and (-c, s)), which halves its arithmetic; the scale is folded into
// pre-scaled twiddle tables:
//   twf[m] = (sc / 2) cos(2 pi m / n), twf[n + m] = (sc / 2) sin(...)  (forward)
//   twi[m] = sc cos(2 pi m / n),       twi[n + m] = sc sin(...)        (inverse)
// tw is the unscaled table of the complex FFT.  SPLIT: tw_l / twf_l / twi_l
// hold the lo parts of the three tables (gb_tmul).
template <int N, typename R = double, bool SPLIT = false, class In, class Out>
GB_D void gb_r2hc_s(In in, Out out, const R *__restrict__ tw, const R *__restrict__ twf,
                    const R *__restrict__ tw_l = nullptr, const R *__restrict__ twf_l = nullptr) {
  // sc = 2 twf[0] (exact doubling of both parts)
  auto scm = [&](R x) { return (R)2 * gb_tmul<SPLIT, R>(twf, twf_l, 0, x); };
  if constexpr (N == 1) {
    out(0, scm(in(0)));
  } else {
    constexpr int H = N / 2;
    R zr[H], zi[H];
#pragma unroll
    for (int j = 0; j < H; ++j) {
      zr[j] = in(2 * j);
      zi[j] = in(2 * j + 1);
    }
    if constexpr (H > 1) gb_cfft<H, N, false, R, SPLIT>(zr, zi, tw, tw_l);
    out(0, scm(zr[0] + zi[0]));
    out(H, scm(zr[0] - zi[0]));
#pragma unroll
    for (int k = 1; 2 * k < H; ++k) {
      const int b = H - k;
      const R P = zr[k] + zr[b], Q = zi[k] + zi[b];
      const R Rd = zr[k] - zr[b], D = zi[k] - zi[b];
      const R hP = gb_tmul<SPLIT, R>(twf, twf_l, 0, P), hD = gb_tmul<SPLIT, R>(twf, twf_l, 0, D);
      R T1, T2;
      if constexpr (SPLIT) {
        const R hc = twf[k], hs = twf[N + k], hcl = twf_l[k], hsl = twf_l[N + k];
        T1 = gb_fma(hc, Q, gb_fma(-hs, Rd, hcl * Q - hsl * Rd));
        T2 = gb_fma(hc, Rd, gb_fma(hs, Q, hcl * Rd + hsl * Q));
      } else {
        const R hc = twf[k], hs = twf[N + k];
        T1 = hc * Q - hs * Rd;
        T2 = hc * Rd + hs * Q;
      }
      out(k, hP + T1);
      out(b, hP - T1);
      out(N - k, hD - T2);
      out(N - b, -hD - T2);
    }
    if constexpr (H % 2 == 0) {  // k = H/2 = n/4: cos = 0, sin = 1
      out(H / 2, scm(zr[H / 2]));
      out(N - H / 2, -scm(zi[H / 2]));
    }
  }
}

template <int N, typename R = double, bool SPLIT = false, class In, class Out>
GB_D void gb_hc2r_s(In in, Out out, const R *__restrict__ tw, const R *__restrict__ twi,
                    const R *__restrict__ tw_l = nullptr, const R *__restrict__ twi_l = nullptr) {
  auto scm = [&](R x) { return gb_tmul<SPLIT, R>(twi, twi_l, 0, x); };  // sc = twi[0]
  if constexpr (N == 1) {
    out(0, scm(in(0)));
  } else {
    constexpr int H = N / 2;
    R zr[H], zi[H];
    {
      const R i0 = in(0), ih = in(H);
      zr[0] = scm(i0 + ih);
      zi[0] = scm(i0 - ih);
    }
#pragma unroll
    for (int k = 1; 2 * k < H; ++k) {
      const int b = H - k;
      // X_k = in(k) + i in(N-k), conj(X_{H-k}) = in(H-k) - i in(H+k)
      const R xr = in(k), xi = in(N - k), cr = in(b), ci = -in(H + k);
      const R A = scm(xr + cr), B = scm(xi + ci);
      const R dr = xr - cr, di = xi - ci;
      R U, V;
      if constexpr (SPLIT) {
        const R c = twi[k], s = twi[N + k], cl = twi_l[k], sl = twi_l[N + k];
        U = gb_fma(c, di, gb_fma(s, dr, cl * di + sl * dr));
        V = gb_fma(c, dr, gb_fma(-s, di, cl * dr - sl * di));
      } else {
        const R c = twi[k], s = twi[N + k];
        U = c * di + s * dr;
        V = c * dr - s * di;
      }
      zr[k] = A - U;
      zr[b] = A + U;
      zi[k] = B + V;
      zi[b] = V - B;
    }
    if constexpr (H % 2 == 0) {  // k = H/2: cos = 0, sin = 1
      const R xr = in(H / 2), xi = in(N - H / 2);
      zr[H / 2] = (R)2 * scm(xr);
      zi[H / 2] = (R)-2 * scm(xi);
    }
    if constexpr (H > 1) gb_cfft<H, N, true, R, SPLIT>(zr, zi, tw, tw_l);
#pragma unroll
    for (int j = 0; j < H; ++j) {
      out(2 * j, zr[j]);
      out(2 * j + 1, zi[j]);
    }
  }
}

// Lane-pair forms of the scaled power-of-two transforms, FP32 (N >= 4, M =
// N/2): two adjacent lanes (q = lane & 1) share one coordinate row.  Lane q
// holds the beads j = 2i + q (i < M) and the half-complex elements h = qM + i:
// lane 0 the real parts Re X_0 .. Re X_{M-1}, lane 1 Re X_M followed by the
// imaginary parts Im X_{M-1} .. Im X_1 (element N - k of the R2HC order is
// Im X_k).  Both lanes of a pair must call, with every lane of the warp.
//
// Forward: each lane takes the unscaled M-point R2HC of its beads (E_k from the
// even beads, O_k from the odd ones), the lanes swap them (M shuffles), and
// X_k = sc (E_k + w^k O_k), w = exp(-2 pi i / N), lane 0 forming the real
// parts and lane 1 the imaginary ones.
// Inverse: the lanes swap their elements (M shuffles); lane 0 forms E'_k =
// sc (X_k + conj X_{M-k}) and lane 1 O'_k = sc (X_k - conj X_{M-k}) exp(2 pi i
// k / N), k <= M/2, and each takes the unscaled M-point HC2R of its sequence
// into its beads.
// Tables (R = float): twm / twm_l: cos, sin of 2 pi m / M (hi, lo); twfm /
// twfm_l: half of those (the M-point forward split); twi / twi_l: sc cos, sc
// sin of 2 pi m / N.  SPLIT uses the lo parts (gb_tmul).
template <int N, bool SPLIT, class In, class Out>
GB_D void gb_r2hc_pair(int q, In in, Out out, const float *__restrict__ twm, const float *__restrict__ twfm,
                       const float *__restrict__ twi, const float *__restrict__ twm_l = nullptr,
                       const float *__restrict__ twfm_l = nullptr, const float *__restrict__ twi_l = nullptr) {
  constexpr int M = N / 2;
  float y[M];
  gb_r2hc_s<M, float, SPLIT>(in, [&](int k, float v) { y[k] = v; }, twm, twfm, twm_l, twfm_l);
  float e[M], o[M];
#pragma unroll
  for (int i = 0; i < M; ++i) {
    const float other = __shfl_xor_sync(0xffffffffu, y[i], 1);
    e[i] = q ? other : y[i];
    o[i] = q ? y[i] : other;
  }
  // E_k, O_k for k < M from their half-complex forms (period M, conjugate
  // symmetric); k and M - k are compile-time after unrolling
  auto re = [&](const float(&z)[M], int k) { return k <= M / 2 ? z[k] : z[M - k]; };
  auto im = [&](const float(&z)[M], int k) {
    return (k == 0 || 2 * k == M) ? 0.f : (2 * k < M ? z[M - k] : -z[k]);
  };
#pragma unroll
  for (int i = 0; i < M; ++i) {
    // lane 0: Re X_i = sc Re E_i + sc c_i Re O_i + sc s_i Im O_i
    // lane 1 (i > 0, k = M - i): Im X_k = sc Im E_k + sc c_k Im O_k - sc s_k Re O_k
    // lane 1, i = 0: Re X_M = sc E_0 - sc O_0 (c_M = -1, s_M = 0)
    const int k1 = M - i;
    float A, B, Cc;
    int kt;
    if (i == 0) {
      A = e[0];
      B = o[0];
      Cc = 0.f;
      kt = q ? M : 0;
    } else {
      A = q ? im(e, k1) : re(e, i);
      B = q ? im(o, k1) : re(o, i);
      Cc = q ? -re(o, k1) : im(o, i);
      kt = q ? k1 : i;
    }
    out(i, gb_tmul<SPLIT, float>(twi, twi_l, 0, A) + gb_tmul<SPLIT, float>(twi, twi_l, kt, B) +
               gb_tmul<SPLIT, float>(twi, twi_l, N + kt, Cc));
  }
}

template <int N, bool SPLIT, class In, class Out>
GB_D void gb_hc2r_pair(int q, In in, Out out, const float *__restrict__ twm, const float *__restrict__ twi,
                       const float *__restrict__ twm_l = nullptr, const float *__restrict__ twi_l = nullptr) {
  constexpr int M = N / 2;
  float l0[M], l1[M];  // the elements of lane 0 and of lane 1
#pragma unroll
  for (int i = 0; i < M; ++i) {
    const float mine = in(i);
    const float other = __shfl_xor_sync(0xffffffffu, mine, 1);
    l0[i] = q ? other : mine;
    l1[i] = q ? mine : other;
  }
  auto reX = [&](int k) { return k < M ? l0[k] : l1[0]; };
  auto imX = [&](int k) { return (k == 0 || k == M) ? 0.f : l1[M - k]; };
  float z[M];  // half-complex input of this lane's M-point HC2R
#pragma unroll
  for (int k = 0; 2 * k <= M; ++k) {
    // lane 0: E'_k = sc (X_k + conj X_{M-k}); lane 1: with D = X_k - conj X_{M-k},
    // O'_k = sc D (c_k + i s_k): Re = sc c Dr - sc s Di, Im = sc s Dr + sc c Di
    const float pr = reX(k) + reX(M - k), pi = imX(k) - imX(M - k);
    const float dr = reX(k) - reX(M - k), di = imX(k) + imX(M - k);
    const int kc = q ? k : 0;  // twi[0] = sc
    const float zr = gb_tmul<SPLIT, float>(twi, twi_l, kc, q ? dr : pr) +
                     gb_tmul<SPLIT, float>(twi, twi_l, N + k, q ? -di : 0.f);
    z[k] = zr;
    if (k > 0 && 2 * k < M) {
      const float zi = gb_tmul<SPLIT, float>(twi, twi_l, N + k, q ? dr : 0.f) +
                       gb_tmul<SPLIT, float>(twi, twi_l, kc, q ? di : pi);
      z[M - k] = zi;
    }
  }
  gb_hc2r_s<M, float, SPLIT>([&](int k) { return z[k]; }, out, twm, twm, twm_l, twm_l);
}

// Lane-quad forms for N = 32 (Q = 8 beads per lane), FP32: four adjacent lanes
// (q = lane & 3) share a row.  Lane q holds the beads j = 4i + q (i < 8) and
// eight half-complex elements, gb_quad_hc(q, e): lane p = 1, 2, 3 the complex
// values X_p, X_{8-p}, X_{8+p}, X_{16-p} (each as Re, Im), lane 0 X_0, X_16
// (real), X_8, X_4 and X_12.  Every lane of the warp must call.
//
// Forward: each lane takes the unscaled 8-point R2HC of its beads (Y_q); the
// lanes exchange the values Y_q[r] each needs (three shuffle rounds of two
// values), and lane p forms, with B_q = w^{q p} Y_q[p] (w = exp(-2 pi i / 32)),
// the 4-point DFT F_m = sum_q B_q (-i)^{q m}: X_p = F_0, X_{8+p} = F_1,
// X_{16-p} = conj F_2, X_{8-p} = conj F_3 (X_{r + 8m} = sum_q w^{q r}
// (-i)^{q m} Y_q[r]); lane 0 does the same for r = 0 and r = 4.
// Inverse: lane p forms G_s = sum_m F_m i^{s m} and Z_s[p] = w^{-s p} G_s for
// each lane s, the lanes exchange them back, and lane s takes the unscaled
// 8-point HC2R of Z_s into its beads (x_{4i+s} = sum_r Z_s[r] e^{2 pi i i r/8}).
// Tables (float): tw8 / tw8_l: cos, sin of 2 pi m / 8 (hi, lo); twf8 / twf8_l:
// half of those; twi / twi_l: sc cos, sc sin of 2 pi m / 32 (sc = 1/sqrt(32)).
GB_HD int gb_quad_hc(int q, int e) {
  if (q == 0) {
    const int h0[8] = {0, 16, 8, 24, 4, 28, 12, 20};
    return h0[e];
  }
  const int hp[8] = {q, 32 - q, 8 - q, 24 + q, 8 + q, 24 - q, 16 - q, 16 + q};
  return hp[e];
}

template <bool SPLIT>
GB_D void gb_quad_cmul(const float *twi, const float *twi_l, int m, bool conj, float ar, float ai, float &br,
                       float &bi) {
  // (c -+ i s)(ar + i ai) with c, s = sc cos, sc sin of 2 pi m / 32
  const float cr = gb_tmul<SPLIT, float>(twi, twi_l, m, ar), ci = gb_tmul<SPLIT, float>(twi, twi_l, m, ai);
  const float sr = gb_tmul<SPLIT, float>(twi, twi_l, 32 + m, ar), si = gb_tmul<SPLIT, float>(twi, twi_l, 32 + m, ai);
  br = conj ? cr - si : cr + si;
  bi = conj ? ci + sr : ci - sr;
}

// z * (-i)^s (rot = s & 3): 0: z, 1: (zi, -zr), 2: -z, 3: (-zi, zr)
GB_D void gb_rot_mi(int s, float zr, float zi, float &outr, float &outi) {
  const int k = s & 3;
  outr = k == 0 ? zr : k == 1 ? zi : k == 2 ? -zr : -zi;
  outi = k == 0 ? zi : k == 1 ? -zr : k == 2 ? -zi : zr;
}

template <bool SPLIT, class In, class Out>
GB_D void gb_r2hc_quad32(int q, In in, Out out, const float *__restrict__ tw8, const float *__restrict__ twf8,
                         const float *__restrict__ twi, const float *__restrict__ tw8_l = nullptr,
                         const float *__restrict__ twf8_l = nullptr, const float *__restrict__ twi_l = nullptr) {
  float y[8];
  gb_r2hc_s<8, float, SPLIT>(in, [&](int k, float v) { y[k] = v; }, tw8, twf8, tw8_l, twf8_l);
  // the pair a lane sends to lane d: d = 0: (Y[0], Y[4]); d > 0: (Re Y[d], Im Y[d]) = (y[d], y[8 - d])
  auto pick0 = [&](int d) { return d == 0 ? y[0] : d == 1 ? y[1] : d == 2 ? y[2] : y[3]; };
  auto pick1 = [&](int d) { return d == 0 ? y[4] : d == 1 ? y[7] : d == 2 ? y[6] : y[5]; };
  // F_0..F_3 of the lane's group (r = q; lane 0: r = 0 with real inputs), and
  // lane 0's second group (r = 4): G_0, G_1
  float f0r = 0.f, f0i = 0.f, f1r = 0.f, f1i = 0.f, f2r = 0.f, f2i = 0.f, f3r = 0.f, f3i = 0.f;
  float g0r = 0.f, g0i = 0.f, g1r = 0.f, g1i = 0.f;
#pragma unroll
  for (int x = 0; x < 4; ++x) {
    const int src = q ^ x;
    float ar = pick0(src), ai = pick1(src);
    if (x) {
      ar = __shfl_xor_sync(0xffffffffu, ar, x);
      ai = __shfl_xor_sync(0xffffffffu, ai, x);
    }
    // B = w^{src q} A (lane 0: A = Y_src[0], real)
    float br, bi;
    gb_quad_cmul<SPLIT>(twi, twi_l, (src * q) & 31, false, ar, q ? ai : 0.f, br, bi);
    float tr, ti;
    f0r += br, f0i += bi;
    gb_rot_mi(src, br, bi, tr, ti);  // (-i)^src B
    f1r += tr, f1i += ti;
    gb_rot_mi(2 * src, br, bi, tr, ti);  // (-1)^src B
    f2r += tr, f2i += ti;
    gb_rot_mi(3 * src, br, bi, tr, ti);  // i^src B
    f3r += tr, f3i += ti;
    // lane 0, r = 4: B = w^{4 src} Y_src[4]
    gb_quad_cmul<SPLIT>(twi, twi_l, (4 * src) & 31, false, ai, 0.f, br, bi);
    g0r += br, g0i += bi;
    gb_rot_mi(src, br, bi, tr, ti);
    g1r += tr, g1i += ti;
  }
  if (q) {
    out(0, f0r), out(1, f0i);   // X_p
    out(2, f3r), out(3, -f3i);  // X_{8-p} = conj F_3
    out(4, f1r), out(5, f1i);   // X_{8+p}
    out(6, f2r), out(7, -f2i);  // X_{16-p} = conj F_2
  } else {
    out(0, f0r), out(1, f2r);   // X_0, X_16
    out(2, f1r), out(3, f1i);   // X_8
    out(4, g0r), out(5, g0i);   // X_4
    out(6, g1r), out(7, g1i);   // X_12
  }
}

template <bool SPLIT, class In, class Out>
GB_D void gb_hc2r_quad32(int q, In in, Out out, const float *__restrict__ tw8, const float *__restrict__ twi,
                         const float *__restrict__ tw8_l = nullptr, const float *__restrict__ twi_l = nullptr) {
  float e[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) e[k] = in(k);
  // F_m of the lane's group: general X_{r+8m}; lane 0, r = 0: (X_0, X_8, X_16, conj X_8)
  float f0r, f0i, f1r, f1i, f2r, f2i, f3r, f3i;
  if (q) {
    f0r = e[0], f0i = e[1];
    f1r = e[4], f1i = e[5];
    f2r = e[6], f2i = -e[7];
    f3r = e[2], f3i = -e[3];
  } else {
    f0r = e[0], f0i = 0.f;
    f1r = e[2], f1i = e[3];
    f2r = e[1], f2i = 0.f;
    f3r = e[2], f3i = -e[3];
  }
  // lane 0, r = 4: (X_4, X_12, conj X_12, conj X_4)
  const float h0r = e[4], h0i = e[5], h1r = e[6], h1i = e[7];
  float z[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) z[k] = 0.f;
#pragma unroll
  for (int x = 0; x < 4; ++x) {
    const int s = q ^ x;  // destination lane of this exchange step's values
    // G_s = F_0 + i^s F_1 + (-1)^s F_2 + (-i)^s F_3
    float t1r, t1i, t2r, t2i, t3r, t3i;
    gb_rot_mi(3 * s, f1r, f1i, t1r, t1i);
    gb_rot_mi(2 * s, f2r, f2i, t2r, t2i);
    gb_rot_mi(s, f3r, f3i, t3r, t3i);
    const float gr = f0r + t1r + t2r + t3r, gi = f0i + t1i + t2i + t3i;
    float zr, zi;  // Z_s[q] = w^{-s q} G_s (lane 0: Z_s[0] = sc G_s, real)
    gb_quad_cmul<SPLIT>(twi, twi_l, (s * q) & 31, true, gr, gi, zr, zi);
    // lane 0, r = 4: G'_s = X_4 + i^s X_12 + (-1)^s conj X_12 + (-i)^s conj X_4; Z_s[4] = Re w^{-4s} G'_s
    gb_rot_mi(3 * s, h1r, h1i, t1r, t1i);
    gb_rot_mi(2 * s, h1r, -h1i, t2r, t2i);
    gb_rot_mi(s, h0r, -h0i, t3r, t3i);
    float z4r, z4i;
    gb_quad_cmul<SPLIT>(twi, twi_l, (4 * s) & 31, true, h0r + t1r + t2r + t3r, h0i + t1i + t2i + t3i, z4r, z4i);
    float v0 = q ? zr : zr, v1 = q ? zi : z4r;  // the pair for lane s
    if (x) {
      v0 = __shfl_xor_sync(0xffffffffu, v0, x);
      v1 = __shfl_xor_sync(0xffffffffu, v1, x);
    }
    // from lane src = q ^ x: src > 0: (Re Z_q[src], Im Z_q[src]) -> z[src], z[8 - src];
    // src = 0: (Z_q[0], Z_q[4]) -> z[0], z[4]
    const int src = q ^ x;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (src == k) {
        if (k == 0) {
          z[0] = v0;
          z[4] = v1;
        } else {
          z[k] = v0;
          z[8 - k] = v1;
        }
      }
    }
  }
  gb_hc2r_s<8, float, SPLIT>([&](int k) { return z[k]; }, out, tw8, tw8, tw8_l, tw8_l);
}
