// orc_setup.cpp -- oracle: random stream, set-up, normal-mode transforms.
// TEST INFRASTRUCTURE ONLY (see orc.h).
#include <cmath>
#include <complex>
#include <cstring>
#include <vector>

#include "orc.h"

namespace orc {

gb_params P;

// ---------------------------------------------------------------------------
// ran2 / gaussian  (random.f90:1-72).  L'Ecuyer two-generator combination with
// a Bays-Durham shuffle table of 32 entries; the state the Fortran keeps in
// SAVE variables lives in Rng.
// ---------------------------------------------------------------------------
void rng_reset(Rng &g) {
  for (int i = 0; i < 32; ++i) g.iv[i] = 0;  // data iv/ntab*0/
  g.iy = 0;                                  // data iy/0/
  g.idum2 = 123456789;                       // data idum2/123456789/
  g.iset = 0;                                // gaussian: data iset/0/
  g.gset = 0.0;
}

double ran2(Rng &g, int &idum, double rmin, double rmax) {
  const int im1 = 2147483563, im2 = 2147483399, imm1 = im1 - 1;
  const int ia1 = 40014, ia2 = 40692, iq1 = 53668, iq2 = 52774, ir1 = 12211, ir2 = 3791;
  const int ntab = 32, ndiv = 1 + imm1 / ntab;
  const double am = 1.0 / im1, eps = 1.2e-7, rnmx = 1.0 - eps;
  int k, j;
  if (idum <= 0) {  // random.f90:49-59
    idum = std::max(-idum, 1);
    g.idum2 = idum;
    for (j = ntab + 8; j >= 1; --j) {
      k = idum / iq1;
      idum = ia1 * (idum - k * iq1) - k * ir1;
      if (idum < 0) idum += im1;
      if (j <= ntab) g.iv[j - 1] = idum;
    }
    g.iy = g.iv[0];
  }
  k = idum / iq1;  // random.f90:60-70
  idum = ia1 * (idum - k * iq1) - k * ir1;
  if (idum < 0) idum += im1;
  k = g.idum2 / iq2;
  g.idum2 = ia2 * (g.idum2 - k * iq2) - k * ir2;
  if (g.idum2 < 0) g.idum2 += im2;
  j = 1 + g.iy / ndiv;
  g.iy = g.iv[j - 1] - g.idum2;
  g.iv[j - 1] = idum;
  if (g.iy < 1) g.iy += imm1;
  return ((rmax - rmin) * (std::min(am * g.iy, rnmx))) + rmin;
}

double gaussian(Rng &g, int &idum, double sigma) {  // random.f90:1-26
  if (g.iset == 0) {
    double v1, v2, rsq;
    do {
      v1 = 2.0 * ran2(g, idum, 0.0, 1.0) - 1.0;
      v2 = 2.0 * ran2(g, idum, 0.0, 1.0) - 1.0;
      rsq = v1 * v1 + v2 * v2;  // v1**2 + v2**2
    } while (rsq >= 1.0 || rsq == 0.0);
    double fac = std::sqrt(-2.0 * std::log(rsq) / rsq);
    g.gset = v1 * fac;
    g.iset = 1;
    return sigma * v2 * fac;
  }
  g.iset = 0;
  return sigma * g.gset;
}

// ---------------------------------------------------------------------------
// setup_box_size for the CUB lattice (setup_options.f90:191-270, nlat = 1)
// ---------------------------------------------------------------------------
int setup_box_size_cub(const int ncell[3], double rho, double wmass, double box[3]) {
  const double emass = 9.1093826e-31, toA = 0.5291772108;  // globals.inc
  int nm = ncell[0] * ncell[1] * ncell[2];
  double vbox = (nm * emass * wmass) / (rho * 1000.0);  // m**3
  vbox = vbox / std::pow(toA * 1e-10, 3);               // bohr**3
  double totcell = (double)(ncell[0] * ncell[1] * ncell[2]);
  double boxl = std::pow(vbox / totcell, 1.0 / 3.0);
  for (int i = 0; i < 3; ++i) box[i] = boxl * ncell[i];
  return nm;
}

// cubic lattice of identically oriented molecules (setup_positions.f90:94-150)
Status cubic(double *r, int nm, const double box[3], const int ncell[3]) {
  const double hx = P.reoh, hy = 0.0, hz = 0.0;
  const double gx = P.reoh * std::cos(P.theta), gy = P.reoh * std::sin(P.theta), gz = 0.0;
  if (ncell[0] * ncell[1] * ncell[2] != nm) return GB_E_ARG;
  double del[3];
  for (int i = 0; i < 3; ++i) del[i] = box[i] / (double)ncell[i];
  int itel = 0;
  double dx = -del[0];
  for (int i = 0; i < ncell[0]; ++i) {
    dx = dx + del[0];
    double dy = -del[1];
    for (int j = 0; j < ncell[1]; ++j) {
      dy = dy + del[1];
      double dz = -del[2];
      for (int k = 0; k < ncell[2]; ++k) {
        dz = dz + del[2];
        if (itel < nm) {
          double *m = r + 9 * itel;
          ++itel;
          m[0] = dx; m[1] = dy; m[2] = dz;
          m[3] = dx + hx; m[4] = dy + hy; m[5] = dz + hz;
          m[6] = dx + gx; m[7] = dy + gy; m[8] = dz + gz;
        }
      }
    }
  }
  return GB_OK;
}

// setup_ewald (setup_options.f90:104-189): writes /ew_setup/ into P.
void setup_ewald(int na, const double box[3]) {
  const double pi = std::acos(-1.0);
  const double cvar = 1.2;
  if (box[0] == box[1] && box[0] == box[2] && P.iamcub) {
    P.iamcub = 1;
    P.wrcut = std::min(0.5, cvar * std::pow((double)na, -1.0 / 6.0));
    if (P.ecut <= 0.0) {
      P.walpha = pi / P.wrcut;
      P.kmax = (int)P.walpha;
      P.rkmax = 2.0 * pi * P.walpha;
    } else {
      double s = std::sqrt(-std::log(P.ecut));
      P.walpha = s / P.wrcut;
      P.kmax = (int)(s * P.walpha / pi);
      P.rkmax = 2.0 * s * P.walpha;
    }
  } else {
    P.iamcub = 0;
    double rshort = std::min(box[0], std::min(box[1], box[2]));
    P.wrcut = rshort * std::min(0.5, cvar * std::pow((double)na, -1.0 / 6.0));
    P.walpha = pi / P.wrcut;
    double rlong = std::max(box[0], std::max(box[1], box[2]));
    P.rkmax = 2.0 * pi * P.walpha;
    P.kmax = (int)(P.walpha * rlong);
  }
}

// ---------------------------------------------------------------------------
// realft (fourier.f90:16-63): per row, FFTW r2r R2HC (mode +1) or HC2R
// (mode -1) of length n, scaled by 1/sqrt(n) in both directions.
//
// FFTW's definitions: R2HC computes X_k = sum_j x_j exp(-2 pi i j k / n) and
// stores r_0..r_{n/2} (real parts) followed by i_{(n+1)/2-1}..i_1 (imaginary
// parts), so out[k] = Re X_k and out[n-k] = Im X_k.  HC2R is the unnormalised
// inverse x_j = sum_k X_k exp(+2 pi i j k / n) with X_{n-k} = conj(X_k).
// ---------------------------------------------------------------------------
namespace {
struct Twiddle {
  int n = 0;
  std::vector<double> c, s;
  void make(int nn) {
    if (n == nn) return;
    n = nn;
    c.resize(n);
    s.resize(n);
    const double two_pi = 2.0 * std::acos(-1.0);
    for (int m = 0; m < n; ++m) {
      c[m] = std::cos(two_pi * m / n);
      s[m] = std::sin(two_pi * m / n);
    }
  }
};

void r2hc_direct(const double *x, double *out, int n, const Twiddle &t) {
  for (int k = 0; k <= n / 2; ++k) {
    double re = 0.0;
    for (int j = 0; j < n; ++j) re += x[j] * t.c[(int)(((long)j * k) % n)];
    out[k] = re;
  }
  for (int k = 1; k <= (n + 1) / 2 - 1; ++k) {
    double im = 0.0;
    for (int j = 0; j < n; ++j) im -= x[j] * t.s[(int)(((long)j * k) % n)];
    out[n - k] = im;
  }
}

void hc2r_direct(const double *in, double *x, int n, const Twiddle &t) {
  for (int j = 0; j < n; ++j) {
    double s = in[0];
    for (int k = 1; k <= (n - 1) / 2; ++k) {
      int m = (int)(((long)j * k) % n);
      s += 2.0 * (in[k] * t.c[m] - in[n - k] * t.s[m]);
    }
    if (n % 2 == 0) s += (j % 2 ? -in[n / 2] : in[n / 2]);
    x[j] = s;
  }
}

using cd = std::complex<double>;

// in-place iterative radix-2 complex FFT of length h (power of two);
// sign = -1 forward (exp(-i...)), +1 backward (unnormalised).  Twiddles
// exp(sign 2 pi i k / h) come from a per-length table.
void cfft(cd *a, int h, int sign) {
  static thread_local int tw_h = 0;
  static thread_local std::vector<cd> tw;
  if (tw_h != h) {
    tw.resize(h);
    const double pi = std::acos(-1.0);
    for (int k = 0; k < h; ++k) tw[k] = cd(std::cos(2.0 * pi * k / h), std::sin(2.0 * pi * k / h));
    tw_h = h;
  }
  for (int i = 1, j = 0; i < h; ++i) {
    int bit = h >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) std::swap(a[i], a[j]);
  }
  for (int len = 2; len <= h; len <<= 1) {
    const int step = h / len;
    for (int i = 0; i < h; i += len) {
      for (int k = 0; k < len / 2; ++k) {
        cd w = tw[k * step];
        if (sign < 0) w = std::conj(w);
        cd u = a[i + k], v = a[i + k + len / 2] * w;
        a[i + k] = u + v;
        a[i + k + len / 2] = u - v;
      }
    }
  }
}

// exp(+2 pi i k / n), k = 0..n/2, cached per length
const std::vector<cd> &post_twiddles(int n) {
  static thread_local int tn = 0;
  static thread_local std::vector<cd> w;
  if (tn != n) {
    w.resize(n / 2 + 1);
    const double pi = std::acos(-1.0);
    for (int k = 0; k <= n / 2; ++k) w[k] = cd(std::cos(2.0 * pi * k / n), std::sin(2.0 * pi * k / n));
    tn = n;
  }
  return w;
}

// R2HC for n = 2h, h a power of two: FFT of the packed sequence
// z_j = x_{2j} + i x_{2j+1}, then X_k = E_k + w^k O_k with
// E_k = (Z_k + conj Z_{h-k})/2, O_k = (Z_k - conj Z_{h-k})/(2i), w = exp(-2 pi i/n).
void r2hc_fft(const double *x, double *out, int n) {
  int h = n / 2;
  std::vector<cd> z(h);
  for (int j = 0; j < h; ++j) z[j] = cd(x[2 * j], x[2 * j + 1]);
  cfft(z.data(), h, -1);
  const std::vector<cd> &wn = post_twiddles(n);
  for (int k = 0; k <= h; ++k) {
    cd zk = z[k % h], zc = std::conj(z[(h - k) % h]);
    cd e = 0.5 * (zk + zc), o = cd(0.0, -0.5) * (zk - zc);
    cd xk = e + std::conj(wn[k]) * o;
    out[k] = xk.real();
    if (k > 0 && k < h) out[n - k] = xk.imag();
  }
}

// HC2R for n = 2h: Z_k = E_k + i O_k with E_k = (X_k + conj X_{h-k})/2,
// O_k = exp(+2 pi i k/n) (X_k - conj X_{h-k})/2; x_{2j} + i x_{2j+1} = 2 IDFT_h(Z).
void hc2r_fft(const double *in, double *x, int n) {
  int h = n / 2;
  auto X = [&](int k) -> cd {
    if (k == 0) return cd(in[0], 0.0);
    if (k == h) return cd(in[h], 0.0);
    return cd(in[k], in[n - k]);
  };
  std::vector<cd> z(h);
  const std::vector<cd> &wn = post_twiddles(n);
  for (int k = 0; k < h; ++k) {
    cd xk = X(k), xc = std::conj(X(h - k));
    cd e = 0.5 * (xk + xc), o = 0.5 * wn[k] * (xk - xc);
    z[k] = e + cd(0.0, 1.0) * o;
  }
  cfft(z.data(), h, +1);
  for (int j = 0; j < h; ++j) {
    x[2 * j] = 2.0 * z[j].real();
    x[2 * j + 1] = 2.0 * z[j].imag();
  }
}

bool pow2(int n) { return n >= 4 && (n & (n - 1)) == 0; }

void realft_impl(double *data, int m, int n, int mode, bool direct) {
  static thread_local Twiddle tw;
  static thread_local std::vector<double> cp, out;
  tw.make(n);
  cp.resize(n);
  out.resize(n);
  const double scale = std::sqrt(1.0 / (double)n);
  const bool fast = !direct && pow2(n);
  for (int k = 0; k < m; ++k) {
    for (int j = 0; j < n; ++j) cp[j] = data[k + (size_t)m * j];
    if (mode == 1) {
      if (fast) r2hc_fft(cp.data(), out.data(), n); else r2hc_direct(cp.data(), out.data(), n, tw);
    } else {
      if (fast) hc2r_fft(cp.data(), out.data(), n); else hc2r_direct(cp.data(), out.data(), n, tw);
    }
    for (int j = 0; j < n; ++j) data[k + (size_t)m * j] = scale * out[j];
  }
}
}  // namespace

void realft(double *data, int m, int n, int mode) { realft_impl(data, m, n, mode, false); }
void realft_direct(double *data, int m, int n, int mode) { realft_impl(data, m, n, mode, true); }

// ring_rpmd (md_pathi.f90:190-231): free ring-polymer monodromy coefficients
// monod(3,4,nb) -> monod[j + 3*(c + 4*k)], atom type j = O,H,H of molecule 1.
void ring_rpmd(const double *mass, double *monod, int na, int nb, double dt, double beta) {
  (void)na;
  const double pi = std::acos(-1.0);
  const double hbar = 1.0;
  auto M = [&](int j, int c, int k) -> double & { return monod[j + 3 * (c + 4 * k)]; };
  for (int j = 0; j < 3; ++j) {
    M(j, 0, 0) = 1.0;
    M(j, 1, 0) = 0.0;
    M(j, 2, 0) = dt / mass[j];
    M(j, 3, 0) = 1.0;
    if (nb > 1) {
      double betan = beta / (double)nb;
      double twown = 2.0 / (betan * hbar);
      double pibyn = pi / (double)nb;
      for (int k = 1; k <= nb / 2; ++k) {
        double wk = twown * std::sin(k * pibyn);
        double wt = wk * dt;
        double wm = wk * mass[j];
        double cwt = std::cos(wt), swt = std::sin(wt);
        M(j, 0, k) = cwt;
        M(j, 1, k) = -wm * swt;
        M(j, 2, k) = swt / wm;
        M(j, 3, k) = cwt;
      }
      for (int k = 1; k <= (nb - 1) / 2; ++k)
        for (int c = 0; c < 4; ++c) M(j, c, nb - k) = M(j, c, k);
    }
  }
}

}  // namespace orc
