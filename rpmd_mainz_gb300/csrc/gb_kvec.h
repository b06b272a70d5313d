// gb_kvec.h -- reciprocal-space k-vector tables (host side, no heap use).
//
// The half space of k vectors kept by kwald (ewald_cubic.f90:292-520): for
// every kx >= 0 the (kx, ky) columns with kx^2 + ky^2 (times (2 pi)^2) within
// rkmax^2, each holding kz = -kzm..kzm (kx = ky = 0: kz = 1..kz0).  Loop exits
// follow the reference's tests and rounding.
//
// The device kernels pair kz with -kz: S(kx, ky, +-m) = P +- i Q with
// P = sum q e^{i(kx x + ky y)} cos(2 pi m z), Q = ... sin(2 pi m z), so one
// "k pair" (kx, ky, m) stands for one or two k vectors:
//   kind 0: m = 0 (one vector), kind 1: m > 0 with both signs, kind 2: the
//   kx = ky = 0 column, m > 0 with +m only.
// Tables built here:
//   KCol  per column: kx, ky, first k pair, m range, and kx, ky as doubles;
//   kp    per k pair: kx, ky, m, kind;  kw per k pair: (4 pi / k^2) e^{-k^2 b};
//   grp   structure-factor work items: up to G consecutive m of one column,
//         ordered by first m, then by decreasing length (gb_order_groups).
#pragma once

#include <cuda_runtime.h>

#include <cmath>

#include "../../include/gbrpmd.h"

struct alignas(16) KCol {
  int kx, ky, koff, mm;  // mm = m_lo | (m_hi << 16)
  double dkx, dky;
};
static_assert(sizeof(KCol) == 32, "KCol layout");

// Stable order of the work items by first m, then by decreasing length: the
// threads of a warp then read the same z powers of a site (shared-memory
// broadcasts) and run loops of the same length.  Insertion sort (no heap).
inline void gb_order_groups(int4 *grp, int n) {
  auto before = [](const int4 &a, const int4 &b) {
    return a.z != b.z ? a.z < b.z : (a.x >> 16) > (b.x >> 16);
  };
  for (int i = 1; i < n; ++i) {
    const int4 v = grp[i];
    int j = i;
    while (j > 0 && before(v, grp[j - 1])) {
      grp[j] = grp[j - 1];
      --j;
    }
    grp[j] = v;
  }
}

struct KTables {
  int ncol = 0, nkp = 0, ngrp = 0, nk = 0;  // nk: k vectors (both kz signs counted)
};

// Fills the caller's arrays (capacities cap_*); returns 0, or 1 when a
// capacity is exceeded.  G: maximum m values per structure-factor work item.
inline int gb_build_ktables(const gb_params &P, int G, KCol *col, int cap_col, int4 *kp, double *kw,
                            int cap_kp, int4 *grp, int cap_grp, KTables *out) {
  const double PI = 3.141592653589793238462643383279502884;
  const int kmax = P.kmax;
  const double rlat = 2.0 * PI;
  const double rkmax2 = P.rkmax * P.rkmax;
  const double b = 0.25 / (P.walpha * P.walpha);
  KTables t;
  auto add_col = [&](int kx, int ky, int mlo, int mhi) -> bool {
    if (t.ncol >= cap_col || t.nkp + (mhi - mlo + 1) > cap_kp) return false;
    KCol &c = col[t.ncol++];
    c.kx = kx;
    c.ky = ky;
    c.koff = t.nkp;
    c.mm = mlo | (mhi << 16);
    c.dkx = (double)kx;
    c.dky = (double)ky;
    for (int m = mlo; m <= mhi; ++m) {
      const int kind = (kx == 0 && ky == 0) ? 2 : (m == 0 ? 0 : 1);
      kp[t.nkp] = make_int4(kx, ky, m, kind);
      const double rkx = rlat * kx, rky = rlat * ky, rkz = rlat * m;
      const double rk2 = rkx * rkx + rky * rky + rkz * rkz;
      kw[t.nkp] = (2.0 * rlat / rk2) * std::exp(-b * rk2);  // 4 pi: k and -k
      ++t.nkp;
      t.nk += kind == 1 ? 2 : 1;
    }
    return true;
  };
  for (int kx = 0; kx <= kmax; ++kx) {
    const double rkx = rlat * kx;
    int kz0 = 0;  // ky = 0: kz = 1.. while rkx^2 + rkz^2 <= rkmax2
    for (int kz = 1; kz <= kmax; ++kz) {
      const double rkz = rlat * kz;
      if (rkx * rkx + rkz * rkz > rkmax2) break;
      kz0 = kz;
    }
    if (kx > 0) {
      if (!add_col(kx, 0, 0, kz0)) return 1;
    } else if (kz0 > 0) {
      if (!add_col(0, 0, 1, kz0)) return 1;
    }
    for (int ky = 1; ky <= kmax; ++ky) {
      const double rky = rlat * ky;
      if (rkx * rkx + rky * rky > rkmax2) break;
      int kzm = 0;
      for (int kz = 1; kz <= kmax; ++kz) {
        const double rkz = rlat * kz;
        if (rkx * rkx + rky * rky + rkz * rkz > rkmax2) break;
        kzm = kz;
      }
      if (!add_col(kx, ky, 0, kzm)) return 1;
      if (kx > 0 && !add_col(kx, -ky, 0, kzm)) return 1;
    }
  }
  // work items: full runs of G first, then the remainders by decreasing length
  auto add_grp = [&](const KCol &c, int m0, int len) -> bool {
    if (t.ngrp >= cap_grp) return false;
    grp[t.ngrp++] = make_int4(c.kx | (len << 16), c.ky, m0, c.koff + (m0 - (c.mm & 0xffff)));
    return true;
  };
  for (int i = 0; i < t.ncol; ++i) {
    const int mlo = col[i].mm & 0xffff, mhi = col[i].mm >> 16;
    for (int m0 = mlo; m0 + G - 1 <= mhi; m0 += G)
      if (!add_grp(col[i], m0, G)) return 1;
  }
  for (int len = G - 1; len >= 1; --len) {
    for (int i = 0; i < t.ncol; ++i) {
      const int mlo = col[i].mm & 0xffff, mhi = col[i].mm >> 16;
      const int n = mhi - mlo + 1;
      if (n % G == len && !add_grp(col[i], mlo + (n / G) * G, len)) return 1;
    }
  }
  gb_order_groups(grp, t.ngrp);
  *out = t;
  return 0;
}

// The half space of the non-cubic sum (kwald_nc, ewald_noncubic.f90:275-460):
// every k with kx = 0..kmax, |ky|, |kz| <= kmax and 0 < |k|^2 < rkmax^2, where
// k = 2 pi (kx / Lx, ky / Ly, kz / Lz) in bohr^-1 (products and sums rounded
// as the reference rounds them).  The reference walks kx = 0 with both signs
// of ky, kz and half the weight; its (0, -ky, -kz) halves are the mirror images
// of the kept (0, ky, kz), so the same column / pair / work-item tables as the
// cubic sum hold, with weights (4 pi / V) / k^2 exp(-k^2 / (4 alpha^2)).
inline int gb_build_ktables_nc(const gb_params &P, const double box[3], int G, KCol *col, int cap_col, int4 *kp,
                               double *kw, int cap_kp, int4 *grp, int cap_grp, KTables *out) {
  const double PI = 3.141592653589793238462643383279502884;
  const int kmax = P.kmax;
  const double twopi = 2.0 * PI;
  const double xlat = twopi / box[0], ylat = twopi / box[1], zlat = twopi / box[2];
  const double rkmax2 = P.rkmax * P.rkmax;
  const double b = 0.25 / (P.walpha * P.walpha);
  const double f2 = 2.0 * (twopi / (box[0] * box[1] * box[2]));  // 4 pi / V
  KTables t;
  auto rk2_of = [&](int kx, int ky, int kz) {
    const double rkx = xlat * kx, rky = ylat * ky, rkz = zlat * kz;
    return rkx * rkx + rky * rky + rkz * rkz;
  };
  auto add_col = [&](int kx, int ky, int mlo, int mhi) -> bool {
    if (t.ncol >= cap_col || t.nkp + (mhi - mlo + 1) > cap_kp) return false;
    KCol &c = col[t.ncol++];
    c.kx = kx;
    c.ky = ky;
    c.koff = t.nkp;
    c.mm = mlo | (mhi << 16);
    c.dkx = (double)kx;
    c.dky = (double)ky;
    for (int m = mlo; m <= mhi; ++m) {
      const int kind = (kx == 0 && ky == 0) ? 2 : (m == 0 ? 0 : 1);
      kp[t.nkp] = make_int4(kx, ky, m, kind);
      const double rk2 = rk2_of(kx, ky, m);
      kw[t.nkp] = (f2 / rk2) * std::exp(-b * rk2);
      ++t.nkp;
      t.nk += kind == 1 ? 2 : 1;
    }
    return true;
  };
  // largest kz in 0..kmax with |k|^2 < rkmax^2 at (kx, ky, kz), or -1
  auto kz_top = [&](int kx, int ky) {
    int top = -1;
    for (int kz = 0; kz <= kmax; ++kz) {
      if (!(rk2_of(kx, ky, kz) < rkmax2)) break;
      top = kz;
    }
    return top;
  };
  for (int kx = 0; kx <= kmax; ++kx) {
    const int kz0 = kz_top(kx, 0);
    if (kx > 0) {
      if (kz0 >= 0 && !add_col(kx, 0, 0, kz0)) return 1;
    } else if (kz0 >= 1) {
      if (!add_col(0, 0, 1, kz0)) return 1;
    }
    for (int ky = 1; ky <= kmax; ++ky) {
      const int kzm = kz_top(kx, ky);
      if (kzm < 0) break;
      if (!add_col(kx, ky, 0, kzm)) return 1;
      if (kx > 0 && !add_col(kx, -ky, 0, kzm)) return 1;
    }
  }
  auto add_grp = [&](const KCol &c, int m0, int len) -> bool {
    if (t.ngrp >= cap_grp) return false;
    grp[t.ngrp++] = make_int4(c.kx | (len << 16), c.ky, m0, c.koff + (m0 - (c.mm & 0xffff)));
    return true;
  };
  for (int i = 0; i < t.ncol; ++i) {
    const int mlo = col[i].mm & 0xffff, mhi = col[i].mm >> 16;
    for (int m0 = mlo; m0 + G - 1 <= mhi; m0 += G)
      if (!add_grp(col[i], m0, G)) return 1;
  }
  for (int len = G - 1; len >= 1; --len) {
    for (int i = 0; i < t.ncol; ++i) {
      const int mlo = col[i].mm & 0xffff, mhi = col[i].mm >> 16;
      const int n = mhi - mlo + 1;
      if (n % G == len && !add_grp(col[i], mlo + (n / G) * G, len)) return 1;
    }
  }
  gb_order_groups(grp, t.ngrp);
  *out = t;
  return 0;
}

// capacities that always suffice for a given kmax (both sums)
inline int gb_kcap_col(int kmax) { return (kmax + 1) * (2 * kmax + 1); }
inline int gb_kcap_kp(int kmax) { return gb_kcap_col(kmax) * (kmax + 1); }

// Virial factors per k pair, GB_KVIR doubles: [0..8] multiply the pair's summed
// energy et(+m) + et(-m) (column-major a + 3 b), [9] and [10] multiply the
// difference et(+m) - et(-m) in the xz and yz entries (and their mirrors).
//   cubic (gb_kvir_table): term |rk_a| |rk_b| - delta_ab on the sum, no
//     difference terms -- the reference multiplies the combined (+-ky, +-kz)
//     energy by |k_a| |k_b| (ewald_cubic.f90:488-503); rk = 2 pi (kx, ky, m);
//   non-cubic (gb_kvir_table_nc): term rk_a rk_b - delta_ab per vector
//     (ewald_noncubic.f90:436-453); kz = +-m flips the sign of rk_z, so xz and
//     yz follow the difference, the rest the sum.
// term = 2 (1/rk^2 + 1/(4 alpha^2)).
constexpr int GB_KVIR = 12;

inline void gb_kvir_table(const int4 *kp, int nkp, double walpha, double *out) {
  const double rlat = 2.0 * 3.141592653589793238462643383279502884;
  const double bfac = 0.25 / (walpha * walpha);
  for (int k = 0; k < nkp; ++k) {
    const double rk[3] = {rlat * kp[k].x, rlat * kp[k].y, rlat * kp[k].z};
    const double rk2 = rk[0] * rk[0] + rk[1] * rk[1] + rk[2] * rk[2];
    const double term = 2.0 * (1.0 / rk2 + bfac);
    double *o = out + GB_KVIR * (size_t)k;
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) o[a + 3 * b] = term * std::fabs(rk[a]) * std::fabs(rk[b]) - (a == b ? 1.0 : 0.0);
    o[9] = o[10] = o[11] = 0.0;
  }
}

inline void gb_kvir_table_nc(const int4 *kp, int nkp, double walpha, const double box[3], double *out) {
  const double twopi = 2.0 * 3.141592653589793238462643383279502884;
  const double lat[3] = {twopi / box[0], twopi / box[1], twopi / box[2]};
  const double bfac = 0.25 / (walpha * walpha);
  for (int k = 0; k < nkp; ++k) {
    const double rk[3] = {lat[0] * kp[k].x, lat[1] * kp[k].y, lat[2] * kp[k].z};
    const double rk2 = rk[0] * rk[0] + rk[1] * rk[1] + rk[2] * rk[2];
    const double term = 2.0 * (1.0 / rk2 + bfac);
    double *o = out + GB_KVIR * (size_t)k;
    for (int b = 0; b < 3; ++b)
      for (int a = 0; a < 3; ++a) {
        const bool zodd = (a == 2) != (b == 2);  // xz, yz and mirrors: odd in kz
        o[a + 3 * b] = zodd ? 0.0 : term * rk[a] * rk[b] - (a == b ? 1.0 : 0.0);
      }
    o[9] = term * rk[0] * rk[2];
    o[10] = term * rk[1] * rk[2];
    o[11] = 0.0;
  }
}
