// orc_forces.cpp -- oracle: force field of the reference path.
// TEST INFRASTRUCTURE ONLY (see orc.h).
//
// Restates md_forces.f90, ewald_cubic.f90, linked_cell.f90, neigh_list.f90,
// ljones.f90, intra_harmonic.f90, intra_spcfw.f90, intra_morse_harm.f90 and
// correct_tem.f90 with the same loop nesting, linked-cell traversal order and
// accumulation order as the Fortran.
#include <cmath>
#include <cstring>
#include <vector>

#include "orc.h"

namespace orc {

namespace {
const int maxnab = 200;  // globals.inc:25

inline double nint(double x) { return std::round(x); }  // Fortran NINT: half away from zero
inline double &V(double *a, int i, int j, int na, int k) { return a[i + 3 * ((size_t)j + (size_t)na * k)]; }
inline double &X(double *a, int i, int j) { return a[i + 3 * (size_t)j]; }
inline double X(const double *a, int i, int j) { return a[i + 3 * (size_t)j]; }
inline double &M33(double *m, int i, int j) { return m[i + 3 * j]; }  // vir(i,j), 0-based

void zero9(double *v) { for (int i = 0; i < 9; ++i) v[i] = 0.0; }
}  // namespace

// ===========================================================================
// linked cells (linked_cell.f90)
// ===========================================================================
namespace {
struct CellNC {
  int ncell[3], mcell[3], nn;
  std::vector<int> link;            // link(ncx,ncy,ncz), 1-based atom index or 0
  std::vector<int> ink;             // ink(3,nn)
  std::vector<int> mapx, mapy, mapz;  // map(ncell, -m:m)
  int &L(int ix, int iy, int iz) { return link[(ix - 1) + ncell[0] * ((iy - 1) + ncell[1] * (iz - 1))]; }
  int Mx(int ix, int j) const { return mapx[(ix - 1) + ncell[0] * (j + mcell[0])]; }
  int My(int iy, int j) const { return mapy[(iy - 1) + ncell[1] * (j + mcell[1])]; }
  int Mz(int iz, int j) const { return mapz[(iz - 1) + ncell[2] * (j + mcell[2])]; }
};

// cell_setup (linked_cell.f90:1-32)
void cell_setup(const double box[3], double rcut, CellNC &c) {
  c.nn = 1;
  for (int i = 0; i < 3; ++i) {
    if (3.0 * rcut > box[i]) {
      c.ncell[i] = 1;
      c.mcell[i] = 0;
    } else {
      c.ncell[i] = std::max(6, (int)(2.0 * box[i] / rcut));
      c.mcell[i] = 2;
    }
    c.nn = c.nn * (2 * c.mcell[i] + 1);
  }
  c.nn = (c.nn - 1) / 2;
}

// cell_map_nc (linked_cell.f90:188-282)
void cell_map_nc(CellNC &c) {
  c.ink.assign(3 * std::max(c.nn, 1), 0);
  int k = 0;
  for (int iz = 1; iz <= c.mcell[2]; ++iz)
    for (int iy = -c.mcell[1]; iy <= c.mcell[1]; ++iy)
      for (int ix = -c.mcell[0]; ix <= c.mcell[0]; ++ix) {
        c.ink[3 * k] = ix; c.ink[3 * k + 1] = iy; c.ink[3 * k + 2] = iz; ++k;
      }
  for (int iy = 1; iy <= c.mcell[1]; ++iy)
    for (int ix = -c.mcell[0]; ix <= c.mcell[0]; ++ix) {
      c.ink[3 * k] = ix; c.ink[3 * k + 1] = iy; c.ink[3 * k + 2] = 0; ++k;
    }
  for (int ix = 1; ix <= c.mcell[0]; ++ix) {
    c.ink[3 * k] = ix; c.ink[3 * k + 1] = 0; c.ink[3 * k + 2] = 0; ++k;
  }
  auto mk = [](std::vector<int> &map, int nc, int mc) {
    map.assign(nc * (2 * mc + 1), 0);
    for (int ix = 1; ix <= nc; ++ix)
      for (int jx = -mc; jx <= mc; ++jx) {
        int kx = ix + jx;
        if (kx < 1) kx += nc; else if (kx > nc) kx -= nc;
        map[(ix - 1) + nc * (jx + mc)] = kx;
      }
  };
  mk(c.mapx, c.ncell[0], c.mcell[0]);
  mk(c.mapy, c.ncell[1], c.mcell[1]);
  mk(c.mapz, c.ncell[2], c.mcell[2]);
}

// cell_list (linked_cell.f90:34-89); list is the chain, 1-based, size n+1
void cell_list(const double *r, std::vector<int> &list, CellNC &c, int n, const double box[3],
               int ijump) {
  double boxx = box[0], boxy = box[1], boxz = box[2];
  double onboxx = 1.0 / boxx, onboxy = 1.0 / boxy, onboxz = 1.0 / boxz;
  double halfx = 0.5 * boxx, halfy = 0.5 * boxy, halfz = 0.5 * boxz;
  c.link.assign(c.ncell[0] * c.ncell[1] * c.ncell[2], 0);
  list.assign(n + 1, 0);
  double cellx = (double)c.ncell[0] / boxx, celly = (double)c.ncell[1] / boxy,
         cellz = (double)c.ncell[2] / boxz;
  for (int i = 1; i <= n; i += ijump) {
    double dx = X(r, 0, i - 1) - boxx * nint(onboxx * X(r, 0, i - 1));
    double dy = X(r, 1, i - 1) - boxy * nint(onboxy * X(r, 1, i - 1));
    double dz = X(r, 2, i - 1) - boxz * nint(onboxz * X(r, 2, i - 1));
    int ix = std::min(c.ncell[0], 1 + (int)((dx + halfx) * cellx));
    int iy = std::min(c.ncell[1], 1 + (int)((dy + halfy) * celly));
    int iz = std::min(c.ncell[2], 1 + (int)((dz + halfz) * cellz));
    list[i] = c.L(ix, iy, iz);
    c.L(ix, iy, iz) = i;
  }
  if (c.nn > 0) cell_map_nc(c);
}

struct CellUnit {
  int ncell, mcell, nn;
  std::vector<int> link, ink, map;
  int &L(int ix, int iy, int iz) { return link[(ix - 1) + ncell * ((iy - 1) + ncell * (iz - 1))]; }
  int Mp(int ix, int j) const { return map[(ix - 1) + ncell * (j + 2)]; }
};

// cell_map (linked_cell.f90:131-186)
void cell_map(CellUnit &c) {
  c.ink.assign(3 * 62, 0);
  int k = 0, m = c.mcell;
  for (int iz = 1; iz <= m; ++iz)
    for (int iy = -m; iy <= m; ++iy)
      for (int ix = -m; ix <= m; ++ix) {
        c.ink[3 * k] = ix; c.ink[3 * k + 1] = iy; c.ink[3 * k + 2] = iz; ++k;
      }
  for (int iy = 1; iy <= m; ++iy)
    for (int ix = -m; ix <= m; ++ix) {
      c.ink[3 * k] = ix; c.ink[3 * k + 1] = iy; c.ink[3 * k + 2] = 0; ++k;
    }
  for (int ix = 1; ix <= m; ++ix) {
    c.ink[3 * k] = ix; c.ink[3 * k + 1] = 0; c.ink[3 * k + 2] = 0; ++k;
  }
  c.map.assign(c.ncell * 5, 0);
  for (int ix = 1; ix <= c.ncell; ++ix)
    for (int jx = -m; jx <= m; ++jx) {
      int kx = ix + jx;
      if (kx < 1) kx += c.ncell; else if (kx > c.ncell) kx -= c.ncell;
      c.map[(ix - 1) + c.ncell * (jx + 2)] = kx;
    }
}

// cell_list_unit (linked_cell.f90:91-129)
void cell_list_unit(const double *r, std::vector<int> &list, CellUnit &c, int n) {
  c.link.assign(c.ncell * c.ncell * c.ncell, 0);
  list.assign(n + 1, 0);
  double cell = (double)c.ncell;
  for (int i = 1; i <= n; ++i) {
    double dx = X(r, 0, i - 1) - nint(X(r, 0, i - 1));
    double dy = X(r, 1, i - 1) - nint(X(r, 1, i - 1));
    double dz = X(r, 2, i - 1) - nint(X(r, 2, i - 1));
    long ix = std::min((long)c.ncell, 1 + (long)((dx + 0.5) * cell));
    long iy = std::min((long)c.ncell, 1 + (long)((dy + 0.5) * cell));
    long iz = std::min((long)c.ncell, 1 + (long)((dz + 0.5) * cell));
    list[i] = c.L((int)ix, (int)iy, (int)iz);
    c.L((int)ix, (int)iy, (int)iz) = i;
  }
  c.nn = ((2 * c.mcell + 1) * (2 * c.mcell + 1) * (2 * c.mcell + 1) - 1) / 2;
  if (c.mcell > 0) cell_map(c); else c.nn = 0;
}
}  // namespace

// ===========================================================================
// Ewald sum, cubic box (ewald_cubic.f90)
// ===========================================================================
void ewald_cubic(int n, const int *mol, const double *q, const double *r, double &v,
                 double vir[9], double *dvdr, double boxl) {
  std::vector<double> rs(3 * (size_t)n);
  double onboxl = 1.0 / boxl;
  for (size_t i = 0; i < 3 * (size_t)n; ++i) rs[i] = onboxl * r[i];
  v = 0.0;
  zero9(vir);
  double rkmax2 = P.rkmax * P.rkmax;
  int ncell, mcell;
  if (3.0 * P.wrcut > 1.0) {
    ncell = 1;
    mcell = 0;
  } else {
    ncell = std::max(6, (int)(2.0 / P.wrcut));
    mcell = 2;
  }
  rwald(n, mol, q, rs.data(), v, vir, dvdr, P.wrcut, P.walpha, mcell, ncell);
  kwald(n, q, rs.data(), v, vir, dvdr, P.walpha, rkmax2, P.kmax);
  v = onboxl * v;
  for (int i = 0; i < 9; ++i) vir[i] = onboxl * vir[i];
  double onbox2 = onboxl * onboxl;
  for (size_t i = 0; i < 3 * (size_t)n; ++i) dvdr[i] = onbox2 * dvdr[i];
}

// rwald (ewald_cubic.f90:78-233): real-space sum with the A&S 7.1.26 erfc
void rwald(int n, const int *mol, const double *q, const double *r, double &v, double vir[9],
           double *dvdr, double rcut, double alpha, int mcell, int ncell) {
  const double p = 3.0525860, a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741,
               a4 = -1.453152027, a5 = 1.061405429;
  CellUnit c;
  c.ncell = ncell;
  c.mcell = mcell;
  std::vector<int> list;
  cell_list_unit(r, list, c, n);
  const double pi = std::acos(-1.0);
  double rfac = alpha / std::sqrt(pi);
  double sfac = -2.0 * rfac;
  double rcutsq = rcut * rcut;

  auto pair = [&](int i, int j) {  // 1-based
    double dx = X(r, 0, i - 1) - X(r, 0, j - 1);
    double dy = X(r, 1, i - 1) - X(r, 1, j - 1);
    double dz = X(r, 2, i - 1) - X(r, 2, j - 1);
    dx = dx - nint(dx);
    dy = dy - nint(dy);
    dz = dz - nint(dz);
    double drsq = dx * dx + dy * dy + dz * dz;
    if (drsq < rcutsq) {
      double dr = std::sqrt(drsq);
      double x = alpha * dr;
      double e = std::exp(-x * x);
      double t = p / (p + x);
      double erfc = e * t * (a1 + t * (a2 + t * (a3 + t * (a4 + t * a5))));
      if (mol[i - 1] == mol[j - 1]) erfc = erfc - 1.0;
      double du = erfc / dr;
      double dur = (sfac * e - du) / drsq;
      double qij = q[i - 1] * q[j - 1];
      double dv = qij * du;
      double dvr = qij * dur;
      double dvx = dvr * dx, dvy = dvr * dy, dvz = dvr * dz;
      v = v + dv;
      X(dvdr, 0, i - 1) += dvx; X(dvdr, 1, i - 1) += dvy; X(dvdr, 2, i - 1) += dvz;
      X(dvdr, 0, j - 1) -= dvx; X(dvdr, 1, j - 1) -= dvy; X(dvdr, 2, j - 1) -= dvz;
      M33(vir, 0, 0) += dx * dvx; M33(vir, 0, 1) += dx * dvy; M33(vir, 0, 2) += dx * dvz;
      M33(vir, 1, 0) += dy * dvx; M33(vir, 1, 1) += dy * dvy; M33(vir, 1, 2) += dy * dvz;
      M33(vir, 2, 0) += dz * dvx; M33(vir, 2, 1) += dz * dvy; M33(vir, 2, 2) += dz * dvz;
    }
  };
  for (int iz = 1; iz <= ncell; ++iz)
    for (int iy = 1; iy <= ncell; ++iy)
      for (int ix = 1; ix <= ncell; ++ix) {
        int i = c.L(ix, iy, iz);
        while (i > 0) {
          int j = list[i];
          while (j > 0) {
            pair(i, j);
            j = list[j];
          }
          i = list[i];
        }
      }
  for (int k = 0; k < c.nn; ++k) {
    int incx = c.ink[3 * k], incy = c.ink[3 * k + 1], incz = c.ink[3 * k + 2];
    for (int iz = 1; iz <= ncell; ++iz) {
      int jz = c.Mp(iz, incz);
      for (int iy = 1; iy <= ncell; ++iy) {
        int jy = c.Mp(iy, incy);
        for (int ix = 1; ix <= ncell; ++ix) {
          int jx = c.Mp(ix, incx);
          int i = c.L(ix, iy, iz);
          while (i > 0) {
            int j = c.L(jx, jy, jz);
            while (j > 0) {
              pair(i, j);
              j = list[j];
            }
            i = list[i];
          }
        }
      }
    }
  }
}

// kwald (ewald_cubic.f90:235-533): reciprocal-space sum over the half space
void kwald(int n, const double *q, const double *r, double &v, double vir[9], double *dvdr,
           double alpha, double rkmax2, int kmax) {
  const int K = kmax + 1;
  // cx(2,n,0:kmax) -> cx[c + 2*(i + n*k)]
  std::vector<double> cx(2 * (size_t)n * K), cy(2 * (size_t)n * K), cz(2 * (size_t)n * K);
  std::vector<double> cj(4 * (size_t)n), ck(8 * (size_t)n);
  auto C = [n](std::vector<double> &a, int c, int i, int k) -> double & { return a[c + 2 * ((size_t)i + (size_t)n * k)]; };
  const double pi = std::acos(-1.0);
  const double rlat = 2.0 * pi;
  for (int i = 0; i < n; ++i) {
    C(cx, 0, i, 0) = q[i];
    C(cx, 1, i, 0) = 0.0;
    double arg = rlat * X(r, 0, i), c = std::cos(arg), s = std::sin(arg);
    for (int k = 1; k <= kmax; ++k) {
      C(cx, 0, i, k) = c * C(cx, 0, i, k - 1) - s * C(cx, 1, i, k - 1);
      C(cx, 1, i, k) = s * C(cx, 0, i, k - 1) + c * C(cx, 1, i, k - 1);
    }
  }
  for (int i = 0; i < n; ++i) {
    C(cy, 0, i, 0) = 1.0;
    C(cy, 1, i, 0) = 0.0;
    double arg = rlat * X(r, 1, i), c = std::cos(arg), s = std::sin(arg);
    for (int k = 1; k <= kmax; ++k) {
      C(cy, 0, i, k) = c * C(cy, 0, i, k - 1) - s * C(cy, 1, i, k - 1);
      C(cy, 1, i, k) = s * C(cy, 0, i, k - 1) + c * C(cy, 1, i, k - 1);
    }
  }
  for (int i = 0; i < n; ++i) {
    C(cz, 0, i, 0) = 1.0;
    C(cz, 1, i, 0) = 0.0;
    double arg = rlat * X(r, 2, i), c = std::cos(arg), s = std::sin(arg);
    for (int k = 1; k <= kmax; ++k) {
      C(cz, 0, i, k) = c * C(cz, 0, i, k - 1) - s * C(cz, 1, i, k - 1);
      C(cz, 1, i, k) = s * C(cz, 0, i, k - 1) + c * C(cz, 1, i, k - 1);
    }
  }
  double b = 0.25 / (alpha * alpha);
  double f = rlat;
  for (int kx = 0; kx <= kmax; ++kx) {
    if (kx == 1) f = 2.0 * f;
    double rkx = rlat * kx, rky = 0.0, rkz = 0.0;
    double rk2 = rkx * rkx;
    if (rk2 > 0.0) {  // ky = 0, kz = 0
      double s1 = 0.0, s2 = 0.0;
      for (int i = 0; i < n; ++i) {
        s1 = s1 + C(cx, 0, i, kx);
        s2 = s2 + C(cx, 1, i, kx);
      }
      double w = (f / rk2) * std::exp(-b * rk2);
      double et = w * (s1 * s1 + s2 * s2);
      v = v + et;
      double term = 2.0 * (1.0 / rk2 + b);
      M33(vir, 0, 0) += et * (term * rkx * rkx - 1.0);
      M33(vir, 1, 1) += et * (-1.0);
      M33(vir, 2, 2) += et * (-1.0);
      w = w + w;
      double wkx = w * rkx;
      for (int i = 0; i < n; ++i) {
        double t2 = s2 * C(cx, 0, i, kx) - s1 * C(cx, 1, i, kx);
        X(dvdr, 0, i) += wkx * t2;
      }
    }
    for (int kz = 1; kz <= kmax; ++kz) {  // ky = 0, |kz| > 0
      rky = 0.0;
      rkz = rlat * kz;
      rk2 = rkx * rkx + rkz * rkz;
      if (rk2 > rkmax2) break;
      double s1 = 0.0, s2 = 0.0, s3 = 0.0, s4 = 0.0;
      for (int i = 0; i < n; ++i) {
        double cc = C(cx, 0, i, kx) * C(cz, 0, i, kz);
        double cs = C(cx, 0, i, kx) * C(cz, 1, i, kz);
        double sc = C(cx, 1, i, kx) * C(cz, 0, i, kz);
        double ss = C(cx, 1, i, kx) * C(cz, 1, i, kz);
        cj[4 * i + 0] = cc - ss;
        cj[4 * i + 1] = sc + cs;
        cj[4 * i + 2] = cc + ss;
        cj[4 * i + 3] = sc - cs;
        s1 = s1 + cj[4 * i + 0];
        s2 = s2 + cj[4 * i + 1];
        s3 = s3 + cj[4 * i + 2];
        s4 = s4 + cj[4 * i + 3];
      }
      double w = (f / rk2) * std::exp(-b * rk2);
      double et = w * (s1 * s1 + s2 * s2 + s3 * s3 + s4 * s4);
      v = v + et;
      double term = 2.0 * (1.0 / rk2 + b);
      double xx = et * (term * rkx * rkx - 1.0);
      double xz = et * (term * rkx * rkz);
      double yy = et * (-1.0);
      double zz = et * (term * rkz * rkz - 1.0);
      M33(vir, 0, 0) += xx;
      M33(vir, 0, 2) += xz;
      M33(vir, 1, 1) += yy;
      M33(vir, 2, 0) += xz;
      M33(vir, 2, 2) += zz;
      w = w + w;
      double wkx = w * rkx, wkz = w * rkz;
      for (int i = 0; i < n; ++i) {
        double t2 = s2 * cj[4 * i + 0] - s1 * cj[4 * i + 1];
        double t4 = s4 * cj[4 * i + 2] - s3 * cj[4 * i + 3];
        X(dvdr, 0, i) += wkx * (t2 + t4);
        X(dvdr, 2, i) += wkz * (t2 - t4);
      }
    }
    for (int ky = 1; ky <= kmax; ++ky) {  // |ky| > 0, kz = 0
      rkz = 0.0;
      rky = rlat * ky;
      rk2 = rkx * rkx + rky * rky;
      if (rk2 > rkmax2) break;
      double s1 = 0.0, s2 = 0.0, s3 = 0.0, s4 = 0.0;
      for (int i = 0; i < n; ++i) {
        double cc = C(cx, 0, i, kx) * C(cy, 0, i, ky);
        double cs = C(cx, 0, i, kx) * C(cy, 1, i, ky);
        double sc = C(cx, 1, i, kx) * C(cy, 0, i, ky);
        double ss = C(cx, 1, i, kx) * C(cy, 1, i, ky);
        cj[4 * i + 0] = cc - ss;
        cj[4 * i + 1] = sc + cs;
        cj[4 * i + 2] = cc + ss;
        cj[4 * i + 3] = sc - cs;
        s1 = s1 + cj[4 * i + 0];
        s2 = s2 + cj[4 * i + 1];
        s3 = s3 + cj[4 * i + 2];
        s4 = s4 + cj[4 * i + 3];
      }
      double w = (f / rk2) * std::exp(-b * rk2);
      double et = w * (s1 * s1 + s2 * s2 + s3 * s3 + s4 * s4);
      v = v + et;
      double term = 2.0 * (1.0 / rk2 + b);
      double xx = et * (term * rkx * rkx - 1.0);
      double xy = et * (term * rkx * rky);
      double yy = et * (term * rky * rky - 1.0);
      double zz = et * (-1.0);
      M33(vir, 0, 0) += xx;
      M33(vir, 0, 1) += xy;
      M33(vir, 1, 0) += xy;
      M33(vir, 1, 1) += yy;
      M33(vir, 2, 2) += zz;
      w = w + w;
      double wkx = w * rkx, wky = w * rky;
      for (int i = 0; i < n; ++i) {
        double t2 = s2 * cj[4 * i + 0] - s1 * cj[4 * i + 1];
        double t4 = s4 * cj[4 * i + 2] - s3 * cj[4 * i + 3];
        X(dvdr, 0, i) += wkx * (t2 + t4);
        X(dvdr, 1, i) += wky * (t2 - t4);
      }
      for (int kz = 1; kz <= kmax; ++kz) {  // |ky| > 0, |kz| > 0
        rkz = rlat * kz;
        rk2 = rkx * rkx + rky * rky + rkz * rkz;
        if (rk2 > rkmax2) break;
        double s[8] = {0, 0, 0, 0, 0, 0, 0, 0};
        for (int i = 0; i < n; ++i) {
          double czr = C(cz, 0, i, kz), czi = C(cz, 1, i, kz);
          double cca = cj[4 * i + 0] * czr, csa = cj[4 * i + 0] * czi;
          double sca = cj[4 * i + 1] * czr, ssa = cj[4 * i + 1] * czi;
          double ccb = cj[4 * i + 2] * czr, csb = cj[4 * i + 2] * czi;
          double scb = cj[4 * i + 3] * czr, ssb = cj[4 * i + 3] * czi;
          double *c8 = &ck[8 * (size_t)i];
          c8[0] = cca - ssa; c8[1] = sca + csa; c8[2] = cca + ssa; c8[3] = sca - csa;
          c8[4] = ccb - ssb; c8[5] = scb + csb; c8[6] = ccb + ssb; c8[7] = scb - csb;
          for (int m = 0; m < 8; ++m) s[m] = s[m] + c8[m];
        }
        double w = (f / rk2) * std::exp(-b * rk2);
        double et = w * (s[0] * s[0] + s[1] * s[1] + s[2] * s[2] + s[3] * s[3] + s[4] * s[4] +
                         s[5] * s[5] + s[6] * s[6] + s[7] * s[7]);
        v = v + et;
        double term = 2.0 * (1.0 / rk2 + b);
        double xx = et * (term * rkx * rkx - 1.0);
        double xy = et * (term * rkx * rky);
        double xz = et * (term * rkx * rkz);
        double yy = et * (term * rky * rky - 1.0);
        double yz = et * (term * rky * rkz);
        double zz = et * (term * rkz * rkz - 1.0);
        M33(vir, 0, 0) += xx; M33(vir, 0, 1) += xy; M33(vir, 0, 2) += xz;
        M33(vir, 1, 0) += xy; M33(vir, 1, 1) += yy; M33(vir, 1, 2) += yz;
        M33(vir, 2, 0) += xz; M33(vir, 2, 1) += yz; M33(vir, 2, 2) += zz;
        w = w + w;
        double wkx = w * rkx, wky = w * rky, wkz = w * rkz;
        for (int i = 0; i < n; ++i) {
          const double *c8 = &ck[8 * (size_t)i];
          double t2 = s[1] * c8[0] - s[0] * c8[1];
          double t4 = s[3] * c8[2] - s[2] * c8[3];
          double t6 = s[5] * c8[4] - s[4] * c8[5];
          double t8 = s[7] * c8[6] - s[6] * c8[7];
          X(dvdr, 0, i) += wkx * (t2 + t4 + t6 + t8);
          X(dvdr, 1, i) += wky * (t2 + t4 - t6 - t8);
          X(dvdr, 2, i) += wkz * (t2 - t4 + t6 - t8);
        }
      }
    }
  }
  double vs = 0.0;  // self term
  for (int i = 0; i < n; ++i) vs = vs + q[i] * q[i];
  double rfac = alpha / std::sqrt(pi);
  vs = rfac * vs;
  v = v - vs;
}

// ===========================================================================
// Ewald sum, non-cubic box (ewald_noncubic.f90)
// ===========================================================================
// one real-space pair of rwald_basic / rwald_cell (ewald_noncubic.f90:103-152,
// 271-308), i, j 1-based, minimum image per side
inline void rwald_nc_pair(int i, int j, const int *mol, const double *q, const double *r, double &v,
                          double vir[9], double *dvdr, double rcutsq, double alpha, double sfac,
                          const double box[3], const double onbox[3]) {
  const double p = 3.0525860, a1 = 0.254829592, a2 = -0.284496736, a3 = 1.421413741,
               a4 = -1.453152027, a5 = 1.061405429;
  double dx = X(r, 0, i - 1) - X(r, 0, j - 1);
  double dy = X(r, 1, i - 1) - X(r, 1, j - 1);
  double dz = X(r, 2, i - 1) - X(r, 2, j - 1);
  dx = dx - box[0] * nint(dx * onbox[0]);
  dy = dy - box[1] * nint(dy * onbox[1]);
  dz = dz - box[2] * nint(dz * onbox[2]);
  double drsq = dx * dx + dy * dy + dz * dz;
  if (drsq < rcutsq) {
    double dr = std::sqrt(drsq);
    double x = alpha * dr;
    double e = std::exp(-x * x);
    double t = p / (p + x);
    double erfc = e * t * (a1 + t * (a2 + t * (a3 + t * (a4 + t * a5))));
    if (mol[i - 1] == mol[j - 1]) erfc = erfc - 1.0;
    double du = erfc / dr;
    double dur = (sfac * e - du) / drsq;
    double qij = q[i - 1] * q[j - 1];
    double dv = qij * du;
    double dvr = qij * dur;
    double dvx = dvr * dx, dvy = dvr * dy, dvz = dvr * dz;
    v = v + dv;
    X(dvdr, 0, i - 1) += dvx; X(dvdr, 1, i - 1) += dvy; X(dvdr, 2, i - 1) += dvz;
    X(dvdr, 0, j - 1) -= dvx; X(dvdr, 1, j - 1) -= dvy; X(dvdr, 2, j - 1) -= dvz;
    M33(vir, 0, 0) += dx * dvx; M33(vir, 0, 1) += dx * dvy; M33(vir, 0, 2) += dx * dvz;
    M33(vir, 1, 0) += dy * dvx; M33(vir, 1, 1) += dy * dvy; M33(vir, 1, 2) += dy * dvz;
    M33(vir, 2, 0) += dz * dvx; M33(vir, 2, 1) += dz * dvy; M33(vir, 2, 2) += dz * dvz;
  }
}

// rwald_basic (ewald_noncubic.f90:204-273) and rwald_cell (ewald_noncubic.f90:56-202)
void rwald_nc(int n, const int *mol, const double *q, const double *r, double &v, double vir[9],
              double *dvdr, double rcut, double alpha, const double box[3], bool cells) {
  const double pi = std::acos(-1.0);
  double rfac = alpha / std::sqrt(pi);
  double sfac = -2.0 * rfac;
  double rcutsq = rcut * rcut;
  const double onbox[3] = {1.0 / box[0], 1.0 / box[1], 1.0 / box[2]};
  if (!cells) {
    for (int i = 1; i <= n; ++i)
      for (int j = 1; j <= i - 1; ++j) rwald_nc_pair(i, j, mol, q, r, v, vir, dvdr, rcutsq, alpha, sfac, box, onbox);
    return;
  }
  CellNC c;
  cell_setup(box, rcut, c);
  std::vector<int> list;
  cell_list(r, list, c, n, box, 1);
  for (int iz = 1; iz <= c.ncell[2]; ++iz)
    for (int iy = 1; iy <= c.ncell[1]; ++iy)
      for (int ix = 1; ix <= c.ncell[0]; ++ix) {
        int i = c.L(ix, iy, iz);
        while (i > 0) {
          int j = list[i];
          while (j > 0) {
            rwald_nc_pair(i, j, mol, q, r, v, vir, dvdr, rcutsq, alpha, sfac, box, onbox);
            j = list[j];
          }
          i = list[i];
        }
      }
  for (int k = 1; k <= c.nn; ++k) {
    int incx = c.ink[3 * (k - 1)], incy = c.ink[3 * (k - 1) + 1], incz = c.ink[3 * (k - 1) + 2];
    for (int iz = 1; iz <= c.ncell[2]; ++iz) {
      int jz = c.Mz(iz, incz);
      for (int iy = 1; iy <= c.ncell[1]; ++iy) {
        int jy = c.My(iy, incy);
        for (int ix = 1; ix <= c.ncell[0]; ++ix) {
          int jx = c.Mx(ix, incx);
          int i = c.L(ix, iy, iz);
          while (i > 0) {
            int j = c.L(jx, jy, jz);
            while (j > 0) {
              rwald_nc_pair(i, j, mol, q, r, v, vir, dvdr, rcutsq, alpha, sfac, box, onbox);
              j = list[j];
            }
            i = list[i];
          }
        }
      }
    }
  }
}

// kwald_nc (ewald_noncubic.f90:275-460): every k with kx >= 0, |ky|, |kz| <= kmax
// and 0 < |k|^2 < rkmax2; weight 2 pi / V at kx = 0, 4 pi / V beyond
void kwald_nc(const double *r, const double *z, int n, double &v, double vir[9], double *dvdr,
              double alpha, double rkmax2, int kmax, const double box[3]) {
  const double pi = std::acos(-1.0);
  double rfac = alpha / std::sqrt(pi);
  double twopi = 2.0 * pi;
  double xbox = box[0], ybox = box[1], zbox = box[2];
  double xlat = twopi / xbox, ylat = twopi / ybox, zlat = twopi / zbox;
  const int K = kmax, W = 2 * kmax + 1;
  std::vector<double> ckx((size_t)n * (K + 1)), skx((size_t)n * (K + 1)), cky((size_t)n * W), sky((size_t)n * W),
      ckz((size_t)n * W), skz((size_t)n * W), cxy(n), sxy(n), dsdr(6 * (size_t)n);
  auto IX = [&](int i, int k) { return (size_t)i + (size_t)n * k; };          // (i, 0:kmax)
  auto IY = [&](int i, int k) { return (size_t)i + (size_t)n * (k + K); };    // (i, -kmax:kmax)
  for (int i = 0; i < n; ++i) {
    ckx[IX(i, 0)] = z[i];
    skx[IX(i, 0)] = 0.0;
    double xi = xlat * X(r, 0, i);
    double c = std::cos(xi), s = std::sin(xi);
    for (int kx = 1; kx <= K; ++kx) {
      ckx[IX(i, kx)] = c * ckx[IX(i, kx - 1)] - s * skx[IX(i, kx - 1)];
      skx[IX(i, kx)] = s * ckx[IX(i, kx - 1)] + c * skx[IX(i, kx - 1)];
    }
  }
  for (int i = 0; i < n; ++i) {
    cky[IY(i, 0)] = 1.0;
    sky[IY(i, 0)] = 0.0;
    double yi = ylat * X(r, 1, i);
    double c = std::cos(yi), s = std::sin(yi);
    for (int ky = 1; ky <= K; ++ky) {
      cky[IY(i, ky)] = c * cky[IY(i, ky - 1)] - s * sky[IY(i, ky - 1)];
      sky[IY(i, ky)] = s * cky[IY(i, ky - 1)] + c * sky[IY(i, ky - 1)];
      cky[IY(i, -ky)] = cky[IY(i, ky)];
      sky[IY(i, -ky)] = -sky[IY(i, ky)];
    }
  }
  for (int i = 0; i < n; ++i) {
    ckz[IY(i, 0)] = 1.0;
    skz[IY(i, 0)] = 0.0;
    double zi = zlat * X(r, 2, i);
    double c = std::cos(zi), s = std::sin(zi);
    for (int kz = 1; kz <= K; ++kz) {
      ckz[IY(i, kz)] = c * ckz[IY(i, kz - 1)] - s * skz[IY(i, kz - 1)];
      skz[IY(i, kz)] = s * ckz[IY(i, kz - 1)] + c * skz[IY(i, kz - 1)];
      ckz[IY(i, -kz)] = ckz[IY(i, kz)];
      skz[IY(i, -kz)] = -skz[IY(i, kz)];
    }
  }
  double b = 0.25 / (alpha * alpha);
  double f = twopi / (xbox * ybox * zbox);
  for (int kx = 0; kx <= K; ++kx) {
    if (kx == 1) f = 2.0 * f;
    double rkx = xlat * kx;
    for (int ky = -K; ky <= K; ++ky) {
      double rky = ylat * ky;
      for (int i = 0; i < n; ++i) {
        cxy[i] = ckx[IX(i, kx)] * cky[IY(i, ky)] - skx[IX(i, kx)] * sky[IY(i, ky)];
        sxy[i] = ckx[IX(i, kx)] * sky[IY(i, ky)] + skx[IX(i, kx)] * cky[IY(i, ky)];
      }
      for (int kz = -K; kz <= K; ++kz) {
        double rkz = zlat * kz;
        double rk2 = rkx * rkx + rky * rky + rkz * rkz;
        if (rk2 < rkmax2 && rk2 != 0.0) {
          double sr = 0.0, si = 0.0;
          for (int i = 0; i < n; ++i) {
            double tr = cxy[i] * ckz[IY(i, kz)] - sxy[i] * skz[IY(i, kz)];
            double ti = cxy[i] * skz[IY(i, kz)] + sxy[i] * ckz[IY(i, kz)];
            sr = sr + tr;
            si = si + ti;
            dsdr[6 * i + 0] = -rkx * ti;
            dsdr[6 * i + 1] = rkx * tr;
            dsdr[6 * i + 2] = -rky * ti;
            dsdr[6 * i + 3] = rky * tr;
            dsdr[6 * i + 4] = -rkz * ti;
            dsdr[6 * i + 5] = rkz * tr;
          }
          double w = (f / rk2) * std::exp(-b * rk2);
          double et = w * (sr * sr + si * si);
          v = v + et;
          w = 2.0 * w;
          sr = w * sr;
          si = w * si;
          for (int i = 0; i < n; ++i) {
            X(dvdr, 0, i) += sr * dsdr[6 * i + 0] + si * dsdr[6 * i + 1];
            X(dvdr, 1, i) += sr * dsdr[6 * i + 2] + si * dsdr[6 * i + 3];
            X(dvdr, 2, i) += sr * dsdr[6 * i + 4] + si * dsdr[6 * i + 5];
          }
          double term = 2.0 * (1.0 / rk2 + b);
          double xx = et * (term * rkx * rkx - 1.0), xy = et * (term * rkx * rky), xz = et * (term * rkx * rkz);
          double yy = et * (term * rky * rky - 1.0), yz = et * (term * rky * rkz), zz = et * (term * rkz * rkz - 1.0);
          M33(vir, 0, 0) += xx; M33(vir, 0, 1) += xy; M33(vir, 0, 2) += xz;
          M33(vir, 1, 0) += xy; M33(vir, 1, 1) += yy; M33(vir, 1, 2) += yz;
          M33(vir, 2, 0) += xz; M33(vir, 2, 1) += yz; M33(vir, 2, 2) += zz;
        }
      }
    }
  }
  double vs = 0.0;
  for (int i = 0; i < n; ++i) vs = vs + z[i] * z[i];
  vs = rfac * vs;
  v = v - vs;
}

// ewald_nc (ewald_noncubic.f90:1-54), point charges: rwald_basic when
// 3 wrcut > the longest side, else rwald_cell; then kwald_nc
void ewald_nc(int n, const int *mol, const double *q, const double *r, double &v, double vir[9],
              double *dvdr, const double box[3]) {
  v = 0.0;
  zero9(vir);
  double boxmax = std::max(box[0], std::max(box[1], box[2]));
  rwald_nc(n, mol, q, r, v, vir, dvdr, P.wrcut, P.walpha, box, !(3.0 * P.wrcut > boxmax));
  kwald_nc(r, q, n, v, vir, dvdr, P.walpha, P.rkmax * P.rkmax, P.kmax, box);
}

// ===========================================================================
// neighbour lists (neigh_list.f90); list/point are 1-based like the Fortran:
// point has na+3 entries at indices 1..na+3, list has maxnab*na entries at
// indices 1..maxnab*na; index 0 of each array is unused.
// ===========================================================================
namespace {
Status nei_list(const double *r, int na, int *list, int *point, int njump, double rcut,
                const double box[3]) {
  double rcutsq = rcut * rcut;
  double boxx = box[0], boxy = box[1], boxz = box[2];
  double onboxx = 1.0 / boxx, onboxy = 1.0 / boxy, onboxz = 1.0 / boxz;
  std::memset(point, 0, sizeof(int) * (na + 4));
  std::memset(list, 0, sizeof(int) * ((size_t)maxnab * na + 1));
  int nlist = 0;
  int jend = na - njump + 1;
  for (int j = 1; j <= jend; j += njump) {
    point[j] = nlist + 1;
    double rxj = X(r, 0, j - 1), ryj = X(r, 1, j - 1), rzj = X(r, 2, j - 1);
    for (int i = j + njump; i <= na; i += njump) {
      double dx = X(r, 0, i - 1) - rxj, dy = X(r, 1, i - 1) - ryj, dz = X(r, 2, i - 1) - rzj;
      dx = dx - boxx * nint(onboxx * dx);
      dy = dy - boxy * nint(onboxy * dy);
      dz = dz - boxz * nint(onboxz * dz);
      double drsq = dx * dx + dy * dy + dz * dz;
      if (drsq < rcutsq) {
        nlist = nlist + 1;
        if (nlist == maxnab * na) return GB_E_LIST;
        list[nlist] = i;
      }
    }
  }
  for (int i = jend + njump; i <= na + njump; i += njump) {
    nlist = nlist + 1;
    point[i] = nlist;
  }
  return GB_OK;
}

Status nei_cell(const double *r, int na, int *list, int *point, int njump, double rcut,
                const double box[3]) {
  CellNC c;
  cell_setup(box, rcut, c);
  std::vector<int> clist;
  cell_list(r, clist, c, na, box, njump);
  double boxx = box[0], boxy = box[1], boxz = box[2];
  double onboxx = 1.0 / boxx, onboxy = 1.0 / boxy, onboxz = 1.0 / boxz;
  double halfx = 0.5 * boxx, halfy = 0.5 * boxy, halfz = 0.5 * boxz;
  double rcutsq = rcut * rcut;
  double cellx = c.ncell[0] / boxx, celly = c.ncell[1] / boxy, cellz = c.ncell[2] / boxz;
  std::memset(point, 0, sizeof(int) * (na + 4));
  std::memset(list, 0, sizeof(int) * ((size_t)maxnab * na + 1));
  int nlist = 0;
  int jend = na - njump + 1;
  for (int j = 1; j <= jend; j += njump) {
    point[j] = nlist + 1;
    double rxj = X(r, 0, j - 1), ryj = X(r, 1, j - 1), rzj = X(r, 2, j - 1);
    double dx = X(r, 0, j - 1) - boxx * nint(onboxx * X(r, 0, j - 1));
    double dy = X(r, 1, j - 1) - boxy * nint(onboxy * X(r, 1, j - 1));
    double dz = X(r, 2, j - 1) - boxz * nint(onboxz * X(r, 2, j - 1));
    int jx = std::min(c.ncell[0], 1 + (int)((dx + halfx) * cellx));
    int jy = std::min(c.ncell[1], 1 + (int)((dy + halfy) * celly));
    int jz = std::min(c.ncell[2], 1 + (int)((dz + halfz) * cellz));
    int i = c.L(jx, jy, jz);
    while (i != j) i = clist[i];
    i = clist[i];
    while (i > 0) {
      dx = X(r, 0, i - 1) - rxj; dy = X(r, 1, i - 1) - ryj; dz = X(r, 2, i - 1) - rzj;
      dx = dx - boxx * nint(onboxx * dx);
      dy = dy - boxy * nint(onboxy * dy);
      dz = dz - boxz * nint(onboxz * dz);
      double drsq = dx * dx + dy * dy + dz * dz;
      if (drsq < rcutsq) {
        nlist = nlist + 1;
        if (nlist == maxnab * na) return GB_E_LIST;
        list[nlist] = i;
      }
      i = clist[i];
    }
    for (int k = 0; k < c.nn; ++k) {
      int ix = c.Mx(jx, c.ink[3 * k]), iy = c.My(jy, c.ink[3 * k + 1]), iz = c.Mz(jz, c.ink[3 * k + 2]);
      i = c.L(ix, iy, iz);
      while (i > 0) {
        dx = X(r, 0, i - 1) - rxj; dy = X(r, 1, i - 1) - ryj; dz = X(r, 2, i - 1) - rzj;
        dx = dx - boxx * nint(onboxx * dx);
        dy = dy - boxy * nint(onboxy * dy);
        dz = dz - boxz * nint(onboxz * dz);
        double drsq = dx * dx + dy * dy + dz * dz;
        if (drsq < rcutsq) {
          nlist = nlist + 1;
          if (nlist == maxnab * na) return GB_E_LIST;
          list[nlist] = i;
        }
        i = clist[i];
      }
    }
  }
  for (int i = jend + njump; i <= na + njump; i += njump) {
    nlist = nlist + 1;
    point[i] = nlist;
  }
  return GB_OK;
}
}  // namespace

// nei_driver (neigh_list.f90:1-21)
Status nei_driver(const double *r, int na, int *list, int *point, int njump, double rcut,
                  const double box[3]) {
  double boxmax = std::max(box[0], std::max(box[1], box[2]));
  if (3.0 * rcut > boxmax) return nei_list(r, na, list, point, njump, rcut, box);
  return nei_cell(r, na, list, point, njump, rcut, box);
}

// ===========================================================================
// Lennard-Jones O-O (ljones.f90)
// ===========================================================================
namespace {
struct LJAcc {
  double sigsq, rcutsq;
  double boxx, boxy, boxz, onboxx, onboxy, onboxz;
};

void lj_scale(double *dvdr, double &v, double vir[9], int na, int njump) {
  double vscale = 4.0 * P.oo_eps, dscale = 48.0 * P.oo_eps;
  v = vscale * v;
  for (int i = 0; i < 9; ++i) vir[i] = dscale * vir[i];
  for (int i = 1; i <= na; i += njump)
    for (int c = 0; c < 3; ++c) X(dvdr, c, i - 1) = dscale * X(dvdr, c, i - 1);
}

void lj_pair_ij(const double *r, double *dvdr, double &v, double vir[9], int i, int j,
                const LJAcc &a) {  // lj_basic / lj_cell form: dx = r(i) - r(j)
  double dx = X(r, 0, i - 1) - X(r, 0, j - 1);
  double dy = X(r, 1, i - 1) - X(r, 1, j - 1);
  double dz = X(r, 2, i - 1) - X(r, 2, j - 1);
  dx = dx - a.boxx * nint(a.onboxx * dx);
  dy = dy - a.boxy * nint(a.onboxy * dy);
  dz = dz - a.boxz * nint(a.onboxz * dz);
  double drsq = dx * dx + dy * dy + dz * dz;
  if (drsq < a.rcutsq) {
    double onr2 = 1.0 / drsq;
    double sr2 = a.sigsq * onr2;
    double sr6 = sr2 * sr2 * sr2;
    double vij = sr6 * (sr6 - 1.0);
    v = v + vij;
    double wij = sr6 * (sr6 - 0.5);
    double fij = wij * onr2;
    double dfx = fij * dx, dfy = fij * dy, dfz = fij * dz;
    X(dvdr, 0, i - 1) -= dfx; X(dvdr, 1, i - 1) -= dfy; X(dvdr, 2, i - 1) -= dfz;
    X(dvdr, 0, j - 1) += dfx; X(dvdr, 1, j - 1) += dfy; X(dvdr, 2, j - 1) += dfz;
    M33(vir, 0, 0) -= dx * dfx; M33(vir, 1, 1) -= dy * dfy; M33(vir, 2, 2) -= dz * dfz;
    M33(vir, 0, 1) -= dx * dfy; M33(vir, 0, 2) -= dx * dfz; M33(vir, 1, 0) -= dy * dfx;
    M33(vir, 1, 2) -= dy * dfz; M33(vir, 2, 0) -= dz * dfx; M33(vir, 2, 1) -= dz * dfy;
  }
}

void lj_basic(const double *r, double *dvdr, double &v, double vir[9], int na,
              const double box[3], int njump) {
  LJAcc a{P.oo_sig * P.oo_sig, P.rcut * P.rcut, box[0], box[1], box[2],
          1.0 / box[0], 1.0 / box[1], 1.0 / box[2]};
  v = 0.0;
  zero9(vir);
  std::memset(dvdr, 0, sizeof(double) * 3 * na);
  for (int j = 1 + njump; j <= na; j += njump)
    for (int i = 1; i <= j - njump; i += njump) lj_pair_ij(r, dvdr, v, vir, i, j, a);
  lj_scale(dvdr, v, vir, na, njump);
}

void lj_list(const double *r, double *dvdr, double &v, double vir[9], int na,
             const double box[3], const int *list, const int *point, int njump) {
  v = 0.0;
  zero9(vir);
  std::memset(dvdr, 0, sizeof(double) * 3 * na);
  double rcutsq = P.rcut * P.rcut;
  double boxx = box[0], boxy = box[1], boxz = box[2];
  double onboxx = 1.0 / boxx, onboxy = 1.0 / boxy, onboxz = 1.0 / boxz;
  double sigsq = P.oo_sig * P.oo_sig;
  for (int j = 1; j <= na; j += njump) {
    int ibeg = point[j], iend = point[j + njump] - 1;
    if (ibeg <= iend) {
      double rxj = X(r, 0, j - 1), ryj = X(r, 1, j - 1), rzj = X(r, 2, j - 1);
      double dvdxj = X(dvdr, 0, j - 1), dvdyj = X(dvdr, 1, j - 1), dvdzj = X(dvdr, 2, j - 1);
      for (int inab = ibeg; inab <= iend; ++inab) {
        int i = list[inab];
        double dx = X(r, 0, i - 1) - rxj, dy = X(r, 1, i - 1) - ryj, dz = X(r, 2, i - 1) - rzj;
        dx = dx - boxx * nint(onboxx * dx);
        dy = dy - boxy * nint(onboxy * dy);
        dz = dz - boxz * nint(onboxz * dz);
        double drsq = dx * dx + dy * dy + dz * dz;
        if (drsq < rcutsq) {
          double onr2 = 1.0 / drsq;
          double sr2 = sigsq * onr2;
          double sr6 = sr2 * sr2 * sr2;
          double vij = sr6 * (sr6 - 1.0);
          v = v + vij;
          double wij = sr6 * (sr6 - 0.5);
          double fij = wij * onr2;
          double dfx = fij * dx, dfy = fij * dy, dfz = fij * dz;
          X(dvdr, 0, i - 1) -= dfx; X(dvdr, 1, i - 1) -= dfy; X(dvdr, 2, i - 1) -= dfz;
          dvdxj = dvdxj + dfx; dvdyj = dvdyj + dfy; dvdzj = dvdzj + dfz;
          M33(vir, 0, 0) -= dx * dfx; M33(vir, 1, 1) -= dy * dfy; M33(vir, 2, 2) -= dz * dfz;
          M33(vir, 0, 1) -= dx * dfy; M33(vir, 0, 2) -= dx * dfz; M33(vir, 1, 0) -= dy * dfx;
          M33(vir, 1, 2) -= dy * dfz; M33(vir, 2, 0) -= dz * dfx; M33(vir, 2, 1) -= dz * dfy;
        }
      }
      X(dvdr, 0, j - 1) = dvdxj; X(dvdr, 1, j - 1) = dvdyj; X(dvdr, 2, j - 1) = dvdzj;
    }
  }
  lj_scale(dvdr, v, vir, na, njump);
}

void lj_cell(const double *r, double &v, double vir[9], double *dvdr, int na,
             const double box[3], int njump) {
  CellNC c;
  cell_setup(box, P.rcut, c);
  std::vector<int> list;
  cell_list(r, list, c, na, box, njump);
  LJAcc a{P.oo_sig * P.oo_sig, P.rcut * P.rcut, box[0], box[1], box[2],
          1.0 / box[0], 1.0 / box[1], 1.0 / box[2]};
  v = 0.0;
  zero9(vir);
  std::memset(dvdr, 0, sizeof(double) * 3 * na);
  for (int iz = 1; iz <= c.ncell[2]; ++iz)
    for (int iy = 1; iy <= c.ncell[1]; ++iy)
      for (int ix = 1; ix <= c.ncell[0]; ++ix) {
        int i = c.L(ix, iy, iz);
        while (i > 0) {
          int j = list[i];
          while (j > 0) {
            lj_pair_ij(r, dvdr, v, vir, i, j, a);
            j = list[j];
          }
          i = list[i];
        }
        for (int k = 0; k < c.nn; ++k) {
          int jx = c.Mx(ix, c.ink[3 * k]), jy = c.My(iy, c.ink[3 * k + 1]), jz = c.Mz(iz, c.ink[3 * k + 2]);
          i = c.L(ix, iy, iz);
          while (i > 0) {
            int j = c.L(jx, jy, jz);
            while (j > 0) {
              lj_pair_ij(r, dvdr, v, vir, i, j, a);
              j = list[j];
            }
            i = list[i];
          }
        }
      }
  lj_scale(dvdr, v, vir, na, njump);
}
}  // namespace

// lj_driver (ljones.f90:1-29)
void lj_driver(const double *r, double *dvdr, double &v, double vir[9], const int *list,
               const int *point, int na, const double box[3], int njump) {
  if (list[1] != 0) {
    lj_list(r, dvdr, v, vir, na, box, list, point, njump);
  } else {
    double boxmax = std::max(box[0], std::max(box[1], box[2]));
    if (3.0 * P.rcut > boxmax) lj_basic(r, dvdr, v, vir, na, box, njump);
    else lj_cell(r, v, vir, dvdr, na, box, njump);
  }
}

// ===========================================================================
// intramolecular potentials
// ===========================================================================
// intra_harmonic (intra_harmonic.f90:1-98): Toukan-Rahman SPC/F constants
void intra_harmonic(const double *r, double *dvdr, int na, double &v, double vir[9]) {
  const double apot = 0.5993, bpot = 0.1466, cpot = -0.09435, dpot = 0.04984;
  double rehh = 2.0 * std::sin(0.5 * P.theta) * P.reoh;
  v = 0.0;
  zero9(vir);
  for (int j = 0; j < na; j += 3) {
    double dx1 = X(r, 0, j + 1) - X(r, 0, j), dy1 = X(r, 1, j + 1) - X(r, 1, j),
           dz1 = X(r, 2, j + 1) - X(r, 2, j);
    double dr1 = std::sqrt(dx1 * dx1 + dy1 * dy1 + dz1 * dz1);
    double dr1dx1 = dx1 / dr1, dr1dy1 = dy1 / dr1, dr1dz1 = dz1 / dr1;
    dr1 = dr1 - P.reoh;
    double dx2 = X(r, 0, j + 2) - X(r, 0, j), dy2 = X(r, 1, j + 2) - X(r, 1, j),
           dz2 = X(r, 2, j + 2) - X(r, 2, j);
    double dr2 = std::sqrt(dx2 * dx2 + dy2 * dy2 + dz2 * dz2);
    double dr2dx2 = dx2 / dr2, dr2dy2 = dy2 / dr2, dr2dz2 = dz2 / dr2;
    dr2 = dr2 - P.reoh;
    double dx3 = X(r, 0, j + 2) - X(r, 0, j + 1), dy3 = X(r, 1, j + 2) - X(r, 1, j + 1),
           dz3 = X(r, 2, j + 2) - X(r, 2, j + 1);
    double dr3 = std::sqrt(dx3 * dx3 + dy3 * dy3 + dz3 * dz3);
    double dr3dx3 = dx3 / dr3, dr3dy3 = dy3 / dr3, dr3dz3 = dz3 / dr3;
    dr3 = dr3 - rehh;
    v = v + 0.5 * apot * (dr1 * dr1 + dr2 * dr2);
    v = v + 0.5 * bpot * dr3 * dr3;
    v = v + cpot * (dr1 + dr2) * dr3;
    v = v + dpot * dr1 * dr2;
    double dvdr1 = apot * dr1 + cpot * dr3 + dpot * dr2;
    double dvdr2 = apot * dr2 + cpot * dr3 + dpot * dr1;
    double dvdr3 = bpot * dr3 + cpot * (dr1 + dr2);
    double dvdx1 = dvdr1 * dr1dx1, dvdy1 = dvdr1 * dr1dy1, dvdz1 = dvdr1 * dr1dz1;
    double dvdx2 = dvdr2 * dr2dx2, dvdy2 = dvdr2 * dr2dy2, dvdz2 = dvdr2 * dr2dz2;
    double dvdx3 = dvdr3 * dr3dx3, dvdy3 = dvdr3 * dr3dy3, dvdz3 = dvdr3 * dr3dz3;
    X(dvdr, 0, j) = X(dvdr, 0, j) - dvdx1 - dvdx2;
    X(dvdr, 1, j) = X(dvdr, 1, j) - dvdy1 - dvdy2;
    X(dvdr, 2, j) = X(dvdr, 2, j) - dvdz1 - dvdz2;
    X(dvdr, 0, j + 1) = X(dvdr, 0, j + 1) + dvdx1 - dvdx3;
    X(dvdr, 1, j + 1) = X(dvdr, 1, j + 1) + dvdy1 - dvdy3;
    X(dvdr, 2, j + 1) = X(dvdr, 2, j + 1) + dvdz1 - dvdz3;
    X(dvdr, 0, j + 2) = X(dvdr, 0, j + 2) + dvdx2 + dvdx3;
    X(dvdr, 1, j + 2) = X(dvdr, 1, j + 2) + dvdy2 + dvdy3;
    X(dvdr, 2, j + 2) = X(dvdr, 2, j + 2) + dvdz2 + dvdz3;
    M33(vir, 0, 0) = M33(vir, 0, 0) + dx1 * dvdx1 + dx2 * dvdx2 + dx3 * dvdx3;
    M33(vir, 1, 1) = M33(vir, 1, 1) + dy1 * dvdy1 + dy2 * dvdy2 + dy3 * dvdy3;
    M33(vir, 2, 2) = M33(vir, 2, 2) + dz1 * dvdz1 + dz2 * dvdz2 + dz3 * dvdz3;
    M33(vir, 0, 1) = M33(vir, 0, 1) + dx1 * dvdy1 + dx2 * dvdy2 + dx3 * dvdy3;
    M33(vir, 0, 2) = M33(vir, 0, 2) + dx1 * dvdz1 + dx2 * dvdz2 + dx3 * dvdz3;
    M33(vir, 1, 2) = M33(vir, 1, 2) + dy1 * dvdz1 + dy2 * dvdz2 + dy3 * dvdz3;
    M33(vir, 2, 1) = M33(vir, 2, 1) + dz1 * dvdy1 + dz2 * dvdy2 + dz3 * dvdy3;
    M33(vir, 1, 0) = M33(vir, 1, 0) + dy1 * dvdx1 + dy2 * dvdx2 + dy3 * dvdx3;
    M33(vir, 2, 0) = M33(vir, 2, 0) + dz1 * dvdx1 + dz2 * dvdx2 + dz3 * dvdx3;
  }
}

namespace {
// bond/angle geometry shared by intra_spcfw and intra_morse_harm
struct Geo {
  double dx1, dy1, dz1, dx2, dy2, dz2, dx3, dy3, dz3;
  double dr1, dr2, dr1dx1, dr1dy1, dr1dz1, dr2dx2, dr2dy2, dr2dz2, dr3dx3, dr3dy3, dr3dz3;
  double dang, dthetadr1, dthetadr2, dthetadr3;
};
void geometry(const double *r, int j, Geo &g) {
  g.dx1 = X(r, 0, j + 1) - X(r, 0, j); g.dy1 = X(r, 1, j + 1) - X(r, 1, j); g.dz1 = X(r, 2, j + 1) - X(r, 2, j);
  double dr1sq = g.dx1 * g.dx1 + g.dy1 * g.dy1 + g.dz1 * g.dz1;
  double dr1 = std::sqrt(dr1sq), dr1a = dr1;
  g.dr1dx1 = g.dx1 / dr1; g.dr1dy1 = g.dy1 / dr1; g.dr1dz1 = g.dz1 / dr1;
  g.dr1 = dr1 - P.reoh;
  g.dx2 = X(r, 0, j + 2) - X(r, 0, j); g.dy2 = X(r, 1, j + 2) - X(r, 1, j); g.dz2 = X(r, 2, j + 2) - X(r, 2, j);
  double dr2sq = g.dx2 * g.dx2 + g.dy2 * g.dy2 + g.dz2 * g.dz2;
  double dr2 = std::sqrt(dr2sq), dr2a = dr2;
  g.dr2dx2 = g.dx2 / dr2; g.dr2dy2 = g.dy2 / dr2; g.dr2dz2 = g.dz2 / dr2;
  g.dr2 = dr2 - P.reoh;
  g.dx3 = X(r, 0, j + 2) - X(r, 0, j + 1); g.dy3 = X(r, 1, j + 2) - X(r, 1, j + 1); g.dz3 = X(r, 2, j + 2) - X(r, 2, j + 1);
  double dr3sq = g.dx3 * g.dx3 + g.dy3 * g.dy3 + g.dz3 * g.dz3;
  double dr3 = std::sqrt(dr3sq), dr3a = dr3;
  g.dr3dx3 = g.dx3 / dr3; g.dr3dy3 = g.dy3 / dr3; g.dr3dz3 = g.dz3 / dr3;
  double u = (dr1sq + dr2sq - dr3sq);
  double vv = (2.0 * dr1a * dr2a);
  double v2 = 1.0 / (vv * vv);
  double arg = u / vv;
  double darg = -1.0 / std::sqrt(1.0 - arg * arg);
  double ang = std::acos(arg);
  g.dang = (ang - P.theta);
  double uprime = 2.0 * dr1a, vprime = 2.0 * dr2a;
  double grad = (uprime * vv - vprime * u) * v2;
  g.dthetadr1 = darg * grad;
  uprime = 2.0 * dr2a;
  vprime = 2.0 * dr1a;
  grad = (uprime * vv - vprime * u) * v2;
  g.dthetadr2 = darg * grad;
  uprime = -2.0 * dr3a;
  grad = (uprime * vv) * v2;
  g.dthetadr3 = darg * grad;
}
}  // namespace

// intra_spcfw (intra_spcfw.f90:1-125), virial W = sum r_i . dvdr_i, diagonal only
void intra_spcfw(const double *r, double *dvdr, int na, double &v, double vir[9]) {
  v = 0.0;
  zero9(vir);
  for (int j = 0; j < na; j += 3) {
    Geo g;
    geometry(r, j, g);
    v = v + 0.5 * P.apot * (g.dr1 * g.dr1 + g.dr2 * g.dr2);
    v = v + 0.5 * P.bpot * (g.dang * g.dang);
    double dvdr1 = P.apot * g.dr1 + P.bpot * g.dang * g.dthetadr1;
    double dvdr2 = P.apot * g.dr2 + P.bpot * g.dang * g.dthetadr2;
    double dvdr3 = P.bpot * g.dang * g.dthetadr3;
    double dvdx1 = dvdr1 * g.dr1dx1, dvdy1 = dvdr1 * g.dr1dy1, dvdz1 = dvdr1 * g.dr1dz1;
    double dvdx2 = dvdr2 * g.dr2dx2, dvdy2 = dvdr2 * g.dr2dy2, dvdz2 = dvdr2 * g.dr2dz2;
    double dvdx3 = dvdr3 * g.dr3dx3, dvdy3 = dvdr3 * g.dr3dy3, dvdz3 = dvdr3 * g.dr3dz3;
    X(dvdr, 0, j) = X(dvdr, 0, j) - dvdx1 - dvdx2;
    X(dvdr, 1, j) = X(dvdr, 1, j) - dvdy1 - dvdy2;
    X(dvdr, 2, j) = X(dvdr, 2, j) - dvdz1 - dvdz2;
    X(dvdr, 0, j + 1) = X(dvdr, 0, j + 1) + dvdx1 - dvdx3;
    X(dvdr, 1, j + 1) = X(dvdr, 1, j + 1) + dvdy1 - dvdy3;
    X(dvdr, 2, j + 1) = X(dvdr, 2, j + 1) + dvdz1 - dvdz3;
    X(dvdr, 0, j + 2) = X(dvdr, 0, j + 2) + dvdx2 + dvdx3;
    X(dvdr, 1, j + 2) = X(dvdr, 1, j + 2) + dvdy2 + dvdy3;
    X(dvdr, 2, j + 2) = X(dvdr, 2, j + 2) + dvdz2 + dvdz3;
    M33(vir, 0, 0) = M33(vir, 0, 0) + X(r, 0, j) * (-dvdx1 - dvdx2) +
                     X(r, 0, j + 1) * (+dvdx1 - dvdx3) + X(r, 0, j + 2) * (+dvdx2 + dvdx3);
    M33(vir, 1, 1) = M33(vir, 1, 1) + X(r, 1, j) * (-dvdy1 - dvdy2) +
                     X(r, 1, j + 1) * (+dvdy1 - dvdy3) + X(r, 1, j + 2) * (+dvdy2 + dvdy3);
    M33(vir, 2, 2) = M33(vir, 2, 2) + X(r, 2, j) * (-dvdz1 - dvdz2) +
                     X(r, 2, j + 1) * (+dvdz1 - dvdz3) + X(r, 2, j + 2) * (+dvdz2 + dvdz3);
  }
}

// intra_morse_harm (intra_morse_harm.f90:1-143): quartic Morse stretch, harmonic bend
void intra_morse_harm(const double *r, double *dvdr, int na, double &v, double vir[9]) {
  double de = P.apot, deb = P.bpot, alp = P.alp;
  double alp2 = alp * alp, alp3 = alp * alp2, alp4 = alp3 * alp;
  double f1 = 7.0 / 12.0, f2 = 7.0 / 3.0;
  v = 0.0;
  zero9(vir);
  for (int j = 0; j < na; j += 3) {
    Geo g;
    geometry(r, j, g);
    double dr1 = g.dr1, dr2 = g.dr2, drasq = dr1 * dr1, drbsq = dr2 * dr2;
    v = v + de * (alp2 * drasq - alp3 * dr1 * drasq + f1 * alp4 * drasq * drasq);
    v = v + de * (alp2 * drbsq - alp3 * dr2 * drbsq + f1 * alp4 * drbsq * drbsq);
    v = v + deb * (g.dang * g.dang);
    double a1 = de * (2.0 * alp2 * dr1 - 3.0 * alp3 * drasq + f2 * alp4 * dr1 * drasq);
    double a2 = de * (2.0 * alp2 * dr2 - 3.0 * alp3 * drbsq + f2 * alp4 * dr2 * drbsq);
    double a3 = 2.0 * deb * g.dang;
    double dvdr1 = a1 + a3 * g.dthetadr1;
    double dvdr2 = a2 + a3 * g.dthetadr2;
    double dvdr3 = a3 * g.dthetadr3;
    double dvdx1 = dvdr1 * g.dr1dx1, dvdy1 = dvdr1 * g.dr1dy1, dvdz1 = dvdr1 * g.dr1dz1;
    double dvdx2 = dvdr2 * g.dr2dx2, dvdy2 = dvdr2 * g.dr2dy2, dvdz2 = dvdr2 * g.dr2dz2;
    double dvdx3 = dvdr3 * g.dr3dx3, dvdy3 = dvdr3 * g.dr3dy3, dvdz3 = dvdr3 * g.dr3dz3;
    X(dvdr, 0, j) = X(dvdr, 0, j) - dvdx1 - dvdx2;
    X(dvdr, 1, j) = X(dvdr, 1, j) - dvdy1 - dvdy2;
    X(dvdr, 2, j) = X(dvdr, 2, j) - dvdz1 - dvdz2;
    X(dvdr, 0, j + 1) = X(dvdr, 0, j + 1) + dvdx1 - dvdx3;
    X(dvdr, 1, j + 1) = X(dvdr, 1, j + 1) + dvdy1 - dvdy3;
    X(dvdr, 2, j + 1) = X(dvdr, 2, j + 1) + dvdz1 - dvdz3;
    X(dvdr, 0, j + 2) = X(dvdr, 0, j + 2) + dvdx2 + dvdx3;
    X(dvdr, 1, j + 2) = X(dvdr, 1, j + 2) + dvdy2 + dvdy3;
    X(dvdr, 2, j + 2) = X(dvdr, 2, j + 2) + dvdz2 + dvdz3;
    double xx = g.dx1 * dvdx1 + g.dx2 * dvdx2 + g.dx3 * dvdx3;
    double xy = g.dx1 * dvdy1 + g.dx2 * dvdy2 + g.dx3 * dvdy3;
    double xz = g.dx1 * dvdz1 + g.dx2 * dvdz2 + g.dx3 * dvdz3;
    double yy = g.dy1 * dvdy1 + g.dy2 * dvdy2 + g.dy3 * dvdy3;
    double yz = g.dy1 * dvdz1 + g.dy2 * dvdz2 + g.dy3 * dvdz3;
    double zz = g.dz1 * dvdz1 + g.dz2 * dvdz2 + g.dz3 * dvdz3;
    M33(vir, 0, 0) += xx; M33(vir, 0, 1) += xy; M33(vir, 0, 2) += xz;
    M33(vir, 1, 0) += xy; M33(vir, 1, 1) += yy; M33(vir, 1, 2) += yz;
    M33(vir, 2, 0) += xz; M33(vir, 2, 1) += yz; M33(vir, 2, 2) += zz;
  }
}

// ===========================================================================
// TEM-switched short-range Coulomb correction (correct_tem.f90)
// ===========================================================================
namespace {
struct Tem {
  double rcutsq, a1, a2, a3, boxx, boxy, boxz, onboxx, onboxy, onboxz;
  Tem(const double box[3]) {
    double sig = P.sig;
    rcutsq = sig * sig;
    a1 = 2.0 / sig;
    a2 = 2.0 / std::pow(sig, 3);
    a3 = 1.0 / std::pow(sig, 4);
    boxx = box[0]; boxy = box[1]; boxz = box[2];
    onboxx = 1.0 / boxx; onboxy = 1.0 / boxy; onboxz = 1.0 / boxz;
  }
};

// one TEM pair, basic/cell form (dx = r(i) - r(j)), i,j 1-based
inline void tem_pair(const double *r, const double *z, double *dvdr, double &v, double vir[9],
                     int i, int j, const Tem &t) {
  double dx = X(r, 0, i - 1) - X(r, 0, j - 1);
  double dy = X(r, 1, i - 1) - X(r, 1, j - 1);
  double dz = X(r, 2, i - 1) - X(r, 2, j - 1);
  dx = dx - t.boxx * nint(t.onboxx * dx);
  dy = dy - t.boxy * nint(t.onboxy * dy);
  dz = dz - t.boxz * nint(t.onboxz * dz);
  double drsq = dx * dx + dy * dy + dz * dz;
  if (drsq < t.rcutsq) {
    double dr = std::sqrt(drsq);
    double onr = 1.0 / dr;
    double zij = z[i - 1] * z[j - 1];
    double vc = zij * onr;
    double dvc = -vc * onr;
    double dr3 = drsq * dr, dr4 = dr3 * dr;
    double f = 1.0 - t.a1 * dr + t.a2 * dr3 - t.a3 * dr4;
    double df = -t.a1 + 3.0 * t.a2 * drsq - 4.0 * t.a3 * dr3;
    double dv = vc * f;
    double dvr = vc * df + dvc * f;
    double dvx = dvr * dx * onr, dvy = dvr * dy * onr, dvz = dvr * dz * onr;
    v = v + dv;
    X(dvdr, 0, i - 1) += dvx; X(dvdr, 1, i - 1) += dvy; X(dvdr, 2, i - 1) += dvz;
    X(dvdr, 0, j - 1) -= dvx; X(dvdr, 1, j - 1) -= dvy; X(dvdr, 2, j - 1) -= dvz;
    M33(vir, 0, 0) += dx * dvx; M33(vir, 1, 1) += dy * dvy; M33(vir, 2, 2) += dz * dvz;
    M33(vir, 0, 1) += dx * dvy; M33(vir, 0, 2) += dx * dvz; M33(vir, 1, 0) += dy * dvx;
    M33(vir, 1, 2) += dy * dvz; M33(vir, 2, 0) += dz * dvx; M33(vir, 2, 1) += dz * dvy;
  }
}

Status ewc_basic_tem(const double *r, const double *z, double *dvdr, double &v, double vir[9],
                     int na, const double box[3]) {
  Tem t(box);
  double boxmin = std::max(box[0], std::max(box[1], box[2]));  // sic: max (correct_tem.f90:104)
  if (P.sig > 0.5 * boxmin) return GB_E_CUTOFF;
  v = 0.0;
  zero9(vir);
  std::memset(dvdr, 0, sizeof(double) * 3 * na);
  for (int j = 1; j <= na; ++j)
    for (int i = 1; i <= j - 1; ++i)
      if ((i - 1) / 3 != (j - 1) / 3) tem_pair(r, z, dvdr, v, vir, i, j, t);
  return GB_OK;
}

Status ewc_list_tem(const double *r, const double *z, double *dvdr, double &v, double vir[9],
                    int na, const double box[3], const int *list, const int *point) {
  Tem t(box);
  double boxmax = std::max(box[0], std::max(box[1], box[2]));
  if (P.sig > 0.5 * boxmax) return GB_E_CUTOFF;
  v = 0.0;
  zero9(vir);
  std::memset(dvdr, 0, sizeof(double) * 3 * na);
  for (int j = 1; j <= na; ++j) {
    int ibeg = point[j], iend = point[j + 1] - 1;
    if (ibeg <= iend) {
      double rxj = X(r, 0, j - 1), ryj = X(r, 1, j - 1), rzj = X(r, 2, j - 1);
      double dvdxj = X(dvdr, 0, j - 1), dvdyj = X(dvdr, 1, j - 1), dvdzj = X(dvdr, 2, j - 1);
      for (int inab = ibeg; inab <= iend; ++inab) {
        int i = list[inab];
        if ((i - 1) / 3 != (j - 1) / 3) {
          double dx = X(r, 0, i - 1) - rxj, dy = X(r, 1, i - 1) - ryj, dz = X(r, 2, i - 1) - rzj;
          dx = dx - t.boxx * nint(t.onboxx * dx);
          dy = dy - t.boxy * nint(t.onboxy * dy);
          dz = dz - t.boxz * nint(t.onboxz * dz);
          double drsq = dx * dx + dy * dy + dz * dz;
          if (drsq < t.rcutsq) {
            double dr = std::sqrt(drsq);
            double onr = 1.0 / dr;
            double zij = z[i - 1] * z[j - 1];
            double vc = zij * onr;
            double dvc = -vc * onr;
            double dr3 = drsq * dr, dr4 = dr3 * dr;
            double f = 1.0 - t.a1 * dr + t.a2 * dr3 - t.a3 * dr4;
            double df = -t.a1 + 3.0 * t.a2 * drsq - 4.0 * t.a3 * dr3;
            double dv = vc * f;
            double dvr = vc * df + dvc * f;
            double dvx = dvr * dx * onr, dvy = dvr * dy * onr, dvz = dvr * dz * onr;
            v = v + dv;
            X(dvdr, 0, i - 1) += dvx; X(dvdr, 1, i - 1) += dvy; X(dvdr, 2, i - 1) += dvz;
            dvdxj = dvdxj - dvx; dvdyj = dvdyj - dvy; dvdzj = dvdzj - dvz;
            M33(vir, 0, 0) += dx * dvx; M33(vir, 1, 1) += dy * dvy; M33(vir, 2, 2) += dz * dvz;
            M33(vir, 0, 1) += dx * dvy; M33(vir, 0, 2) += dx * dvz; M33(vir, 1, 0) += dy * dvx;
            M33(vir, 1, 2) += dy * dvz; M33(vir, 2, 0) += dz * dvx; M33(vir, 2, 1) += dz * dvy;
          }
        }
      }
      X(dvdr, 0, j - 1) = dvdxj; X(dvdr, 1, j - 1) = dvdyj; X(dvdr, 2, j - 1) = dvdzj;
    }
  }
  return GB_OK;
}

Status ewc_cell_tem(const double *r, const double *z, double *dvdr, double &v, double vir[9],
                    int na, const double box[3]) {
  CellNC c;
  cell_setup(box, P.sig, c);
  std::vector<int> list;
  cell_list(r, list, c, na, box, 1);
  Tem t(box);
  double boxmin = std::min(box[0], std::min(box[1], box[2]));
  if (P.sig > 0.5 * boxmin) return GB_E_CUTOFF;
  v = 0.0;
  zero9(vir);
  std::memset(dvdr, 0, sizeof(double) * 3 * na);
  for (int iz = 1; iz <= c.ncell[2]; ++iz)
    for (int iy = 1; iy <= c.ncell[1]; ++iy)
      for (int ix = 1; ix <= c.ncell[0]; ++ix) {
        int i = c.L(ix, iy, iz);
        while (i > 0) {
          int j = list[i];
          while (j > 0) {
            if ((i - 1) / 3 != (j - 1) / 3) tem_pair(r, z, dvdr, v, vir, i, j, t);
            j = list[j];
          }
          i = list[i];
        }
      }
  for (int k = 0; k < c.nn; ++k) {
    int incx = c.ink[3 * k], incy = c.ink[3 * k + 1], incz = c.ink[3 * k + 2];
    for (int iz = 1; iz <= c.ncell[2]; ++iz) {
      int jz = c.Mz(iz, incz);
      for (int iy = 1; iy <= c.ncell[1]; ++iy) {
        int jy = c.My(iy, incy);
        for (int ix = 1; ix <= c.ncell[0]; ++ix) {
          int jx = c.Mx(ix, incx);
          int i = c.L(ix, iy, iz);
          while (i > 0) {
            int j = c.L(jx, jy, jz);
            while (j > 0) {
              if ((i - 1) / 3 != (j - 1) / 3) tem_pair(r, z, dvdr, v, vir, i, j, t);
              j = list[j];
            }
            i = list[i];
          }
        }
      }
    }
  }
  return GB_OK;
}
}  // namespace

// ewc_driver_tem (correct_tem.f90:1-71)
Status ewc_driver_tem(double *r, const double *z, double *dvdr, double &v, double vir[9],
                      int na, const double box[3], const int *list, const int *point) {
  if (P.wm > 0.0 || P.wh > 0.0) return GB_E_UNSUPPORTED;
  double alpha = P.alpha;
  double alpha2 = 0.5 * (1.0 - alpha);
  const bool msite = std::fabs(alpha - 1.0) > 1e-4;
  std::vector<double> ro;
  if (msite) {
    ro.resize(na);
    for (int i = 0, ic = 0; i < na; i += 3, ++ic)
      for (int j = 0; j < 3; ++j) {
        ro[3 * ic + j] = X(r, j, i);
        X(r, j, i) = alpha * X(r, j, i) + alpha2 * (X(r, j, i + 1) + X(r, j, i + 2));
      }
  }
  Status st;
  if (list[1] != 0) {
    st = ewc_list_tem(r, z, dvdr, v, vir, na, box, list, point);
  } else {
    double boxmax = std::max(box[0], std::max(box[1], box[2]));
    if (3.0 * P.sig > boxmax) st = ewc_basic_tem(r, z, dvdr, v, vir, na, box);
    else st = ewc_cell_tem(r, z, dvdr, v, vir, na, box);
  }
  if (msite) {
    for (int j = 0, ic = 0; j < na; j += 3, ++ic)
      for (int i = 0; i < 3; ++i) {
        X(dvdr, i, j + 1) += alpha2 * X(dvdr, i, j);
        X(dvdr, i, j + 2) += alpha2 * X(dvdr, i, j);
        X(dvdr, i, j) = alpha * X(dvdr, i, j);
        X(r, i, j) = ro[3 * ic + i];
      }
  }
  return st;
}

// ===========================================================================
// potenl_opt / forces / full_forces (md_forces.f90)
// ===========================================================================
Status potenl_opt(double *r, double &v, double *dvdr, double vir[9], int na, int nb,
                  const double box[3], const double *z, const int *list, const int *point,
                  int iopt) {
  (void)nb;
  v = 0.0;
  std::memset(dvdr, 0, sizeof(double) * 3 * na);
  zero9(vir);
  int nm = na / 3;
  if (3 * nm != na) return GB_E_ARG;
  if (iopt <= 2) {
    if (P.wm > 0.0 || P.wh > 0.0) return GB_E_UNSUPPORTED;  // rwald_smeared (ewald_smeared.f90)
    double alpha = P.alpha;
    double alpha2 = 0.5 * (1.0 - alpha);
    std::vector<int> mol(na);
    for (int j = 0; j < na; ++j) mol[j] = j / 3 + 1;
    std::vector<double> ro(3 * (size_t)nm);
    for (int i = 0, ic = 0; i < na; i += 3, ++ic)
      for (int j = 0; j < 3; ++j) {
        ro[3 * ic + j] = X(r, j, i);
        X(r, j, i) = alpha * X(r, j, i) + alpha2 * (X(r, j, i + 1) + X(r, j, i + 2));
      }
    double vew, vir_ew[9];
    if (P.iamcub) ewald_cubic(na, mol.data(), z, r, vew, vir_ew, dvdr, box[0]);
    else ewald_nc(na, mol.data(), z, r, vew, vir_ew, dvdr, box);  // md_forces.f90:192-197
    v = v + vew;
    for (int i = 0; i < 9; ++i) vir[i] += vir_ew[i];
    for (int j = 0, ic = 0; j < na; j += 3, ++ic)
      for (int i = 0; i < 3; ++i) {
        X(dvdr, i, j + 1) += alpha2 * X(dvdr, i, j);
        X(dvdr, i, j + 2) += alpha2 * X(dvdr, i, j);
        X(dvdr, i, j) = alpha * X(dvdr, i, j);
        X(r, i, j) = ro[3 * ic + i];
      }
  }
  if (iopt == 0 || iopt == 1 || iopt == 3) {
    if (P.oo_gam != 0.0) return GB_E_UNSUPPORTED;  // buckingham.f90
    std::vector<double> dvdroo(3 * (size_t)na);
    double voo, vir_oo[9];
    lj_driver(r, dvdroo.data(), voo, vir_oo, list, point, na, box, 3);
    for (size_t i = 0; i < 3 * (size_t)na; ++i) dvdr[i] += dvdroo[i];
    v = v + voo;
    for (int i = 0; i < 9; ++i) vir[i] += vir_oo[i];
  }
  if (iopt == 0 || iopt == 4) {
    double vint, vir_int[9];
    if (P.intra_model == GB_INTRA_SPCFW) {
      intra_spcfw(r, dvdr, na, vint, vir_int);
    } else if (P.alp == 0.0) {
      intra_harmonic(r, dvdr, na, vint, vir_int);
    } else if (P.alpb != 0.0) {
      return GB_E_UNSUPPORTED;  // intra_morse (intra_morse.f90)
    } else {
      intra_morse_harm(r, dvdr, na, vint, vir_int);
    }
    v = v + vint;
    for (int i = 0; i < 9; ++i) vir[i] += vir_int[i];
  }
  return GB_OK;
}

Status forces(double *r, double &v, double *dvdr, int nb, int na, const double box[3],
              const double *z, double virial[9], int iopt) {
  std::vector<int> point(na + 4, 0), list((size_t)maxnab * na + 1, 0);
  const double rgmax = 5.0;
  v = 0.0;
  std::memset(dvdr, 0, sizeof(double) * 3 * (size_t)na * nb);
  double vir[9];
  zero9(vir);
  zero9(virial);
  Status st = GB_OK;
  double boxmin = std::min(box[0], std::min(box[1], box[2]));
  auto centroid = [&](std::vector<double> &rc) {
    rc.assign(3 * (size_t)na, 0.0);
    for (int j = 0; j < nb; ++j)
      for (size_t i = 0; i < 3 * (size_t)na; ++i) rc[i] = rc[i] + r[i + 3 * (size_t)na * j];
    for (size_t i = 0; i < 3 * (size_t)na; ++i) rc[i] = rc[i] / (double)nb;
  };
  if (iopt == 3 || iopt <= 1) {
    if (nb > 3) {
      std::vector<double> rc;
      centroid(rc);
      double cut = std::min(P.rcut, 0.5 * boxmin);
      st = nei_driver(rc.data(), na, list.data(), point.data(), 3, cut, box);
      if (st) return st;
    } else {
      list[1] = 0;
    }
  }
  if (iopt != 5) {
    for (int k = 0; k < nb; ++k) {
      double dv;
      st = potenl_opt(r + 3 * (size_t)na * k, dv, dvdr + 3 * (size_t)na * k, vir, na, nb, box, z,
                      list.data(), point.data(), iopt);
      if (st) return st;
      v = v + dv;
      for (int i = 0; i < 9; ++i) virial[i] += vir[i];
    }
  } else {
    if (nb > 1) {
      std::vector<double> rc;
      centroid(rc);
      double cut = P.sig + rgmax;
      if (cut > 0.5 * boxmin) cut = std::min(cut, 0.5 * boxmin);
      st = nei_driver(rc.data(), na, list.data(), point.data(), 1, cut, box);
      if (st) return st;
    } else {
      list[1] = 0;
    }
    for (int k = 0; k < nb; ++k) {
      double dv;
      st = ewc_driver_tem(r + 3 * (size_t)na * k, z, dvdr + 3 * (size_t)na * k, dv, vir, na, box,
                          list.data(), point.data());
      if (st) return st;
      v = v + dv;
      for (int i = 0; i < 9; ++i) virial[i] += vir[i];
    }
  }
  v = v / (double)nb;
  for (int i = 0; i < 9; ++i) virial[i] = virial[i] / (double)nb;
  return GB_OK;
}

Status full_forces(double *r, int na, int nb, double &v, double &vew, double &voo,
                   double &vint, double vir[9], const double *z, const double box[3],
                   double *dvdr, double *dvdr2) {
  const size_t N = 3 * (size_t)na * nb;
  std::vector<double> dvdre(N, 0.0), dvdrl(N, 0.0);
  vew = voo = vint = 0.0;
  std::memset(dvdr, 0, sizeof(double) * N);
  double vir_itr[9], vir_oo[9], vir_ew[9], vir_ewc[9];
  zero9(vir); zero9(vir_itr); zero9(vir_oo); zero9(vir_ew);
  double ve = 0.0;
  Status st = forces(r, vint, dvdr2, nb, na, box, z, vir_itr, 4);
  if (st) return st;
  const int nbdf1 = P.nbdf1, nbdf2 = P.nbdf2;
  if (nb > 1) {
    if (nbdf1 > 0 || nbdf2 > 0) {
      realft(r, 3 * na, nb, +1);
      if (nbdf1 > 0) {
        st = rp_contract_nm(r, vew, dvdr, nb, na, box, z, vir_ew, nbdf1, 2);
        if (st) return st;
        if (P.sig > 0.0) {
          st = rp_contract_nm(r, ve, dvdre.data(), nb, na, box, z, vir_ewc, nbdf1, 5);
          if (st) return st;
          vew = vew - ve;
          for (int i = 0; i < 9; ++i) vir_ew[i] -= vir_ewc[i];
          for (size_t i = 0; i < N; ++i) dvdr[i] -= dvdre[i];
        }
      }
      if (nbdf2 > 0) {
        st = rp_contract_nm(r, voo, dvdrl.data(), nb, na, box, z, vir_oo, nbdf2, 3);
        if (st) return st;
      }
      realft(r, 3 * na, nb, -1);
    }
    if (nbdf1 > 0 && nbdf2 > 0) {
      for (size_t i = 0; i < N; ++i) dvdr[i] += dvdrl[i];
      realft(dvdr, 3 * na, nb, -1);
    } else if (nbdf1 > 0) {
      realft(dvdr, 3 * na, nb, -1);
    } else if (nbdf2 > 0) {
      realft(dvdrl.data(), 3 * na, nb, -1);
    }
  }
  if (nb == 1 || nbdf1 == 0) {
    st = forces(r, vew, dvdr, nb, na, box, z, vir_ew, 2);
    if (st) return st;
  } else if (P.sig > 0.0) {
    st = forces(r, ve, dvdre.data(), nb, na, box, z, vir_ewc, 5);
    if (st) return st;
    vew = vew + ve;
    for (int i = 0; i < 9; ++i) vir_ew[i] += vir_ewc[i];
    for (size_t i = 0; i < N; ++i) dvdr[i] += dvdre[i];
  }
  if (nb == 1 || nbdf2 == 0) {
    st = forces(r, voo, dvdrl.data(), nb, na, box, z, vir_oo, 3);
    if (st) return st;
  }
  if (nb == 1 || nbdf1 <= 0 || nbdf2 <= 0)
    for (size_t i = 0; i < N; ++i) dvdr[i] += dvdrl[i];
  v = vew + voo + vint;
  for (int i = 0; i < 9; ++i) vir[i] = vir_oo[i] + vir_ew[i] + vir_itr[i];
  return GB_OK;
}

}  // namespace orc
