// io.cpp -- the reference's on-disk formats for restarts and trajectories
// (io.f90), host-side: a driver that replaces main.f90's loop around the
// library reads and writes the same files.
//
//   print_structure (io.f90:1-17): "nm na nb", the three box lengths, then
//     r(:,:,:) in Fortran order, all list-directed; read back by main.f90 with
//     list-directed reads, so any whitespace layout is equivalent.
//   print_vmd_full / _forces / _vels (io.f90:310-547) and print_vmd_bead /
//     _forces / _vels (io.f90:549-770): an xyz frame -- the atom count, a
//     "BOX" line in Angstrom, one "<element> x y z" line per atom -- of the
//     bead-averaged (centroid) or one bead's positions (Angstrom, each oxygen
//     moved into the box by L (nint(x / L) - 1/2) and its hydrogens with it,
//     unless reftraj), forces -(dvdr + dvdr2) or velocities p / m (atomic units).
// Numbers are written with 17 significant digits (exact round trip), in
// gfortran's list-directed style: fixed notation for 0.1 <= |x| < 1e16, else
// an E exponent of three digits.
#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gbrpmd.h"

int ctx_set_error(int code, const std::string &msg);

namespace {

const double TOA = 0.5291772108;  // bohr -> Angstrom (globals.inc:12)

std::string fnum(double x) {
  char buf[64];
  const double a = std::fabs(x);
  if (a == 0.0) {
    std::snprintf(buf, sizeof buf, "%25.17f", 0.0);
  } else if (a >= 0.1 && a < 1e16) {
    const int ip = (int)std::floor(std::log10(a)) + 1;  // digits before the point
    std::snprintf(buf, sizeof buf, "%25.*f", std::max(0, 17 - ip), x);
  } else {
    char t[48];
    std::snprintf(t, sizeof t, "%.16E", x);  // correctly rounded mantissa, then a 3-digit exponent
    char *E = std::strchr(t, 'E');
    const int e = std::atoi(E + 1);
    *E = '\0';
    std::snprintf(buf, sizeof buf, "%21sE%c%03d", t, e < 0 ? '-' : '+', std::abs(e));
  }
  return buf;
}

FILE *open_out(const char *path, int append) { return std::fopen(path, append ? "a" : "w"); }

// whitespace-separated numbers of a list-directed file; Fortran D exponents accepted
bool read_numbers(const char *path, std::vector<double> &out, size_t want) {
  FILE *f = std::fopen(path, "r");
  if (!f) return false;
  char tok[128];
  while (out.size() < want && std::fscanf(f, "%127s", tok) == 1) {
    for (char *q = tok; *q; ++q)
      if (*q == 'D' || *q == 'd') *q = 'E';
    char *end = nullptr;
    errno = 0;
    const double v = std::strtod(tok, &end);
    if (end == tok || *end != '\0' || errno == ERANGE) {
      std::fclose(f);
      return false;
    }
    out.push_back(v);
  }
  std::fclose(f);
  return out.size() == want;
}

}  // namespace

extern "C" {

int gbrpmd_write_structure(const char *path, int append, const double *r, const double *box, int nm, int na,
                           int nb) {
  if (!path || !r || !box || nm < 0 || na < 0 || nb < 1) return ctx_set_error(GB_E_ARG, "bad argument");
  FILE *f = open_out(path, append);
  if (!f) return ctx_set_error(GB_E_ARG, std::string("cannot open ") + path);
  std::fprintf(f, " %11d %11d %11d\n", nm, na, nb);
  std::fprintf(f, "%s%s%s\n", fnum(box[0]).c_str(), fnum(box[1]).c_str(), fnum(box[2]).c_str());
  const size_t n = 3 * (size_t)na * nb;
  for (size_t i = 0; i < n; ++i) std::fprintf(f, "%s%s", fnum(r[i]).c_str(), (i % 4 == 3 || i + 1 == n) ? "\n" : "");
  const bool ok = std::fclose(f) == 0;
  return ok ? GB_OK : ctx_set_error(GB_E_ARG, std::string("write failed: ") + path);
}

// Reads a restart file of print_structure.  With r == NULL only the header is
// read (nm, na, nb, box), so that the caller can size r (3 na nb doubles).
int gbrpmd_read_structure(const char *path, int *nm, int *na, int *nb, double *box, double *r) {
  if (!path || !nm || !na || !nb || !box) return ctx_set_error(GB_E_ARG, "null argument");
  std::vector<double> v;
  if (!read_numbers(path, v, 6)) return ctx_set_error(GB_E_ARG, std::string("cannot read the header of ") + path);
  *nm = (int)v[0];
  *na = (int)v[1];
  *nb = (int)v[2];
  if (*nm < 0 || *na != 3 * *nm || *nb < 1) return ctx_set_error(GB_E_ARG, "inconsistent nm, na, nb in the header");
  for (int d = 0; d < 3; ++d) box[d] = v[3 + d];
  if (!r) return GB_OK;
  const size_t n = 3 * (size_t)(*na) * (*nb);
  v.clear();
  if (!read_numbers(path, v, 6 + n)) return ctx_set_error(GB_E_ARG, std::string("short restart file: ") + path);
  std::memcpy(r, v.data() + 6, sizeof(double) * n);
  return GB_OK;
}

// One xyz frame of print_vmd_*: kind 0 positions a = r, 1 forces -(a + a2)
// with a = dvdr, a2 = dvdr2, 2 velocities a / mass with a = p; bead 0 takes
// the bead average (print_vmd_full*), bead k = 1..nb that bead
// (print_vmd_bead*); isotope 0 H2O, 1 D2O, 2 HDO (element labels); reftraj
// nonzero leaves positions unwrapped.
int gbrpmd_write_vmd(const char *path, int append, int kind, int bead, const double *a, const double *a2,
                     const double *mass, const double *box, int na, int nb, int isotope, int reftraj) {
  if (!path || !a || !box || na <= 0 || na % 3 || nb < 1 || bead < 0 || bead > nb || kind < 0 || kind > 2)
    return ctx_set_error(GB_E_ARG, "bad argument");
  if (kind == 1 && !a2) return ctx_set_error(GB_E_ARG, "forces need dvdr and dvdr2");
  if (kind == 2 && !mass) return ctx_set_error(GB_E_ARG, "velocities need the masses");
  std::vector<double> c(3 * (size_t)na, 0.0);
  const size_t S = 3 * (size_t)na;
  auto val = [&](size_t o, int i) {  // the per-bead quantity at flat index o of atom i
    if (kind == 0) return a[o];
    if (kind == 1) return a[o] + a2[o];
    return a[o] / mass[i];
  };
  for (int i = 0; i < na; ++i)
    for (int j = 0; j < 3; ++j) {
      const size_t o = (size_t)j + 3 * (size_t)i;
      if (bead > 0) {
        c[o] = val(o + S * (bead - 1), i);
      } else {
        double s = 0.0;
        for (int k = 0; k < nb; ++k) s = s + val(o + S * k, i);
        c[o] = s / (double)nb;
      }
    }
  if (kind == 1)
    for (double &x : c) x = -x;  // forces, not gradients
  if (kind == 0 && !reftraj) {
    const double onbox[3] = {1.0 / box[0], 1.0 / box[1], 1.0 / box[2]};
    for (int m = 0; m < na / 3; ++m) {
      double *O = &c[9 * (size_t)m];
      for (int j = 0; j < 3; ++j) {
        const double dh1 = O[3 + j] - O[j], dh2 = O[6 + j] - O[j];
        O[j] = O[j] - box[j] * (std::round(O[j] * onbox[j]) - 0.5);  // Fortran nint
        O[3 + j] = dh1 + O[j];
        O[6 + j] = dh2 + O[j];
      }
    }
  }
  const double unit = kind == 0 ? TOA : 1.0;
  static const char *labels[3][3] = {{"O ", "H ", "H "}, {"O ", "D ", "D "}, {"O ", "D ", "H "}};
  const int iso = isotope >= 0 && isotope <= 2 ? isotope : 0;
  FILE *f = open_out(path, append);
  if (!f) return ctx_set_error(GB_E_ARG, std::string("cannot open ") + path);
  std::fprintf(f, " %11d\n", na);
  std::fprintf(f, " BOX %s%s%s\n", fnum(TOA * box[0]).c_str(), fnum(TOA * box[1]).c_str(), fnum(TOA * box[2]).c_str());
  for (int i = 0; i < na; ++i)
    std::fprintf(f, " %s%s%s%s\n", labels[iso][i % 3], fnum(unit * c[3 * (size_t)i]).c_str(),
                 fnum(unit * c[3 * (size_t)i + 1]).c_str(), fnum(unit * c[3 * (size_t)i + 2]).c_str());
  const bool ok = std::fclose(f) == 0;
  return ok ? GB_OK : ctx_set_error(GB_E_ARG, std::string("write failed: ") + path);
}

// Reads frame `frame` (0-based) of an xyz file of print_vmd_*: box (Angstrom,
// as printed) and the 3 na numbers of its atom lines (as printed)
int gbrpmd_read_vmd(const char *path, int frame, int na, double *box, double *xyz) {
  if (!path || !box || !xyz || na <= 0 || frame < 0) return ctx_set_error(GB_E_ARG, "bad argument");
  FILE *f = std::fopen(path, "r");
  if (!f) return ctx_set_error(GB_E_ARG, std::string("cannot open ") + path);
  char line[512];
  int fr = 0, st = GB_E_ARG;
  while (std::fgets(line, sizeof line, f)) {
    char *end = nullptr;
    const long n = std::strtol(line, &end, 10);
    if (end == line) continue;  // blank or unexpected line between frames
    if (n != na) break;
    if (!std::fgets(line, sizeof line, f)) break;
    if (fr == frame && std::sscanf(line, " BOX %lf %lf %lf", box, box + 1, box + 2) != 3) break;
    bool good = true;
    for (int i = 0; i < na && good; ++i) {
      if (!std::fgets(line, sizeof line, f)) {
        good = false;
        break;
      }
      if (fr == frame) {
        char el[8];
        for (char *q = line; *q; ++q)
          if (*q == 'D' && q > line && (q[-1] >= '0' && q[-1] <= '9')) *q = 'E';
        good = std::sscanf(line, " %7s %lf %lf %lf", el, xyz + 3 * (size_t)i, xyz + 3 * (size_t)i + 1,
                           xyz + 3 * (size_t)i + 2) == 4;
      }
    }
    if (!good) break;
    if (fr == frame) {
      st = GB_OK;
      break;
    }
    ++fr;
  }
  std::fclose(f);
  return st == GB_OK ? GB_OK : ctx_set_error(GB_E_ARG, std::string("no such frame in ") + path);
}

}  // extern "C"
