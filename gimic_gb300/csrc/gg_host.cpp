// Host-side readers (INTGRL basis, XDENS densities), basis normalisation,
// screening radii and composite quadrature for the GB300 GIMIC path.
#include "gg_host.h"

#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <cstring>
#include <fstream>
#include <sstream>

namespace gg {

namespace {

// Component exponent tables, src/libgimic/gtodefs.f90:86-123.  Stored as
// packed (i*100 + j*10 + k) codes.
const int kStd[kMaxL + 1][21] = {
    {0},
    {100, 10, 1},
    {200, 110, 101, 20, 11, 2},
    {300, 210, 201, 120, 111, 102, 30, 21, 12, 3},
    {400, 310, 301, 220, 211, 202, 130, 121, 112, 103, 40, 31, 22, 13, 4},
    {500, 410, 401, 320, 311, 302, 230, 221, 212, 203, 140, 131, 122, 113, 104, 50, 41, 32, 23, 14, 5},
};
const int kTurbo[kMaxL + 1][21] = {
    {0},
    {100, 10, 1},
    {200, 20, 2, 110, 101, 11},
    {300, 30, 3, 210, 201, 120, 21, 102, 12, 111},
    {400, 40, 4, 310, 301, 130, 31, 103, 13, 220, 202, 22, 211, 121, 112},
    {500, 50, 5, 410, 401, 140, 41, 104, 14, 320, 302, 230, 32, 203, 23, 311, 131, 113, 221, 212, 122},
};

// Fortran list-directed input over a text file: each read() starts on a new
// record, consumes values across records (blank records are skipped) and
// drops whatever remains of its last record.
class ListReader {
 public:
  explicit ListReader(const std::string& path) : in_(path) {}
  bool ok() const { return static_cast<bool>(in_); }
  bool line(std::string* s) {
    if (!std::getline(in_, cur_)) return false;
    pos_ = 0;
    have_ = true;
    if (s) *s = cur_;
    return true;
  }
  // start a new read statement
  void begin() { have_ = false; }
  bool token(std::string* t) {
    for (;;) {
      if (!have_) {
        if (!std::getline(in_, cur_)) return false;
        pos_ = 0;
        have_ = true;
      }
      while (pos_ < cur_.size() && (std::isspace(static_cast<unsigned char>(cur_[pos_])) || cur_[pos_] == ','))
        ++pos_;
      if (pos_ >= cur_.size()) {
        have_ = false;
        continue;
      }
      size_t e = pos_;
      while (e < cur_.size() && !std::isspace(static_cast<unsigned char>(cur_[e])) && cur_[e] != ',') ++e;
      *t = cur_.substr(pos_, e - pos_);
      pos_ = e;
      return true;
    }
  }
  bool number(double* v) {
    std::string t;
    if (!token(&t)) return false;
    for (char& c : t)
      if (c == 'd' || c == 'D') c = 'E';
    char* end = nullptr;
    *v = std::strtod(t.c_str(), &end);
    return end != t.c_str();
  }
  bool integer(int* v) {
    double d;
    if (!number(&d)) return false;
    *v = static_cast<int>(d);
    return true;
  }
  // continue reading values from a given column of the current record
  void seek_column(size_t col) {
    pos_ = col;
    have_ = true;
  }

 private:
  std::ifstream in_;
  std::string cur_;
  size_t pos_ = 0;
  bool have_ = false;
};

// norm_ctr, src/libgimic/basis.f90:164-191
void normalise(Shell* s) {
  const double jl = static_cast<double>(s->l + 1);
  double n = 0.0;
  const size_t np = s->xp.size();
  for (size_t l = 0; l < np; ++l) {
    for (size_t m = 0; m <= l; ++m) {
      double t = 2.0 * std::sqrt(s->xp[l] * s->xp[m]) / (s->xp[l] + s->xp[m]);
      t = s->cc[l] * s->cc[m] * std::pow(t, jl + 0.5);
      n += t;
      if (l != m) n += t;
    }
  }
  n = 1.0 / std::sqrt(n);
  s->ncc.resize(np);
  for (size_t l = 0; l < np; ++l)
    s->ncc[l] = s->cc[l] * n * std::pow(4.0 * s->xp[l], 0.5 * jl + 0.25) * std::pow(0.5 / 3.141592653589793, 0.75);
}

// setup_screening, src/libgimic/basis.f90:90-112: first distance d on a
// 0.25 Bohr ladder with d^l exp(-alpha_min d^2) <= thrs.
double screening_radius(const Shell& s, double thrs) {
  double amin = 1e15;
  for (double a : s.xp) amin = std::min(amin, a);
  double x = 1e15, d = 0.0;
  while (x > thrs) {
    d += 0.25;
    double dl = 1.0;
    for (int i = 0; i < s.l; ++i) dl *= d;
    x = dl * std::exp(-amin * d * d);
  }
  return d;
}

}  // namespace

void component_exponents(int l, int c, bool turbomole, int out[3]) {
  const int code = (turbomole ? kTurbo : kStd)[l][c];
  out[0] = code / 100;
  out[1] = (code / 10) % 10;
  out[2] = code % 10;
}

void set_screening(Basis* b, double thrs) {
  for (Shell& s : b->shells) s.radius = thrs <= 0.0 ? 1e10 : screening_radius(s, thrs);
}

std::string read_intgrl(const std::string& path, double screen_thrs, Basis* out) {
  ListReader rd(path);
  if (!rd.ok()) return "read_intgrl(): open failed: " + path;
  std::string s;
  if (!rd.line(&s) || s.compare(0, 6, "INTGRL") != 0) return "not an INTGRL file: " + path;
  Basis b;
  if (!rd.line(&s)) return "truncated INTGRL file";
  b.turbomole = s.compare(0, 9, "TURBOMOLE") == 0;
  if (!rd.line(nullptr)) return "truncated INTGRL file";
  rd.begin();
  int natoms = 0;
  if (!rd.integer(&natoms) || natoms <= 0) return "bad atom count in " + path;
  if (!rd.line(nullptr)) return "truncated INTGRL file";
  const std::string bad = "malformed INTGRL file: " + path;
  for (int a = 0; a < natoms; ++a) {
    Atom at;
    double charge;
    int dummy, nsh;
    rd.begin();
    if (!rd.number(&charge) || !rd.integer(&dummy) || !rd.integer(&nsh)) return bad;
    if (nsh < 1 || nsh - 1 > kMaxL) return "Largest allowed l-quantum number in basis exceeded";
    int nctrps[kMaxL + 1] = {0};
    for (int i = 0; i < nsh; ++i)
      if (!rd.integer(&nctrps[i])) return bad;
    at.charge = charge;
    at.nshells = nsh;
    // atom record: symbol in columns 1-2, id in 3-4, coordinates from 5
    if (!rd.line(&s) || s.size() < 5) return bad;
    at.symbol[0] = s[0];
    at.symbol[1] = s[1];
    rd.seek_column(4);
    for (int d = 0; d < 3; ++d)
      if (!rd.number(&at.coord[d])) return bad;
    for (int l = 0; l < nsh; ++l) {
      int nseg = 0;
      for (int j = 0; j < nctrps[l]; ++j) {
        int npf, ncf;
        rd.begin();
        if (!rd.integer(&npf) || !rd.integer(&ncf) || npf < 1 || ncf < 1) return bad;
        std::vector<Shell> seg(ncf);
        for (Shell& sh : seg) {
          sh.atom = a;
          sh.l = l;
          sh.ncomp = (l + 1) * (l + 2) / 2;
          sh.xp.resize(npf);
          sh.cc.resize(npf);
        }
        for (int p = 0; p < npf; ++p) {
          double xp;
          rd.begin();
          if (!rd.number(&xp)) return bad;
          for (int k = 0; k < ncf; ++k) {
            double cc;
            if (!rd.number(&cc)) return bad;
            seg[k].xp[p] = xp;
            seg[k].cc[p] = cc;
          }
        }
        for (Shell& sh : seg) b.shells.push_back(std::move(sh));
        nseg += ncf;
      }
      at.nctrps[l] = nseg;
    }
    b.atoms.push_back(at);
  }
  // function numbering (calc_basdim, basis.f90:216-249) and normalisation
  int f = 0;
  for (size_t i = 0; i < b.shells.size(); ++i) {
    Shell& sh = b.shells[i];
    normalise(&sh);
    sh.first = f;
    for (int c = 0; c < sh.ncomp; ++c) {
      b.func_atom.push_back(sh.atom);
      b.func_shell.push_back(static_cast<int>(i));
      b.func_comp.push_back(c);
    }
    f += sh.ncomp;
    b.atoms[sh.atom].nfunc += sh.ncomp;
    b.nprim += static_cast<int>(sh.xp.size()) * sh.ncomp;
  }
  b.nbf = f;
  set_screening(&b, screen_thrs);
  *out = std::move(b);
  return "";
}

std::string read_xdens(const std::string& path, const Basis& basis, bool uhf, Density* out) {
  ListReader rd(path);
  if (!rd.ok()) return "Density file not found: " + path;
  const int n = basis.nbf;
  const size_t nn = static_cast<size_t>(n) * n;
  Density d;
  d.nbf = n;
  d.uhf = uhf;
  d.a.assign(4 * nn, 0.0);
  if (uhf) d.b.assign(4 * nn, 0.0);
  for (int spin = 0; spin < (uhf ? 2 : 1); ++spin) {
    std::vector<double>& m = spin == 0 ? d.a : d.b;
    for (size_t i = 0; i < 4 * nn; ++i) {
      rd.begin();
      if (!rd.number(&m[i])) return "XDENS file too short for nbf=" + std::to_string(n) + ": " + path;
      // the reference reads whatever is there (read_array, src/libgimic/
      // dens.f90:125-131); a NaN or infinity would reach every point's
      // tensor, so it is refused here with its position
      if (!std::isfinite(m[i]))
        return "XDENS value " + std::to_string(spin * 4 * nn + i + 1) + " is not finite: " + path;
    }
  }
  // The reference stops reading after the blocks it needs and ignores the
  // rest, so a density of a larger basis (or an open-shell file read as
  // closed shell) would silently give wrong currents.  Trailing numbers are
  // therefore an error.
  {
    double extra = 0.0;
    rd.begin();
    if (rd.number(&extra))
      return "XDENS holds more values than the " + std::to_string((uhf ? 2 : 1) * 4 * nn) + " that nbf=" +
             std::to_string(n) + (uhf ? " (open shell)" : " (closed shell)") +
             " needs: the density belongs to another basis or spin treatment: " + path;
  }
  if (uhf) {
    for (size_t i = nn; i < 4 * nn; ++i) {
      d.a[i] /= 2.0;
      d.b[i] /= 2.0;
    }
  }
  if (basis.turbomole) {
    // sv[q] = atom-major index of the q-th function in l-major order
    std::vector<int> lvec(n), sv;
    for (int i = 0; i < n; ++i) lvec[i] = basis.shells[basis.func_shell[i]].l;
    for (int l = 0; static_cast<int>(sv.size()) < n; ++l)
      for (int i = 0; i < n; ++i)
        if (lvec[i] == l) sv.push_back(i);
    std::vector<double> tmp(nn);
    for (int spin = 0; spin < (uhf ? 2 : 1); ++spin) {
      std::vector<double>& m = spin == 0 ? d.a : d.b;
      for (int blk = 0; blk < 4; ++blk) {
        double* x = m.data() + blk * nn;
        for (int j = 0; j < n; ++j)
          for (int i = 0; i < n; ++i) tmp[sv[i] + static_cast<size_t>(sv[j]) * n] = x[i + static_cast<size_t>(j) * n];
        std::copy(tmp.begin(), tmp.end(), x);
      }
    }
  }
  *out = std::move(d);
  return "";
}

// ---------------------------------------------------------------------------
// Spherical basis (Advanced.spherical, src/fgimic/gimic.F90:85-87).  The
// reference evaluates Cartesian functions and projects them per point,
// sbf = po . bf (src/libgimic/bfeval.f90:116-117, dfdr :330-333), with po
// block diagonal per shell (cao2sao.f90:64-101).  Every output is a bilinear
// form in the basis values and their derivatives, and the GIAO factors
// depend only on the function's atom, which po never mixes, so
//   sbf^T M sbf' = bf^T (po^T M po) bf'
// exactly: the densities are projected once to the Cartesian basis and the
// evaluation stays Cartesian.
// ---------------------------------------------------------------------------
namespace {
long factorial(int n) {
  long m = 1;
  for (int i = 2; i <= n; ++i) m *= i;
  return m;
}
long binomial(int a, int b) { return factorial(a) / (factorial(b) * factorial(a - b)); }

// integer-rescaled row, as cao2sao.f90:205-235 (renorm): divide by the
// smallest magnitude, then multiply by the largest reciprocal needed to
// clear the fractions
void integer_row(std::vector<double>& row) {
  double amin = 1e10;
  for (double v : row)
    if (std::fabs(v) > 0.0) amin = std::min(amin, std::fabs(v));
  for (double& v : row) v /= amin;
  double mult = 1.0;
  for (double v : row) {
    double a = std::fabs(v);
    if (!(a > 0.0)) continue;
    double f = std::fmod(a, 1.0);
    if (f > 1e-10) {
      a = 1.0 / f;
      while (std::fmod(a, 1.0) > 1e-10) {
        f = std::fmod(a, 1.0);
        if (f > 1e-10) a /= f;
      }
      mult = std::max(mult, a);
    }
  }
  for (double& v : row) v *= mult;
}
}  // namespace

std::vector<double> spherical_projection(int l) {
  // rows m = -l..l over the shell's Cartesian components (standard order):
  // the solid-harmonic expansion of cao2sao.f90:153-201 (clmtuv, mkc2sop),
  // each (t, u, v) term assigned to its component x^i y^j z^k
  const int nc = (l + 1) * (l + 2) / 2;
  std::vector<double> op(static_cast<size_t>(2 * l + 1) * nc, 0.0);
  for (int m = -l; m <= l; ++m) {
    std::vector<double> row(nc, 0.0);
    const int am = std::abs(m);
    const int half = m < 0 ? 1 : 0;  // v runs over half-integers for m < 0
    for (int t = 0; t <= (l - am) / 2; ++t)
      for (int u = 0; u <= t; ++u)
        for (int v = 0; 2 * v + half <= am; ++v) {
          const int two_v = 2 * v + half;  // 2 (v + v_m)
          const int i = 2 * t + am - (2 * u + two_v), j = 2 * u + two_v, k = l - 2 * t - am;
          double q = std::ldexp(1.0, -2 * t) *
                     static_cast<double>(binomial(l, t) * binomial(l - t, am + t) * binomial(t, u) * binomial(am, two_v));
          if ((t + v) & 1) q = -q;
          for (int c = 0; c < nc; ++c) {
            int e[3];
            component_exponents(l, c, false, e);
            if (e[0] == i && e[1] == j && e[2] == k) row[c] = q;
          }
        }
    integer_row(row);
    std::copy(row.begin(), row.end(), op.begin() + static_cast<size_t>(m + l) * nc);
  }
  return op;
}

int spherical_count(const Basis& b) {
  int n = 0;
  for (const Shell& s : b.shells) n += 2 * s.l + 1;
  return n;
}

std::string read_xdens_spherical(const std::string& path, const Basis& basis, bool uhf, Density* out) {
  if (basis.turbomole) return "spherical basis with the TURBOMOLE component order is not supported";
  const int ns = spherical_count(basis), nc = basis.nbf;
  // the file holds ns x ns blocks: read them through a basis-sized stand-in
  Basis sb;
  sb.nbf = ns;
  Density ds;
  std::string e = read_xdens(path, sb, uhf, &ds);
  if (!e.empty()) return e;
  // per Cartesian function: the spherical rows of its shell and their weights
  std::vector<int> srow0(basis.shells.size());
  for (size_t k = 0, r = 0; k < basis.shells.size(); ++k) {
    srow0[k] = static_cast<int>(r);
    r += 2 * basis.shells[k].l + 1;
  }
  std::vector<std::vector<double>> ops(kMaxL + 1);
  for (int l = 0; l <= kMaxL; ++l) ops[l] = spherical_projection(l);
  auto weight = [&](int s_row, int mu) -> double {  // po(s_row, mu), zero off the shell
    const int k = basis.func_shell[mu];
    const Shell& sh = basis.shells[k];
    const int ls = s_row - srow0[k];
    if (ls < 0 || ls > 2 * sh.l) return 0.0;
    return ops[sh.l][static_cast<size_t>(ls) * sh.ncomp + basis.func_comp[mu]];
  };
  Density d;
  d.nbf = nc;
  d.uhf = uhf;
  const size_t nn = static_cast<size_t>(nc) * nc, ss = static_cast<size_t>(ns) * ns;
  d.a.assign(4 * nn, 0.0);
  if (uhf) d.b.assign(4 * nn, 0.0);
  std::vector<double> x(static_cast<size_t>(ns) * nc);  // M po, column-major ns x nc
  for (int spin = 0; spin < (uhf ? 2 : 1); ++spin) {
    const std::vector<double>& src = spin == 0 ? ds.a : ds.b;
    std::vector<double>& dst = spin == 0 ? d.a : d.b;
    for (int blk = 0; blk < 4; ++blk) {
      const double* m = src.data() + blk * ss;
      double* o = dst.data() + blk * nn;
      for (int nu = 0; nu < nc; ++nu) {
        const int k = basis.func_shell[nu];
        const int r0 = srow0[k], nr = 2 * basis.shells[k].l + 1;
        for (int s = 0; s < ns; ++s) {
          double acc = 0.0;
          for (int t = r0; t < r0 + nr; ++t) acc += m[s + static_cast<size_t>(t) * ns] * weight(t, nu);
          x[s + static_cast<size_t>(nu) * ns] = acc;
        }
      }
      for (int nu = 0; nu < nc; ++nu)
        for (int mu = 0; mu < nc; ++mu) {
          const int k = basis.func_shell[mu];
          const int r0 = srow0[k], nr = 2 * basis.shells[k].l + 1;
          double acc = 0.0;
          for (int s = r0; s < r0 + nr; ++s) acc += weight(s, mu) * x[s + static_cast<size_t>(nu) * ns];
          o[mu + static_cast<size_t>(nu) * nc] = acc;
        }
    }
  }
  *out = std::move(d);
  return "";
}

// ---------------------------------------------------------------------------
// Quadrature, src/libgimic/gaussint.f90:21-112 (gaussl, lobattomy) and
// :144-222 (Legendre recurrences).  Newton tolerance 3e-12, at most 10 steps.
// ---------------------------------------------------------------------------
namespace {
constexpr double kPi = 3.141592653589793;
constexpr double kEps = 3.0e-12;
constexpr int kNewtonMax = 10;

// P_n(x), P_n'(x), P_n''(x) by the three-term recurrence
void legendre(double x, int n, double* p, double* dp, double* d2p) {
  *p = 1.0;
  *dp = 0.0;
  *d2p = 0.0;
  if (n == 0) return;
  *p = x;
  *dp = 1.0;
  if (n == 1) return;
  double pm = 1.0, dpm = 0.0, d2pm = 0.0;
  for (int i = 2; i <= n; ++i) {
    const double c1 = i, c2 = c1 * 2.0 - 1.0, c4 = c1 - 1.0;
    const double p0 = *p;
    *p = (c2 * x * *p - c4 * pm) / c1;
    pm = p0;
    const double dp0 = *dp;
    *dp = (c2 * x * *dp - c4 * dpm + c2 * pm) / c1;
    dpm = dp0;
    const double d2p0 = *d2p;
    *d2p = (c2 * x * *d2p - c4 * d2pm + c2 * 2.0 * dpm) / c1;
    d2pm = d2p0;
  }
}

int gauss_legendre(int n, double* x, double* w) {
  const int m = (n % 2 == 0) ? n / 2 : (n + 1) / 2;
  for (int i = 1; i <= m; ++i) {
    double z = std::cos(kPi * (i - 0.25) / (n + 0.5)), p = 0, dp = 0, d2p = 0;
    int it = 1;
    for (; it <= kNewtonMax; ++it) {
      legendre(z, n, &p, &dp, &d2p);
      const double z1 = z;
      z = z1 - p / dp;
      if (std::fabs(z - z1) <= kEps) break;
    }
    if (it >= kNewtonMax) return -1;
    x[i - 1] = -z;
    x[n - i] = z;
    w[i - 1] = 2.0 / ((1.0 - z * z) * dp * dp);
    w[n - i] = w[i - 1];
  }
  return 0;
}

int gauss_lobatto(int n, double* x, double* w) {
  x[0] = -1.0;
  x[n - 1] = 1.0;
  w[0] = 2.0 / static_cast<double>(n * n - n);
  w[n - 1] = w[0];
  for (int i = 2; i <= n - 1; ++i) {
    double z = std::cos(kPi * (i - 0.25) / (n + 0.5)), p = 0, dp = 0, d2p = 0;
    int it = 1;
    for (; it <= kNewtonMax; ++it) {
      legendre(z, n - 1, &p, &dp, &d2p);
      const double z1 = z;
      z = z1 - dp / d2p;
      double damp = 0.5;
      while (std::fabs(z) > 1.0) {
        z = z1 - dp / d2p * damp;
        damp = damp * damp;
      }
      if (std::fabs(z - z1) <= kEps) break;
    }
    if (it >= kNewtonMax) return -1;
    x[i - 1] = -z;
    w[i - 1] = 2.0 / (static_cast<double>(n * n - n) * p * p);
  }
  return 0;
}
}  // namespace

int gauss_data(double a, double b, int order, int npts, int quadrature, double* pts, double* wgt) {
  if (npts == 1) {
    pts[0] = 0.0;
    wgt[0] = 1.0;
    return 0;
  }
  if (order <= 0 || npts <= 0 || npts % order != 0) return -1;
  std::vector<double> x(order), w(order);
  // nodes on [-1, 1]: xm = 0, xl = 1, so xm - xl*z is -z exactly
  const int rc = quadrature == 1 ? gauss_lobatto(order, x.data(), w.data()) : gauss_legendre(order, x.data(), w.data());
  if (rc != 0) return rc;
  const int nblock = npts / order;
  const double step = (b - a) / static_cast<double>(nblock);
  const double half = step * 0.5;
  for (int i = 0; i < order; ++i) x[i] = x[i] + 1.0;
  for (int blk = 0; blk < nblock; ++blk)
    for (int i = 0; i < order; ++i) {
      pts[blk * order + i] = x[i] * half + static_cast<double>(blk) * step;
      wgt[blk * order + i] = w[i] * half;
    }
  return 0;
}

namespace {

// Visiting order of the atoms: start at the atom farthest from the centroid,
// then always step to the nearest atom not yet visited.
std::vector<int> atom_tour(const Basis& b) {
  const int na = static_cast<int>(b.atoms.size());
  double c[3] = {0, 0, 0};
  for (const Atom& a : b.atoms)
    for (int d = 0; d < 3; ++d) c[d] += a.coord[d] / na;
  auto dist2 = [&](const double* x, const double* y) {
    double s = 0;
    for (int d = 0; d < 3; ++d) s += (x[d] - y[d]) * (x[d] - y[d]);
    return s;
  };
  int cur = 0;
  for (int a = 1; a < na; ++a)
    if (dist2(b.atoms[a].coord, c) > dist2(b.atoms[cur].coord, c)) cur = a;
  std::vector<char> seen(na, 0);
  std::vector<int> tour;
  for (int step = 0; step < na; ++step) {
    tour.push_back(cur);
    seen[cur] = 1;
    int next = -1;
    double best = 0;
    for (int a = 0; a < na; ++a) {
      if (seen[a]) continue;
      const double d2 = dist2(b.atoms[a].coord, b.atoms[cur].coord);
      if (next < 0 || d2 < best) {
        next = a;
        best = d2;
      }
    }
    cur = next;
  }
  return tour;
}

// Active (K block, chunk) pairs of a shell order summed over the bricks;
// dist[i * natoms + a] = distance from brick i's centre to atom a.
double order_cost(const Basis& b, const std::vector<int>& order, const std::vector<double>& dist, int nbricks,
                  double brick_radius) {
  const int na = static_cast<int>(b.atoms.size());
  const int nkb = (b.nbf + 63) / 64, nch = (b.nbf + 31) / 32;
  std::vector<int> f0(order.size());
  int f = 0;
  for (size_t k = 0; k < order.size(); ++k) {
    f0[k] = f;
    f += b.shells[order[k]].ncomp;
  }
  std::vector<char> kb(nkb), ch(nch);
  double cost = 0;
  for (int i = 0; i < nbricks; ++i) {
    std::fill(kb.begin(), kb.end(), 0);
    std::fill(ch.begin(), ch.end(), 0);
    for (size_t k = 0; k < order.size(); ++k) {
      const Shell& s = b.shells[order[k]];
      if (dist[static_cast<size_t>(i) * na + s.atom] - brick_radius > s.radius) continue;
      const int a = f0[k], e = f0[k] + s.ncomp - 1;
      for (int q = a / 64; q <= e / 64; ++q) kb[q] = 1;
      for (int q = a / 32; q <= e / 32; ++q) ch[q] = 1;
    }
    double nk = 0, nc = 0;
    for (char v : kb) nk += v;
    for (char v : ch) nc += v;
    cost += nk * nc;
  }
  return cost;
}

}  // namespace

std::vector<int> locality_shell_order(const Basis& b) {
  const int ns = static_cast<int>(b.shells.size()), na = static_cast<int>(b.atoms.size());
  std::vector<int> ident(ns);
  for (int k = 0; k < ns; ++k) ident[k] = k;
  if (ns < 2 || na < 1) return ident;
  // bricks of 2 x 1 x 1 Bohr over the atoms' bounding box + 4 Bohr, thinned
  // to at most 8192 by a stride
  double lo[3], hi[3];
  for (int d = 0; d < 3; ++d) {
    lo[d] = hi[d] = b.atoms[0].coord[d];
    for (const Atom& a : b.atoms) {
      lo[d] = std::min(lo[d], a.coord[d]);
      hi[d] = std::max(hi[d], a.coord[d]);
    }
    lo[d] -= 4.0;
    hi[d] += 4.0;
  }
  const double edge[3] = {2.0, 1.0, 1.0};
  int nb[3];
  for (int d = 0; d < 3; ++d) nb[d] = std::max(1, static_cast<int>(std::ceil((hi[d] - lo[d]) / edge[d])));
  const int64_t total = static_cast<int64_t>(nb[0]) * nb[1] * nb[2];
  const int64_t stride = std::max<int64_t>(1, (total + 8191) / 8192);
  std::vector<double> dist;
  int nbricks = 0;
  for (int64_t i = 0; i < total; i += stride, ++nbricks) {
    const int64_t ix = i / (static_cast<int64_t>(nb[1]) * nb[2]), iy = (i / nb[2]) % nb[1], iz = i % nb[2];
    const double c[3] = {lo[0] + (ix + 0.5) * edge[0], lo[1] + (iy + 0.5) * edge[1], lo[2] + (iz + 0.5) * edge[2]};
    for (const Atom& a : b.atoms) {
      double s = 0;
      for (int d = 0; d < 3; ++d) s += (c[d] - a.coord[d]) * (c[d] - a.coord[d]);
      dist.push_back(std::sqrt(s));
    }
  }
  const double brick_radius = 0.5 * std::sqrt(edge[0] * edge[0] + edge[1] * edge[1] + edge[2] * edge[2]);
  const std::vector<int> tour = atom_tour(b);
  std::vector<int> tpos(na);
  for (int k = 0; k < na; ++k) tpos[tour[k]] = k;
  std::vector<double> radii;
  for (const Shell& s : b.shells) radii.push_back(s.radius);
  std::sort(radii.begin(), radii.end());
  std::vector<int> best = ident;
  double best_cost = order_cost(b, ident, dist, nbricks, brick_radius);
  for (int nclass = 1; nclass <= 4; ++nclass) {
    // class boundaries at the radius quantiles; class 0 holds the widest shells
    std::vector<double> edges;
    for (int q = 1; q < nclass; ++q) edges.push_back(radii[static_cast<size_t>(q) * ns / nclass]);
    std::vector<int> cls(ns);
    for (int k = 0; k < ns; ++k) {
      const double r = b.shells[k].radius;
      cls[k] = nclass - 1 - static_cast<int>(std::upper_bound(edges.begin(), edges.end(), r) - edges.begin());
    }
    std::vector<int> ord = ident;
    std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
      if (cls[x] != cls[y]) return cls[x] < cls[y];
      return tpos[b.shells[x].atom] < tpos[b.shells[y].atom];
    });
    const double c = order_cost(b, ord, dist, nbricks, brick_radius);
    if (c < best_cost) {
      best_cost = c;
      best = ord;
    }
  }
  return best;
}

void permute_shells(Basis* b, Density* d, const std::vector<int>& order) {
  const int n = b->nbf;
  std::vector<int> src(n);  // new function -> current function
  std::vector<Shell> shells;
  shells.reserve(order.size());
  int f = 0;
  for (int k : order) {
    Shell s = b->shells[k];
    for (int c = 0; c < s.ncomp; ++c) src[f + c] = s.first + c;
    s.first = f;
    f += s.ncomp;
    shells.push_back(std::move(s));
  }
  b->shells = std::move(shells);
  b->func_atom.clear();
  b->func_shell.clear();
  b->func_comp.clear();
  for (size_t i = 0; i < b->shells.size(); ++i)
    for (int c = 0; c < b->shells[i].ncomp; ++c) {
      b->func_atom.push_back(b->shells[i].atom);
      b->func_shell.push_back(static_cast<int>(i));
      b->func_comp.push_back(c);
    }
  const size_t nn = static_cast<size_t>(n) * n;
  for (std::vector<double>* m : {&d->a, &d->b}) {
    if (m->empty()) continue;
    std::vector<double> out(m->size());
    const size_t nblk = m->size() / nn;
    for (size_t blk = 0; blk < nblk; ++blk)
      for (int j = 0; j < n; ++j)
        for (int i = 0; i < n; ++i)
          out[blk * nn + i + static_cast<size_t>(j) * n] = (*m)[blk * nn + src[i] + static_cast<size_t>(src[j]) * n];
    m->swap(out);
  }
}

double au2si(double au) {
  const double aulength = 0.52917726e-10, auspeedoflight = 137.03599, speedoflight = 299792458.0;
  const double aucharge = 1.60217733e-19, hbar = 1.05457267e-34;
  const double autime = aulength * auspeedoflight / speedoflight;
  const double autesla = hbar / aucharge / aulength / aulength;
  const double audjdb = aucharge / autime / autesla;
  return au * audjdb * 1.0e9;
}

}  // namespace gg
