// Host-side data model of the GB300 GIMIC path: basis set, densities and
// quadrature.  Pure C++ (no CUDA), compiled into libgimic_gb300.so.
#pragma once
#include <cstdint>
#include <string>
#include <vector>

namespace gg {

constexpr int kMaxL = 5;  // s..h, src/libgimic/globals.f90:30

// One segmented contraction (src/libgimic/globals.f90:95-100).
struct Shell {
  int atom = 0;
  int l = 0;
  int ncomp = 1;
  int first = 0;  // first basis function (global, atom-major order)
  std::vector<double> xp, cc, ncc;
  double radius = 1e10;  // screening radius (basis%thrs)
};

struct Atom {
  double coord[3] = {0, 0, 0};
  double charge = 0;
  char symbol[3] = {' ', ' ', 0};
  int nshells = 0;
  int nctrps[kMaxL + 1] = {0};
  int nfunc = 0;
};

struct Basis {
  std::vector<Atom> atoms;
  std::vector<Shell> shells;  // atom-major, then l, then order in file
  int nbf = 0;
  int nprim = 0;              // sum over shells of npf * ncomp (ngto)
  bool turbomole = false;
  std::vector<int> func_atom;   // atom of each function
  std::vector<int> func_shell;  // shell of each function
  std::vector<int> func_comp;   // component index within its shell
};

// Cartesian exponents (i, j, k) of component c of an l shell, standard or
// TURBOMOLE order (src/libgimic/gtodefs.f90:86-123).
void component_exponents(int l, int c, bool turbomole, int out[3]);

// Reads an INTGRL file (src/libgimic/intgrl.f90:20-264), normalises the
// contractions (basis.f90:164-191) and sets the screening radii
// (basis.f90:90-112); screen_thrs <= 0 disables screening.
// Returns an empty string on success, else an error message.
std::string read_intgrl(const std::string& path, double screen_thrs, Basis* out);

// Recomputes the screening radii for a new threshold (<= 0: none).
void set_screening(Basis* b, double screen_thrs);

// Density matrices for one spin: four column-major nbf x nbf blocks
// (D, dD/dBx, dD/dBy, dD/dBz).
struct Density {
  int nbf = 0;
  bool uhf = false;
  std::vector<double> a;  // 4 * nbf * nbf, alpha (or closed shell)
  std::vector<double> b;  // beta (uhf only)
};

// Reads XDENS (src/libgimic/dens.f90:56-135), halves the perturbed blocks for
// UHF (dens.f90:94-98) and reorders TURBOMOLE files to atom-major order
// (reorder.f90:54-96, dens.f90:210-234).
std::string read_xdens(const std::string& path, const Basis& basis, bool uhf, Density* out);

// Spherical basis: rows m = -l..l of the integer-rescaled projection of a
// shell's Cartesian components (standard order) onto real solid harmonics,
// (2l+1) x ncomp row-major (src/libgimic/cao2sao.f90:153-235).
std::vector<double> spherical_projection(int l);
int spherical_count(const Basis& b);
// XDENS over the spherical functions (2l+1 per shell), projected to the
// Cartesian basis: M_cart = po^T M_sph po per block.  Standard component
// order only.
std::string read_xdens_spherical(const std::string& path, const Basis& basis, bool uhf, Density* out);

// Shell order for the screened split path.  Tile screening skips the
// 64-function K blocks and 32-function column chunks in which no shell
// reaches a tile, so the work falls when the shells that are in range of the
// same region of space sit next to each other.  Candidates: the file order,
// and shells grouped into 1..4 screening-radius classes (widest first) with
// the atoms of each class along a nearest-neighbour tour.  Each candidate is
// scored by the number of (K block, chunk) pairs active over 2 x 1 x 1 Bohr
// bricks covering the atoms' bounding box plus 4 Bohr; the file order wins
// ties.  Returns order[k] = index of the shell placed at position k.
std::vector<int> locality_shell_order(const Basis& b);

// Moves the shells to the given order (order[k] = current index of the shell
// placed at k): renumbers the basis functions and permutes the rows and
// columns of every density block to match.  The current and magnetically
// induced densities are sums over function pairs, so nothing computed from
// them changes beyond rounding.
void permute_shells(Basis* b, Density* d, const std::vector<int>& order);

// Composite Gauss / Gauss-Lobatto nodes (src/libgimic/gaussint.f90:267-319):
// npts points made of npts/order panels on [0, b - a].  quadrature: 0 gauss,
// 1 lobatto.  Returns 0, or -1 (npts not divisible / Newton failed).
int gauss_data(double a, double b, int order, int npts, int quadrature, double* pts, double* wgt);

// Unit conversion au -> nA/T (src/libgimic/globals.f90 au2si).
double au2si(double au);

}  // namespace gg
