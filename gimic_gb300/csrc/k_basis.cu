// Basis-function evaluation on grid points for the plain FP64 path:
// basis_fp64_kernel computes phi, grad phi and the Laplacian in fp64,
// following src/libgimic/bfeval.f90:81-122 (bfeval), :295-338 (dfdr) with the
// per-shell screening of src/libgimic/basis.f90:118-136 (a contraction
// contributes only when |r - R_A| <= its radius; squared distances are
// compared here).  One warp handles one point; lanes stride over functions so
// that stores are coalesced.  The split-FP16 operand is built by
// k_basis_tile.cu.
#include "gg_device.cuh"
#include "gg_kernels.h"

namespace gg {

namespace {
constexpr int kWarps = 8;
}  // namespace

__global__ void __launch_bounds__(kWarps * 32) basis_fp64_kernel(DevBasis B, const double* __restrict__ pts,
                                                                 int64_t npts, int64_t ld, double* __restrict__ phi,
                                                                 double* __restrict__ gx, double* __restrict__ gy,
                                                                 double* __restrict__ gz, double* __restrict__ lap) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t p = static_cast<int64_t>(blockIdx.x) * kWarps + warp;
  if (p >= npts) return;
  const double r[3] = {pts[3 * p], pts[3 * p + 1], pts[3 * p + 2]};
  for (int mu = lane; mu < B.nbf; mu += 32) {
    const int sh = __ldg(B.f_shell + mu);
    const int a = __ldg(B.sh_atom + sh);
    const double x = r[0] - B.atom_xyz[3 * a], y = r[1] - B.atom_xyz[3 * a + 1], z = r[2] - B.atom_xyz[3 * a + 2];
    const double d2 = x * x + y * y + z * z;
    double v = 0, dx = 0, dy = 0, dz = 0, l2 = 0;
    if (d2 <= __ldg(B.sh_rad2 + sh)) {
      const int p0 = __ldg(B.sh_prim + sh), np = __ldg(B.sh_npf + sh);
      double f1 = 0, f2 = 0, f3 = 0;
      for (int q = 0; q < np; ++q) {
        const double al = __ldg(B.p_xpd + p0 + q);
        const double e = __ldg(B.p_ccd + p0 + q) * exp(-al * d2);
        f1 += e;
        f2 += al * e;
        f3 += al * al * e;
      }
      cart_eval<double>(__ldg(B.f_ijk + mu), x, y, z, f1, f2, f3, &v, &dx, &dy, &dz, &l2);
    }
    const int64_t o = p * ld + mu;
    phi[o] = v;
    gx[o] = dx;
    gy[o] = dy;
    gz[o] = dz;
    lap[o] = l2;
  }
}

void launch_basis_fp64(const DevBasis& B, const double* pts, int64_t npts, int64_t ld, double* phi, double* gx,
                       double* gy, double* gz, double* lap, cudaStream_t st) {
  if (npts <= 0) return;
  const int64_t blocks = (npts + kWarps - 1) / kWarps;
  basis_fp64_kernel<<<static_cast<unsigned>(blocks), kWarps * 32, 0, st>>>(B, pts, npts, ld, phi, gx, gy, gz, lap);
}

}  // namespace gg
