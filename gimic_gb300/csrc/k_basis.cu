// Basis-function evaluation on grid points.
//
//  * basis_split_kernel: phi at every point in fp32, scaled per point by a
//    power of two and written as two fp16 pieces (hi + lo) in the row-major
//    [point][kpad] layout that the tensor-core GEMM loads with TMA.
//  * basis_fp64_kernel: phi, grad phi and the Laplacian in fp64 for the plain
//    FP64 path.
//
// Both follow src/libgimic/bfeval.f90:81-122 (bfeval), :295-338 (dfdr) with
// the per-shell screening of src/libgimic/basis.f90:118-136 (a contraction
// contributes only when |r - R_A| <= its radius; squared distances are
// compared here).  One warp handles one point; lanes stride over functions so
// that stores are coalesced.
#include "gg_device.cuh"
#include "gg_kernels.h"

namespace gg {

namespace {

constexpr int kWarps = 8;

// Per-warp scratch: position of the point relative to every atom (fp32 x,
// y, z), its squared distance as a double-float (hi, lo) and the radial
// factor sum_p c_p exp(-a_p r^2) of every shell (0 when screened).  All
// per-atom and per-shell arithmetic is fp32 / double-float: none of it runs
// on the FP64 pipe.
struct AtomScratch {
  float* s;     // natoms x 4 (x, y, z, unused)
  float2* d2;   // natoms
  float* rad;   // nshells
};

__device__ __forceinline__ AtomScratch atom_scratch(int warp, int natoms, int nshells) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* d2 = reinterpret_cast<float2*>(smem_raw) + static_cast<size_t>(warp) * natoms;
  float* s = reinterpret_cast<float*>(reinterpret_cast<float2*>(smem_raw) + static_cast<size_t>(kWarps) * natoms) +
             static_cast<size_t>(warp) * natoms * 4;
  float* rad = reinterpret_cast<float*>(reinterpret_cast<float2*>(smem_raw) + static_cast<size_t>(kWarps) * natoms) +
               static_cast<size_t>(kWarps) * natoms * 4 + static_cast<size_t>(warp) * nshells;
  return {s, d2, rad};
}

// The point as double-floats: lanes 0-2 split one coordinate each and the
// warp shares them.
__device__ __forceinline__ void point_df(const double* __restrict__ pts, int64_t p, int lane, DFloat r[3]) {
  DFloat mine{0.f, 0.f};
  if (lane < 3) mine = df_split(pts[3 * p + lane]);
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    r[c].h = __shfl_sync(0xffffffffu, mine.h, c);
    r[c].l = __shfl_sync(0xffffffffu, mine.l, c);
  }
}

__device__ __forceinline__ void fill_atoms(const DevBasis& B, const DFloat r[3], AtomScratch sc, int lane) {
  for (int a = lane; a < B.natoms; a += 32) {
    float s3[3];
    const DFloat d2 = atom_offset(r, B.atom_df, a, s3);
    sc.d2[a] = make_float2(d2.h, d2.l);
    sc.s[4 * a] = s3[0];
    sc.s[4 * a + 1] = s3[1];
    sc.s[4 * a + 2] = s3[2];
  }
  __syncwarp();
  for (int sh = lane; sh < B.nshells; sh += 32) {
    const int a = __ldg(B.sh_atom + sh);
    const float2 d2 = sc.d2[a];
    float f1 = 0.f;
    if (df_le(DFloat{d2.x, d2.y}, __ldg(B.sh_rad2_df + sh))) {
      const int p0 = __ldg(B.sh_prim + sh), np = __ldg(B.sh_npf + sh);
      for (int p = 0; p < np; ++p)
        f1 += __ldg(B.p_cc + p0 + p) * gauss_df(__ldg(B.p_xp + p0 + p), __ldg(B.p_xplo + p0 + p), d2.x, d2.y);
    }
    sc.rad[sh] = f1;
  }
  __syncwarp();
}

__device__ __forceinline__ float phi32(const DevBasis& B, AtomScratch sc, int mu) {
  if (mu >= B.nbf) return 0.f;
  const int sh = __ldg(B.f_shell + mu);
  const float f1 = sc.rad[sh];
  if (f1 == 0.f) return 0.f;
  const int a = __ldg(B.sh_atom + sh);
  const float x = sc.s[4 * a], y = sc.s[4 * a + 1], z = sc.s[4 * a + 2];
  const int ijk = __ldg(B.f_ijk + mu);
  return powi(x, ijk & 15) * powi(y, (ijk >> 4) & 15) * powi(z, (ijk >> 8) & 15) * f1;
}

constexpr int kMaxPairs = 16;  // phi kept in registers for kpad <= 32 * 2 * kMaxPairs

}  // namespace

// One warp per point.  Lane l owns the function pairs (2l + 64t, 2l + 1 + 64t)
// so that every store is a coalesced 128-byte row segment of packed halves.
__global__ void __launch_bounds__(kWarps * 32, 2) basis_split_kernel(DevBasis B, const double* __restrict__ pts,
                                                                  int64_t npts, __half* __restrict__ a_hi,
                                                                  __half* __restrict__ a_lo,
                                                                  float* __restrict__ inv_scale) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t p = static_cast<int64_t>(blockIdx.x) * kWarps + warp;
  if (p >= npts) return;
  AtomScratch sc = atom_scratch(warp, B.natoms, B.nshells);
  DFloat r[3];
  point_df(pts, p, lane, r);
  fill_atoms(B, r, sc, lane);
  const int npairs = B.kpad / 64;
  const bool cached = npairs <= kMaxPairs;
  float2 val[kMaxPairs];
  float vmax = 0.f;
#pragma unroll
  for (int t = 0; t < kMaxPairs; ++t) {
    if (t < npairs) {
      const int mu = 64 * t + 2 * lane;
      val[t] = make_float2(phi32(B, sc, mu), phi32(B, sc, mu + 1));
      vmax = fmaxf(vmax, fmaxf(fabsf(val[t].x), fabsf(val[t].y)));
    }
  }
  for (int t = kMaxPairs; t < npairs; ++t) {
    const int mu = 64 * t + 2 * lane;
    vmax = fmaxf(vmax, fmaxf(fabsf(phi32(B, sc, mu)), fabsf(phi32(B, sc, mu + 1))));
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
  // scale = 2^(14 - e) with vmax = m 2^e, m in [0.5, 1): scaled values < 2^14
  float scale = 1.f;
  if (vmax > 0.f) {
    int e;
    frexpf(vmax, &e);
    scale = ldexpf(1.f, 14 - e);
  }
  __half2* hi_row = reinterpret_cast<__half2*>(a_hi + p * B.kpad);
  __half2* lo_row = reinterpret_cast<__half2*>(a_lo + p * B.kpad);
  auto store = [&](int t, float2 v) {
    v.x *= scale;
    v.y *= scale;
    const __half2 h = __floats2half2_rn(v.x, v.y);
    const float2 hf = __half22float2(h);
    hi_row[32 * t + lane] = h;
    lo_row[32 * t + lane] = __floats2half2_rn(v.x - hf.x, v.y - hf.y);
  };
#pragma unroll
  for (int t = 0; t < kMaxPairs; ++t)
    if (t < npairs && cached) store(t, val[t]);
  for (int t = cached ? npairs : 0; t < npairs; ++t) {
    const int mu = 64 * t + 2 * lane;
    store(t, make_float2(phi32(B, sc, mu), phi32(B, sc, mu + 1)));
  }
  if (lane == 0) inv_scale[p] = 1.f / scale;
}

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

const void* basis_split_kernel_ptr() { return reinterpret_cast<const void*>(&basis_split_kernel); }

size_t basis_smem_bytes(int natoms, int nshells) {
  return static_cast<size_t>(kWarps) * (natoms * (sizeof(float2) + 4 * sizeof(float)) + nshells * sizeof(float));
}

void launch_basis_split(const DevBasis& B, const double* pts, int64_t npts, __half* a_hi, __half* a_lo,
                        float* inv_scale, cudaStream_t st) {
  if (npts <= 0) return;
  const int64_t blocks = (npts + kWarps - 1) / kWarps;
  basis_split_kernel<<<static_cast<unsigned>(blocks), kWarps * 32, basis_smem_bytes(B.natoms, B.nshells), st>>>(
      B, pts, npts, a_hi, a_lo, inv_scale);
}

void launch_basis_fp64(const DevBasis& B, const double* pts, int64_t npts, int64_t ld, double* phi, double* gx,
                       double* gy, double* gz, double* lap, cudaStream_t st) {
  if (npts <= 0) return;
  const int64_t blocks = (npts + kWarps - 1) / kWarps;
  basis_fp64_kernel<<<static_cast<unsigned>(blocks), kWarps * 32, 0, st>>>(B, pts, npts, ld, phi, gx, gy, gz, lap);
}

}  // namespace gg
