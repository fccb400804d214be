// Tile screening pieces shared by tile_screen_kernel (k_tiles.cu) and the
// short-pass basis kernel (k_basis_tile.cu), which screens its own tile when
// a pass has no more tiles than SMs.  Both give the same lists bit for bit.
//
// A shell is out of range for a tile when |R_A - c| - rho > radius (c, rho:
// centre and radius of the tile's bounding box), which by the triangle
// inequality excludes it for every point of the tile (basis.f90:90-136
// screens point by point; this is the tile-level bound).  The box is formed
// in fp32 from coordinates rounded outwards, and rho is widened by far more
// than the fp32 rounding of the centre, so the test stays conservative
// without FP64 arithmetic.
#pragma once

#include "gg_device.cuh"

namespace gg {

// Bounding sphere of tile t (points t*128 .. +127, the tile's first point
// standing in past the end n), computed by one whole warp; every lane gets
// the centre cf and the widened radius rhof.  A coordinate is converted to
// fp32 once (round to nearest, within 2^-24 |x| plus a subnormal step of
// it) and widened outwards by 2^-23 |x| + 2^-126 in fp32, which contains the
// fp64 value: one conversion on the FP64 pipe instead of two directed ones.
__device__ __forceinline__ void warp_tile_sphere(const double* __restrict__ pts, int64_t n, int64_t t, int lane,
                                                 float cf[3], float* rhof) {
  float lo[3], hi[3];
  for (int k = 0; k < kBlockM / 32; ++k) {
    const int64_t p = t * kBlockM + k * 32 + lane;
    const int64_t q = p < n ? p : t * kBlockM;
    for (int d = 0; d < 3; ++d) {
      const float v = __double2float_rn(pts[3 * q + d]);
      const float e = __fmaf_ru(fabsf(v), 0x1p-23f, 0x1p-126f);
      const float l = __fsub_rd(v, e), h = __fadd_ru(v, e);
      lo[d] = k == 0 ? l : fminf(lo[d], l);
      hi[d] = k == 0 ? h : fmaxf(hi[d], h);
    }
  }
  for (int o = 16; o > 0; o >>= 1)
    for (int d = 0; d < 3; ++d) {
      lo[d] = fminf(lo[d], __shfl_xor_sync(0xffffffffu, lo[d], o));
      hi[d] = fmaxf(hi[d], __shfl_xor_sync(0xffffffffu, hi[d], o));
    }
  float rho2 = 0.f, cmax = 0.f;
  for (int d = 0; d < 3; ++d) {
    cf[d] = 0.5f * (lo[d] + hi[d]);
    const float h = __fmul_ru(0.5f, __fsub_ru(hi[d], lo[d]));
    rho2 = __fmaf_ru(h, h, rho2);
    cmax = fmaxf(cmax, fabsf(cf[d]));
  }
  // the centre's fp32 rounding is below 2^-23 |c| per axis; widen by 2^-16
  *rhof = __fmul_ru(sqrtf(rho2), 1.f + 1e-6f) + 1.6e-5f * (1.f + cmax);
}

// Shell sh in range of the sphere: mark the chunks and K blocks its
// (contiguous) functions fall in.  Out of range when |R_A - c|^2 >
// (radius + rho)^2, the right side widened by 1e-5 relative and 1e-4 Bohr^2
// against the rounding of both.
__device__ __forceinline__ void mark_shell(const DevBasis& B, int sh, const float cf[3], float rhof,
                                           unsigned char* chunk_on, unsigned char* kb_on) {
  const float4 at = __ldg(B.atom_f4 + __ldg(B.sh_atom + sh));
  const float dx = at.x - cf[0], dy = at.y - cf[1], dz = at.z - cf[2];
  const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
  const float reach = __ldg(B.sh_rad + sh) + rhof;
  const int nc = __ldg(B.sh_ncomp + sh);
  if (nc > 0 && !(d2 > fmaf(reach * reach, 1.00001f, 1e-4f))) {
    const int f0 = __ldg(B.sh_f0 + sh), f1 = f0 + nc - 1;
    for (int c = f0 / kChunkF; c <= f1 / kChunkF; ++c) chunk_on[c] = 1;
    for (int c = f0 / kBlockK; c <= f1 / kBlockK; ++c) kb_on[c] = 1;
  }
}

// The tile's lists out[0 .. stride) = {#chunks, #kblocks, chunk ids...,
// kblock ids...} from the marks, compacted in index order by one warp.
__device__ __forceinline__ void warp_write_lists(const DevBasis& B, const unsigned char* chunk_on,
                                                 const unsigned char* kb_on, int* out, int lane) {
  const int nkb = B.kpad / kBlockK;
  int nc = 0, nk = 0;
  for (int i0 = 0; i0 < B.nchunk; i0 += 32) {
    const int i = i0 + lane;
    const bool on = i < B.nchunk && chunk_on[i];
    const unsigned m = __ballot_sync(0xffffffffu, on);
    if (on) out[2 + nc + __popc(m & ((1u << lane) - 1u))] = i;
    nc += __popc(m);
  }
  for (int i0 = 0; i0 < nkb; i0 += 32) {
    const int i = i0 + lane;
    const bool on = i < nkb && kb_on[i];
    const unsigned m = __ballot_sync(0xffffffffu, on);
    if (on) out[2 + B.nchunk + nk + __popc(m & ((1u << lane) - 1u))] = i;
    nk += __popc(m);
  }
  if (lane == 0) {
    out[0] = nc;
    out[1] = nk;
  }
}

}  // namespace gg
