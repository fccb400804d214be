// Plane / volume quadrature of the current tensor field, following
// src/fgimic/integral.f90:50-186 (integrate_current), :190-324
// (integrate_modulus) and :414-511 (integrate_acid) with the ACID density of
// src/libgimic/acid.f90:11-43, for a batch of planes at once (bond-current
// profile scans).  Row partial sums (over i) are formed by one block per row
// with a fixed reduction tree and then summed over the rows with a fixed
// split and tree, all in fp64, so the result is deterministic.
#include "gg_kernels.h"

namespace gg {

namespace {
constexpr int kRowThreads = 128;
constexpr int kQ = 7;
}

// Contributions of one point (i of its row) to the seven sums.
__device__ __forceinline__ void point_terms(const double* t, const double* rr, const double* center,
                                            const double* normal, const double* bb, double radius, double wi,
                                            double acc[kQ]) {
  double jv[3];
  for (int m = 0; m < 3; ++m) jv[m] = t[m] * bb[0] + t[m + 3] * bb[1] + t[m + 6] * bb[2];
  const double dx = rr[0] - center[0], dy = rr[1] - center[1], dz = rr[2] - center[2];
  const double d2 = dx * dx + dy * dy + dz * dz;
  // !(|d| > radius) as the reference tests it; the square root only near
  // the boundary (and for a negative or NaN radius or distance)
  bool inside;
  if (radius >= 0.0 && d2 < radius * radius * (1.0 - 1e-12))
    inside = true;
  else if (radius >= 0.0 && d2 > radius * radius * (1.0 + 1e-12))
    inside = false;
  else
    inside = !(sqrt(d2) > radius);
  const double w = inside ? wi : 0.0;
  const double jn = normal[0] * jv[0] + normal[1] * jv[1] + normal[2] * jv[2];
  // current: jp = (n . j) w
  const double jp = inside ? jn * w : 0.0;
  acc[0] += jp;
  if (jp > 0.0) acc[1] += jp; else acc[2] += jp;
  // modulus with the sign of n . j (|n . j| < 1e-12 counts as 0)
  const double sgn = fabs(jn) < 1e-12 ? 0.0 : (jn > 0.0 ? 1.0 : -1.0);
  const double jm = sgn * sqrt(jv[0] * jv[0] + jv[1] * jv[1] + jv[2] * jv[2]);
  acc[3] += jm * w;
  if (jm > 0.0) acc[4] += jm * w; else acc[5] += jm * w;
  // ACID: 0.3333333 (diagonal differences) + 0.5 (off-diagonal sums)
  const double xx = t[0] - t[4], yy = t[4] - t[8], zz = t[8] - t[0];
  const double xy = t[3] + t[1], xz = t[6] + t[2], yz = t[7] + t[5];
  acc[6] += (0.3333333 * (xx * xx + yy * yy + zz * zz) + 0.5 * (xy * xy + xz * xz + yz * yz)) * w;
}

// The block's sums of the seven quantities: a fixed butterfly within each
// warp, then the warps' results in warp order (one barrier), times w_j.
__device__ __forceinline__ void block_reduce_store(double acc[kQ], double wj, double* dst) {
  __shared__ double red[kRowThreads / 32][kQ];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < kQ; ++q) {
    double v = acc[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[warp][q] = v;
  }
  __syncthreads();
  if (threadIdx.x < kQ) {
    double v = red[0][threadIdx.x];
    for (int w = 1; w < kRowThreads / 32; ++w) v += red[w][threadIdx.x];
    dst[threadIdx.x] = v * wj;
  }
}

// One block per row of one plane of a batch: the row's sums over i (fixed
// tree), times w_j, to row_out.  The block that finishes a plane's last row
// (counted in done[plane], zero at launch) then sums the plane's rows, each
// times w_k (the reference's s3 += w_k s2 over k of s2 over j,
// integral.f90:107-165, as one sum), with a fixed split and tree, so the
// plane's result does not depend on which block came last.
__global__ void __launch_bounds__(kRowThreads) plane_batch_kernel(const double* __restrict__ jt,
                                                                  const double* __restrict__ pts,
                                                                  const double* __restrict__ w,
                                                                  const PlaneDesc* __restrict__ planes,
                                                                  const int* __restrict__ row_plane,
                                                                  const double* __restrict__ field, double* row_out,
                                                                  double* __restrict__ out, unsigned* done) {
  const int64_t row = blockIdx.x;
  const int q = row_plane[row];
  const PlaneDesc& pl = planes[q];
  const int64_t r = row - pl.row_off;
  const int j = static_cast<int>(r % pl.p2), k = static_cast<int>(r / pl.p2);
  const double bb[3] = {field[0], field[1], field[2]};
  double acc[kQ] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < pl.p1; i += kRowThreads) {
    const int64_t idx = pl.pt_off + i + static_cast<int64_t>(pl.p1) * (j + static_cast<int64_t>(pl.p2) * k);
    point_terms(jt + 9 * idx, pts + 3 * idx, pl.center, pl.normal, bb, pl.radius, w[pl.w_off + i], acc);
  }
  block_reduce_store(acc, w[pl.w_off + pl.p1 + j], row_out + row * kQ);
  __threadfence();  // this row's sums are visible before it is counted
  __shared__ bool last;
  __syncthreads();
  const int64_t nr = static_cast<int64_t>(pl.p2) * pl.p3;
  if (threadIdx.x == 0) last = atomicAdd(done + q, 1u) == static_cast<unsigned>(nr - 1);
  __syncthreads();
  if (!last) return;
  __threadfence();
  // the plane's sums: sum over k of w_k times the sum over j of its rows,
  // taken as one sum over the rows, each times the w_k of its k; thread t
  // adds rows t, t + 128, ... in order, then the fixed block tree
  const double* wk = w + pl.w_off + pl.p1 + pl.p2;
  double s[kQ] = {0, 0, 0, 0, 0, 0, 0};
  for (int64_t rr = threadIdx.x; rr < nr; rr += kRowThreads) {
    const double f = wk[rr / pl.p2];
    const double* src = row_out + (pl.row_off + rr) * kQ;
#pragma unroll
    for (int c = 0; c < kQ; ++c) s[c] += f * __ldcg(src + c);
  }
  block_reduce_store(s, 1.0, out + q * kQ);
  if (threadIdx.x == 0) done[q] = 0;
}

__global__ void __launch_bounds__(kRowThreads) plane_points_kernel(const double* __restrict__ xs,
                                                                   const PlaneDesc* __restrict__ planes,
                                                                   const int* __restrict__ row_plane,
                                                                   double* __restrict__ pts, unsigned* done,
                                                                   int nplanes) {
  const int64_t row = blockIdx.x;
  if (row == 0)
    for (int q = threadIdx.x; q < nplanes; q += kRowThreads) done[q] = 0;
  const PlaneDesc& pl = planes[row_plane[row]];
  const int64_t r = row - pl.row_off;
  const int j = static_cast<int>(r % pl.p2), k = static_cast<int>(r / pl.p2);
  const double x2 = xs[pl.x_off + pl.p1 + j], x3 = xs[pl.x_off + pl.p1 + pl.p2 + k];
  for (int i = threadIdx.x; i < pl.p1; i += kRowThreads) {
    const double x1 = xs[pl.x_off + i];
    const int64_t idx = pl.pt_off + i + static_cast<int64_t>(pl.p1) * (j + static_cast<int64_t>(pl.p2) * k);
    for (int c = 0; c < 3; ++c)
      pts[3 * idx + c] = __dadd_rn(__dadd_rn(__dadd_rn(pl.origin[c], __dmul_rn(x1, pl.basv[c])),
                                             __dmul_rn(x2, pl.basv[3 + c])),
                                   __dmul_rn(x3, pl.basv[6 + c]));
  }
}

void launch_plane_points(const double* xs, const PlaneDesc* planes, const int* row_plane, int64_t nrows, double* pts,
                         unsigned* done, int nplanes, cudaStream_t st) {
  if (nrows <= 0) return;
  plane_points_kernel<<<static_cast<unsigned>(nrows), kRowThreads, 0, st>>>(xs, planes, row_plane, pts, done,
                                                                             nplanes);
}

void launch_plane_batch(const double* jt, const double* pts, const double* w, const PlaneDesc* planes, int nplanes,
                        const int* row_plane, int64_t nrows, const double* field, double* row_out, double* out,
                        unsigned* done, cudaStream_t st) {
  if (nplanes <= 0) return;
  plane_batch_kernel<<<static_cast<unsigned>(nrows), kRowThreads, 0, st>>>(jt, pts, w, planes, row_plane, field,
                                                                            row_out, out, done);
}

// ---------------------------------------------------------------------------
// Property quadratures over a molecular grid (src/fgimic/jfield.f90:584-929,
// get_property): nuclear shielding of every centre and the magnetizability,
// both from the current tensor with the field along -x, -y, -z.  Points come
// in consecutive blocks (one per atom of the grid generator); one CTA sums one
// (centre, block) pair, or one block for the magnetizability, with a fixed
// tree in fp64, so the sums are deterministic.
//   sigma_a(K) = sum_i w_i 1e6 f_i ((r_i - R_K) x j_i^(a))_a,
//   f_i = -1 / |r_i - R_K|^3 / c^2,  c = 137.0359998,  j^(a) = t . (-e_a);
//   chi_a = sum_i w_i 0.5 (r_i x j_i^(a))_a.
// Each output record holds the three diagonal sums and the positive and
// negative parts of sum_a (per-point value) w_i.
// ---------------------------------------------------------------------------
namespace {
constexpr int kPropThreads = 128;
constexpr int kPropQ = 5;

__device__ __forceinline__ void prop_block_reduce(double acc[kPropQ], double* dst) {
  __shared__ double red[kPropQ][kPropThreads];
  for (int q = 0; q < kPropQ; ++q) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int s = kPropThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int q = 0; q < kPropQ; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < kPropQ) dst[threadIdx.x] = red[threadIdx.x][0];
}

// (d x j^(a))_a for the field along -e_a, j^(a)_m = -t(m, a) = -t[m + 3a]
__device__ __forceinline__ void cross_diag(const double* t, const double d[3], double out[3]) {
  out[0] = -(d[1] * t[2 + 0] - d[2] * t[1 + 0]);
  out[1] = -(d[2] * t[0 + 3] - d[0] * t[2 + 3]);
  out[2] = -(d[0] * t[1 + 6] - d[1] * t[0 + 6]);
}
}  // namespace

__global__ void __launch_bounds__(kPropThreads) prop_sigma_kernel(const double* __restrict__ jt,
                                                                  const double* __restrict__ pts,
                                                                  const double* __restrict__ w,
                                                                  const double* __restrict__ centres,
                                                                  const int64_t* __restrict__ block_off, int nblocks,
                                                                  double* __restrict__ out) {
  const int k = blockIdx.y, l = blockIdx.x;
  const double R[3] = {centres[3 * k], centres[3 * k + 1], centres[3 * k + 2]};
  const double c2 = 137.0359998 * 137.0359998;
  double acc[kPropQ] = {0, 0, 0, 0, 0};
  for (int64_t i = block_off[l] + threadIdx.x; i < block_off[l + 1]; i += kPropThreads) {
    const double d[3] = {pts[3 * i] - R[0], pts[3 * i + 1] - R[1], pts[3 * i + 2] - R[2]};
    const double r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    const double f = -1.0 / (r2 * sqrt(r2)) / c2;
    double c[3];
    cross_diag(jt + 9 * i, d, c);
    double sum = 0.0;
    for (int a = 0; a < 3; ++a) {
      const double v = 1.0e6 * f * c[a];
      acc[a] += w[i] * v;
      sum += v;
    }
    if (sum >= 0.0) acc[3] += sum * w[i]; else acc[4] += sum * w[i];
  }
  prop_block_reduce(acc, out + (static_cast<int64_t>(k) * nblocks + l) * kPropQ);
}

__global__ void __launch_bounds__(kPropThreads) prop_chi_kernel(const double* __restrict__ jt,
                                                                const double* __restrict__ pts,
                                                                const double* __restrict__ w,
                                                                const int64_t* __restrict__ block_off,
                                                                double* __restrict__ out) {
  const int l = blockIdx.x;
  double acc[kPropQ] = {0, 0, 0, 0, 0};
  for (int64_t i = block_off[l] + threadIdx.x; i < block_off[l + 1]; i += kPropThreads) {
    const double r[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    double c[3];
    cross_diag(jt + 9 * i, r, c);
    double sum = 0.0;
    for (int a = 0; a < 3; ++a) {
      const double v = 0.5 * c[a];
      acc[a] += w[i] * v;
      sum += v;
    }
    if (sum >= 0.0) acc[3] += sum * w[i]; else acc[4] += sum * w[i];
  }
  prop_block_reduce(acc, out + static_cast<int64_t>(l) * kPropQ);
}

void launch_properties(const double* jt, const double* pts, const double* w, const double* centres, int ncentres,
                       const int64_t* block_off, int nblocks, double* sigma_out, double* chi_out, cudaStream_t st) {
  if (nblocks <= 0) return;
  if (ncentres > 0)
    prop_sigma_kernel<<<dim3(static_cast<unsigned>(nblocks), static_cast<unsigned>(ncentres)), kPropThreads, 0, st>>>(
        jt, pts, w, centres, block_off, nblocks, sigma_out);
  prop_chi_kernel<<<static_cast<unsigned>(nblocks), kPropThreads, 0, st>>>(jt, pts, w, block_off, chi_out);
}

}  // namespace gg
