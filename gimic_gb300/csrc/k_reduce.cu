// Plane / volume quadrature of the current tensor field, following
// src/fgimic/integral.f90:50-186 (integrate_current), :190-324
// (integrate_modulus) and :414-511 (integrate_acid) with the ACID density of
// src/libgimic/acid.f90:11-43.  Row partial sums (over i) are formed by one
// block per (j, k) row with a fixed reduction tree, then summed over rows in
// order by a single block, all in fp64, so the result is deterministic.
#include "gg_kernels.h"

namespace gg {

namespace {
constexpr int kRowThreads = 128;
constexpr int kQ = 7;
}

__global__ void __launch_bounds__(kRowThreads) plane_rows_kernel(PlaneArgs a) {
  const int j = blockIdx.x, k = blockIdx.y;
  __shared__ double red[kQ][kRowThreads];
  double acc[kQ] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = threadIdx.x; i < a.p1; i += kRowThreads) {
    const int64_t idx = i + static_cast<int64_t>(a.p1) * (j + static_cast<int64_t>(a.p2) * k);
    const double* t = a.jt + 9 * idx;
    double jv[3];
    for (int m = 0; m < 3; ++m) jv[m] = t[m] * a.bb[0] + t[m + 3] * a.bb[1] + t[m + 6] * a.bb[2];
    const double* rr = a.pts + 3 * idx;
    const double dx = rr[0] - a.center[0], dy = rr[1] - a.center[1], dz = rr[2] - a.center[2];
    const double dist = sqrt(dx * dx + dy * dy + dz * dz);
    const bool inside = !(dist > a.radius);
    const double w = inside ? a.w1[i] : 0.0;
    const double jn = a.normal[0] * jv[0] + a.normal[1] * jv[1] + a.normal[2] * jv[2];
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
    const double acid = 0.3333333 * (xx * xx + yy * yy + zz * zz) + 0.5 * (xy * xy + xz * xz + yz * yz);
    acc[6] += acid * w;
  }
  for (int q = 0; q < kQ; ++q) red[q][threadIdx.x] = acc[q];
  __syncthreads();
  for (int s = kRowThreads / 2; s > 0; s >>= 1) {
    if (threadIdx.x < s)
      for (int q = 0; q < kQ; ++q) red[q][threadIdx.x] += red[q][threadIdx.x + s];
    __syncthreads();
  }
  if (threadIdx.x < kQ) {
    const double wj = a.w2[j];
    a.row_out[(static_cast<int64_t>(k) * a.p2 + j) * kQ + threadIdx.x] = red[threadIdx.x][0] * wj;
  }
}

__global__ void plane_sum_kernel(PlaneArgs a) {
  const int q = threadIdx.x;
  if (q >= kQ) return;
  double s3 = 0.0;
  for (int k = 0; k < a.p3; ++k) {
    double s2 = 0.0;
    for (int j = 0; j < a.p2; ++j) s2 += a.row_out[(static_cast<int64_t>(k) * a.p2 + j) * kQ + q];
    s3 = s3 + a.w3[k] * s2;
  }
  a.out[q] = s3;
}

void launch_plane_reduce(const PlaneArgs& a, cudaStream_t st) {
  dim3 grid(a.p2, a.p3);
  plane_rows_kernel<<<grid, kRowThreads, 0, st>>>(a);
  plane_sum_kernel<<<1, 32, 0, st>>>(a);
}

}  // namespace gg
