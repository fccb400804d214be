// Plain FP64 GPU path: W = phi^T [D | C | P] as an FP64 SIMT GEMM, then a
// warp-per-point assembly of the bilinear forms and their FP64 combination.
// This path is the accuracy baseline of the split-precision tensor-core path
// and the "plain FP64 GPU path" the throughput target is measured against.
// With tile screening it skips the same work as the split path: the points
// are in the split path's Z order, dgemm_tiles_kernel forms W only for each
// tile's active column chunks over its active K blocks, and the assembly
// walks only the active chunks (the skipped basis values are exact zeros).
#include "gg_combine.cuh"
#include "gg_kernels.h"

namespace gg {

namespace {
constexpr int kTM = 64, kTN = 64, kTK = 16;
}

// 64x64 output tile per 256-thread block, 4x4 register tile per thread.
__global__ void __launch_bounds__(256) dgemm_kernel(const double* __restrict__ A, int64_t lda,
                                                    const double* __restrict__ B, int64_t ldb, double* __restrict__ C,
                                                    int64_t ldc, int64_t M, int64_t N, int64_t K) {
  __shared__ double As[kTK][kTM + 1];
  __shared__ double Bs[kTK][kTN + 1];
  const int tx = threadIdx.x % 16, ty = threadIdx.x / 16;
  const int64_t m0 = static_cast<int64_t>(blockIdx.y) * kTM, n0 = static_cast<int64_t>(blockIdx.x) * kTN;
  double acc[4][4] = {};
  for (int64_t k0 = 0; k0 < K; k0 += kTK) {
    for (int i = threadIdx.x; i < kTM * kTK; i += 256) {
      const int mm = i / kTK, kk = i % kTK;
      const int64_t gm = m0 + mm, gk = k0 + kk;
      As[kk][mm] = (gm < M && gk < K) ? A[gm * lda + gk] : 0.0;
    }
    for (int i = threadIdx.x; i < kTN * kTK; i += 256) {
      const int kk = i / kTN, nn = i % kTN;
      const int64_t gk = k0 + kk, gn = n0 + nn;
      Bs[kk][nn] = (gk < K && gn < N) ? B[gk * ldb + gn] : 0.0;
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kTK; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[kk][ty + 16 * i];
#pragma unroll
      for (int j = 0; j < 4; ++j) b[j] = Bs[kk][tx + 16 * j];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int64_t gm = m0 + ty + 16 * i, gn = n0 + tx + 16 * j;
      if (gm < M && gn < N) C[gm * ldc + gn] = acc[i][j];
    }
}

void launch_dgemm(const double* A, int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc, int64_t M,
                  int64_t N, int64_t K, cudaStream_t st) {
  if (M <= 0 || N <= 0) return;
  dim3 grid(static_cast<unsigned>((N + kTN - 1) / kTN), static_cast<unsigned>((M + kTM - 1) / kTM));
  dgemm_kernel<<<grid, 256, 0, st>>>(A, lda, B, ldb, C, ldc, M, N, K);
}

namespace {
constexpr int kQM = 64, kQN = 32;  // one output block: half a tile x the 32 functions of a chunk
}

// W[p, m ld + c 32 + j] = sum over the tile's active K blocks k of
// phi[p, k] M[k, m ld + c 32 + j] for every active chunk c of the tile of
// point p.  Grid (2 ntiles, nchunk, 7): block x is half a tile, y the
// tile's y-th active chunk (none past its count), z the matrix m.  128
// threads, 4 x 4 outputs each.  Columns of inactive chunks are not written.
__global__ void __launch_bounds__(128) dgemm_tiles_kernel(const double* __restrict__ phi, int64_t ld,
                                                          const double* __restrict__ M, int64_t ldm,
                                                          double* __restrict__ W, int64_t ldw, int64_t n, int nbf,
                                                          const int* __restrict__ tiles, int stride, int nchunk) {
  __shared__ double As[kTK][kQM + 1];
  __shared__ double Bs[kTK][kQN + 1];
  const int64_t t = blockIdx.x >> 1;
  const int* tl = tiles + t * stride;
  if (static_cast<int>(blockIdx.y) >= tl[0]) return;
  const int c = tl[2 + blockIdx.y], nk = tl[1];
  const int* kl = tl + 2 + nchunk;
  const int64_t r0 = t * 128 + (blockIdx.x & 1) * kQM;
  const int64_t col0 = static_cast<int64_t>(blockIdx.z) * ld + c * 32;  // column of the block's first function
  const int f0 = c * 32;
  const int tx = threadIdx.x % 8, ty = threadIdx.x / 8;  // columns tx + 8 j, rows ty + 16 i
  double acc[4][4] = {};
  for (int i = 0; i < nk; ++i) {
    for (int k0 = kl[i] * 64; k0 < kl[i] * 64 + 64; k0 += kTK) {
      for (int e = threadIdx.x; e < kQM * kTK; e += 128) {
        const int mm = e / kTK, kk = e % kTK;
        const int64_t gr = r0 + mm, gk = k0 + kk;
        As[kk][mm] = (gr < n && gk < nbf) ? phi[gr * ld + gk] : 0.0;
      }
      for (int e = threadIdx.x; e < kQN * kTK; e += 128) {
        const int kk = e / kQN, nn = e % kQN;
        const int64_t gk = k0 + kk;
        Bs[kk][nn] = (gk < nbf && f0 + nn < nbf) ? M[gk * ldm + col0 + nn] : 0.0;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < kTK; ++kk) {
        double a[4], b[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) a[q] = As[kk][ty + 16 * q];
#pragma unroll
        for (int q = 0; q < 4; ++q) b[q] = Bs[kk][tx + 8 * q];
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
          for (int u = 0; u < 4; ++u) acc[q][u] = fma(a[q], b[u], acc[q][u]);
      }
      __syncthreads();
    }
  }
#pragma unroll
  for (int q = 0; q < 4; ++q)
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const int64_t gr = r0 + ty + 16 * q;
      const int fn = f0 + tx + 8 * u;
      if (gr < n && fn < nbf) W[gr * ldw + col0 + tx + 8 * u] = acc[q][u];
    }
}

void launch_dgemm_tiles(const double* phi, int64_t ld, const double* M, int64_t ldm, double* W, int64_t ldw,
                        int64_t n, int nbf, const int* tiles, int stride, int nchunk, cudaStream_t st) {
  if (n <= 0) return;
  const int64_t ntiles = (n + 127) / 128;
  dim3 grid(static_cast<unsigned>(2 * ntiles), static_cast<unsigned>(nchunk), 7u);
  dgemm_tiles_kernel<<<grid, 128, 0, st>>>(phi, ld, M, ldm, W, ldw, n, nbf, tiles, stride, nchunk);
}

// One warp per point: lanes stride over basis functions and accumulate the
// kNDots bilinear forms in fp64; lane 0 combines and stores.  With tile
// lists (points in Z order) the lanes walk only the active chunks of the
// point's tile, and the outputs go to perm[p] (the caller's order).
__global__ void __launch_bounds__(256) assemble_fp64_kernel(DevBasis Bs, const double* __restrict__ pts, int64_t npts,
                                                            const double* __restrict__ W, int64_t ldw,
                                                            const double* __restrict__ phi,
                                                            const double* __restrict__ gx,
                                                            const double* __restrict__ gy,
                                                            const double* __restrict__ gz,
                                                            const double* __restrict__ lap, int64_t ld, Flags fl,
                                                            Outputs out, const int* __restrict__ tiles, int stride,
                                                            const int* __restrict__ perm) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t p = static_cast<int64_t>(blockIdx.x) * 8 + warp;
  if (p >= npts) return;
  const double r[3] = {pts[3 * p], pts[3 * p + 1], pts[3 * p + 2]};
  const int n = Bs.nbf;
  double d[kNDots];
#pragma unroll
  for (int i = 0; i < kNDots; ++i) d[i] = 0.0;
  const double* w = W + p * ldw;
  const int* tl = tiles ? tiles + (p / 128) * stride : nullptr;
  const int nsteps = tl ? tl[0] : (n + 31) / 32;  // active chunks, or all functions 32 at a time
  for (int step = 0; step < nsteps; ++step) {
    const int mu = (tl ? tl[2 + step] * 32 : step * 32) + lane;
    if (mu >= n) continue;
    const int64_t o = p * ld + mu;
    const double f = phi[o], g[3] = {gx[o], gy[o], gz[o]}, l = lap[o];
    const int a = __ldg(Bs.sh_atom + __ldg(Bs.f_shell + mu));
    const double s[3] = {r[0] - Bs.atom_xyz[3 * a], r[1] - Bs.atom_xyz[3 * a + 1], r[2] - Bs.atom_xyz[3 * a + 2]};
    const double w0 = w[mu];
    d[0] += w0 * f;
#pragma unroll
    for (int c = 0; c < 3; ++c) d[1 + c] += w0 * s[c] * f;
#pragma unroll
    for (int m = 0; m < 3; ++m)
#pragma unroll
      for (int c = 0; c < 3; ++c)
        if (m != c) d[4 + 3 * m + c] += w0 * s[c] * g[m];
#pragma unroll
    for (int dd = 0; dd < 3; ++dd) {
      const double wc = w[(1 + dd) * n + mu];
#pragma unroll
      for (int m = 0; m < 3; ++m) d[13 + 3 * dd + m] += wc * g[m];
      d[22 + dd] += wc * l;
    }
#pragma unroll
    for (int b = 0; b < 3; ++b) {
      const double q = w[(4 + b) * n + mu];
#pragma unroll
      for (int m = 0; m < 3; ++m) d[25 + 3 * b + m] += q * g[m];
      d[34 + b] += q * l;
    }
  }
#pragma unroll
  for (int i = 0; i < kNDots; ++i)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) d[i] += __shfl_xor_sync(0xffffffffu, d[i], o);
  if (lane == 0) {
    double ct[9], dv[3];
    combine_point(d, r, fl, ct, dv);
    store_outputs(out, perm ? static_cast<int64_t>(perm[p]) : p, ct, d[0], dv);
  }
}

void launch_assemble_fp64(const DevBasis& B, const double* pts, int64_t npts, const double* W, int64_t ldw,
                          const double* phi, const double* gx, const double* gy, const double* gz, const double* lap,
                          int64_t ld, Flags fl, Outputs out, const int* tiles, int stride, const int* perm,
                          cudaStream_t st) {
  if (npts <= 0) return;
  assemble_fp64_kernel<<<static_cast<unsigned>((npts + 7) / 8), 256, 0, st>>>(B, pts, npts, W, ldw, phi, gx, gy, gz,
                                                                              lap, ld, fl, out, tiles, stride, perm);
}

}  // namespace gg
