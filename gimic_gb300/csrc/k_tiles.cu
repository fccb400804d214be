// Tile-level exponent screening for the tensor-core contraction.
//
// The reference screens per point and per contraction: a shell contributes
// to a point only within its screening radius (src/libgimic/basis.f90:90-136,
// used by bfeval/dfdr).  For a compact tile of points, every shell that is
// out of range for the whole tile contributes exact zeros both to the GEMM
// (its rows of the point operand are zero: those K blocks can be skipped) and
// to the epilogue (its columns are multiplied by zero basis values: those
// column chunks can be skipped).  Skipping them changes no result.
//
//  1. morton_key_kernel + a radix sort order the points along a Z curve so
//     that 128 consecutive points form a compact tile;
//  2. gather_kernel copies the points into that order;
//  3. tile_screen_kernel lists, per tile (one warp each), the active
//     32-function column chunks and 64-function K blocks with a conservative
//     bounding-sphere test.
#include <cub/device/device_radix_sort.cuh>

#include "gg_kernels.h"
#include "gg_tiles.cuh"

namespace gg {

namespace {
__device__ __forceinline__ uint32_t spread3(uint32_t v) {
  v &= 0x3ffu;
  v = (v | (v << 16)) & 0x030000ffu;
  v = (v | (v << 8)) & 0x0300f00fu;
  v = (v | (v << 4)) & 0x030c30c3u;
  v = (v | (v << 2)) & 0x09249249u;
  return v;
}
}  // namespace

// The cell of a coordinate in fp32 (one conversion from fp64 per coordinate:
// this GPU's FP64 pipe is narrow, and the order is a heuristic, so a point
// within a few 1e-6 Bohr of a cell boundary may fall on either side).
__global__ void morton_key_kernel(const double* __restrict__ pts, int64_t n, float lox, float loy, float loz,
                                  float inv_cell, uint32_t* __restrict__ keys, int* __restrict__ idx) {
  const int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const float lo[3] = {lox, loy, loz};
  uint32_t c[3];
  for (int d = 0; d < 3; ++d) {
    const float q = (__double2float_rn(pts[3 * p + d]) - lo[d]) * inv_cell;
    c[d] = static_cast<uint32_t>(fminf(fmaxf(q, 0.f), 1023.f));  // NaN goes to 0; far points share edge cells
  }
  keys[p] = spread3(c[0]) | (spread3(c[1]) << 1) | (spread3(c[2]) << 2);
  idx[p] = static_cast<int>(p);
}

// Four points per thread: the four indices in one load, then twelve
// independent coordinate loads in flight (the loads through perm are a
// latency chain), and the 96 contiguous output bytes in six 16-byte stores.
__global__ void gather_kernel(const double* __restrict__ pts, const int* __restrict__ perm, int64_t n,
                              double* __restrict__ out) {
  const int64_t p0 = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) * 4;
  if (p0 >= n) return;
  if (p0 + 4 <= n) {
    const int4 s = *reinterpret_cast<const int4*>(perm + p0);  // perm is 16-byte aligned, p0 a multiple of 4
    const int64_t src[4] = {s.x, s.y, s.z, s.w};
    double v[12];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
      for (int c = 0; c < 3; ++c) v[3 * k + c] = pts[3 * src[k] + c];
    double2* o = reinterpret_cast<double2*>(out + 3 * p0);  // 96 p0 / 4 bytes: 16-byte aligned
#pragma unroll
    for (int k = 0; k < 6; ++k) o[k] = make_double2(v[2 * k], v[2 * k + 1]);
  } else {
    for (int64_t p = p0; p < n; ++p) {
      const int64_t s = perm[p];
      out[3 * p] = pts[3 * s];
      out[3 * p + 1] = pts[3 * s + 1];
      out[3 * p + 2] = pts[3 * s + 2];
    }
  }
}

// One warp per tile, four tiles per block of 128 threads: the tile's
// bounding sphere, every shell against it, and the lists tiles[t * stride]
// = {#chunks, #kblocks, chunk ids..., kblock ids...} (gg_tiles.cuh).
__global__ void __launch_bounds__(128) tile_screen_kernel(DevBasis B, const double* __restrict__ pts, int64_t n,
                                                          int64_t ntiles, int stride, int* __restrict__ tiles,
                                                          unsigned long long* __restrict__ xneed) {
  extern __shared__ unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nkb = B.kpad / kBlockK;
  const int64_t t = static_cast<int64_t>(blockIdx.x) * 4 + warp;
  if (t >= ntiles) return;  // the whole warp
  if (xneed && lane < 2) xneed[2 * t + lane] = ~0ull;  // every half K block needs cross products until shown small
  unsigned char* chunk_on = smem_raw + warp * (B.nchunk + nkb);  // nchunk
  unsigned char* kb_on = chunk_on + B.nchunk;                      // kpad / 64
  float cf[3], rhof;
  warp_tile_sphere(pts, n, t, lane, cf, &rhof);
  for (int i = lane; i < B.nchunk; i += 32) chunk_on[i] = 0;
  for (int i = lane; i < nkb; i += 32) kb_on[i] = 0;
  __syncwarp();
  for (int sh = lane; sh < B.nshells; sh += 32) mark_shell(B, sh, cf, rhof, chunk_on, kb_on);
  __syncwarp();
  warp_write_lists(B, chunk_on, kb_on, tiles + t * stride, lane);
}

// Sum over tiles of (active chunks x active K blocks): the number of
// (224-column, 64-deep) GEMM blocks the contraction issues, for profiling.
__global__ void tile_work_kernel(const int* __restrict__ tiles, int64_t ntiles, int stride,
                                 unsigned long long* __restrict__ acc) {
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  unsigned long long v = 0;
  if (t < ntiles) v = static_cast<unsigned long long>(tiles[t * stride]) * tiles[t * stride + 1];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(acc, v);
}

void launch_tile_work(const int* tiles, int64_t ntiles, int stride, unsigned long long* acc, cudaStream_t st) {
  tile_work_kernel<<<static_cast<unsigned>((ntiles + 255) / 256), 256, 0, st>>>(tiles, ntiles, stride, acc);
}

__global__ void cross_work_kernel(const int* __restrict__ tiles, const unsigned long long* __restrict__ xneed,
                                  int64_t ntiles, int stride, int nchunk, unsigned long long* __restrict__ acc) {
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  unsigned long long v = 0;
  if (t < ntiles) {
    const int* tl = tiles + t * stride;
    const int nk = tl[1];
    int n = 0;
    for (int i = 0; i < nk; ++i) {
      const int h = 2 * tl[2 + nchunk + i];
      n += ((xneed[2 * t + (h >> 6)] >> (h & 63)) & 3ull) != 0;
    }
    v = static_cast<unsigned long long>(tl[0]) * n;
  }
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(acc, v);
}

void launch_cross_work(const int* tiles, const unsigned long long* xneed, int64_t ntiles, int stride, int nchunk,
                       unsigned long long* acc, cudaStream_t st) {
  cross_work_kernel<<<static_cast<unsigned>((ntiles + 255) / 256), 256, 0, st>>>(tiles, xneed, ntiles, stride,
                                                                                  nchunk, acc);
}

int tile_stride(const DevBasis& B) { return 2 + B.nchunk + B.kpad / kBlockK; }

__global__ void tile_work_keys_kernel(const int* __restrict__ tiles, int64_t ntiles, int stride,
                                      uint32_t* __restrict__ work, int* __restrict__ ids) {
  const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  work[t] = static_cast<uint32_t>(tiles[t * stride]) * static_cast<uint32_t>(tiles[t * stride + 1]);
  ids[t] = static_cast<int>(t);
}

size_t tile_order_temp_bytes(int64_t ntiles) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairsDescending(nullptr, bytes, static_cast<const uint32_t*>(nullptr),
                                            static_cast<uint32_t*>(nullptr), static_cast<const int*>(nullptr),
                                            static_cast<int*>(nullptr), static_cast<int>(ntiles), 0, 20);
  return bytes;
}

cudaError_t launch_tile_order(const int* tiles, int64_t ntiles, int stride, uint32_t* work, uint32_t* work_sorted,
                              int* ids, int* order, void* temp, size_t temp_bytes, cudaStream_t st) {
  tile_work_keys_kernel<<<static_cast<unsigned>((ntiles + 255) / 256), 256, 0, st>>>(tiles, ntiles, stride, work, ids);
  return cub::DeviceRadixSort::SortPairsDescending(temp, temp_bytes, work, work_sorted, ids, order,
                                                   static_cast<int>(ntiles), 0, 20, st);
}

size_t sort_temp_bytes(int64_t n) {
  size_t bytes = 0;
  cub::DeviceRadixSort::SortPairs(nullptr, bytes, static_cast<const uint32_t*>(nullptr),
                                  static_cast<uint32_t*>(nullptr), static_cast<const int*>(nullptr),
                                  static_cast<int*>(nullptr), static_cast<int>(n), 0, 30);
  return bytes;
}

cudaError_t launch_spatial_order(const double* pts, int64_t n, const double lo[3], double cell, uint32_t* keys,
                                 uint32_t* keys_sorted, int* idx, int* perm, void* temp, size_t temp_bytes,
                                 double* pts_sorted, cudaStream_t st) {
  const unsigned blocks = static_cast<unsigned>((n + 255) / 256);
  morton_key_kernel<<<blocks, 256, 0, st>>>(pts, n, static_cast<float>(lo[0]), static_cast<float>(lo[1]),
                                            static_cast<float>(lo[2]), static_cast<float>(1.0 / cell), keys, idx);
  cudaError_t e = cub::DeviceRadixSort::SortPairs(temp, temp_bytes, keys, keys_sorted, idx, perm, static_cast<int>(n),
                                                  0, 30, st);
  if (e != cudaSuccess) return e;
  gather_kernel<<<static_cast<unsigned>((n + 1023) / 1024), 256, 0, st>>>(pts, perm, n, pts_sorted);
  return cudaGetLastError();
}

void launch_tile_screen(const DevBasis& B, const double* pts_sorted, int64_t n, int* tiles, unsigned long long* xneed,
                        cudaStream_t st) {
  const int64_t ntiles = (n + kBlockM - 1) / kBlockM;
  if (ntiles <= 0) return;
  const size_t smem = 4 * static_cast<size_t>(B.nchunk + B.kpad / kBlockK);
  const unsigned blocks = static_cast<unsigned>((ntiles + 3) / 4);
  tile_screen_kernel<<<blocks, 128, smem, st>>>(B, pts_sorted, n, ntiles, tile_stride(B), tiles, xneed);
}

}  // namespace gg
