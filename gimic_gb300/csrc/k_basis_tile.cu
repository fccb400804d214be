// Shell-blocked basis evaluation for the split-FP16 point operand.
//
// One CTA handles one tile of 128 consecutive points (the M tile of the
// tensor-core contraction), one thread per point (passes with fewer tiles
// than two per SM use basis_tile_short_kernel below, which splits a tile's
// K range over several CTAs and a point's shells over four threads).  All threads walk the
// shells in the same order (uniform control flow, shell data broadcast), so
// each thread evaluates the radial factor of a shell once and then its
// Cartesian components (bfeval.f90:81-122 with the per-shell screening of
// basis.f90:118-136).  Geometry is double-float fp32 (no FP64 pipe work per
// shell).
//
// The row's power-of-two scale has to be known before the first value is
// written, so a first pass computes an upper bound of max_mu |phi_mu| in the
// log domain, without exponentials:
//   |x^i y^j z^k sum_p c_p e^{-a_p d^2}| <= d^l npf max_p |c_p| e^{-a_p d^2},
// read per atom from a host-built envelope of its shells' bounds over bins
// of log2 d^2 (one lookup per atom instead of a walk over the shells and
// primitives).  The scale puts that bound just under 2^14.  When the bound
// exceeds the true row maximum by 2^k, the values whose fp16 lo part is
// subnormal are stored with an absolute error of at most 2^(k-38) times the
// row maximum.  The per-shell bound exceeds the maximum by 2^0.05..2^3.8 on
// the seeded bases (checked against the oracle's basis values) and the
// envelope adds at most 2.4 bits (median 0.1), so k < 7: far below 1e-9 of
// the maximum.
//
// Values go to a 16 KiB shared-memory tile (hi and lo halves of 128 rows x
// 32 columns, 64-byte swizzle), and every finished half K block is written
// to HBM with a TMA tensor store; the global layout is the plain row-major
// one the contraction loads in 64-column boxes.  Staging 32 columns instead
// of 64 halves the shared memory per CTA, so 10 CTAs (40 warps) fit an SM
// instead of 6 (1.92 -> 1.59 ms per 2^21 points).  With tile screening on,
// K blocks that are inactive for the tile (all their shells out of range
// for every point) are neither staged nor stored: the contraction never
// reads them.
#include <cuda.h>

#include <algorithm>
#include <type_traits>

#include "gg_cart.cuh"
#include "gg_device.cuh"
#include "gg_kernels.h"
#include "gg_once.h"
#include "gg_tiles.cuh"

namespace gg {

namespace {

constexpr int kTileThreads = kBlockM;                   // one thread per point of the tile
constexpr int kHalfK = kBlockK / 2;                     // columns staged and stored at a time
constexpr int kStageBytes = kBlockM * kHalfK * 2;       // one 128 x 32 fp16 tile: 8 KiB
constexpr int kBufBytes = 2 * kStageBytes;              // hi + lo
constexpr int kTileSmem = kBufBytes + 1024;             // one buffer + alignment slack
constexpr int kMaxScreenChunks = 4096 / kChunkF;        // chunks a short pass screens in the kernel
// the short kernel's screening marks and the tile's sphere (centre, radius)
struct ScreenSmem {
  float sph[4];
  unsigned char chunk[kMaxScreenChunks], kb[64];
};

__device__ __forceinline__ void tma_store_2d(const void* tmap, const void* src, int c0, int c1) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%2, %3}], [%1];" ::"l"(
                   reinterpret_cast<uint64_t>(tmap)),
               "r"(smem_u32(src)), "r"(c0), "r"(c1)
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// wait until no committed group still reads shared memory
__device__ __forceinline__ void bulk_wait_read_0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// byte offset of column pair (col, col + 1) of row `row` in a 64B-swizzled
// 128 x 32 fp16 tile: 16-byte chunk c of row r sits at chunk c ^ ((r >> 1) & 3)
__device__ __forceinline__ uint32_t swz(int row, int col) {
  const int byte = col * 2;
  return static_cast<uint32_t>(row * 64 + ((((byte >> 4) ^ ((row >> 1) & 3)) << 4) | (byte & 15)));
}

// byte offset of column col of the row whose offset is rowoff = row * 64
// and swizzle bits rxs = ((row >> 1) & 3) << 4 (the same as swz)
__device__ __forceinline__ uint32_t swz_col(uint32_t rowoff, uint32_t rxs, int col) {
  return rowoff + ((static_cast<uint32_t>(col) << 1) ^ rxs);
}

// the current atom of a point's shell walk: r - R_A (fp32 high parts, with
// squares) and |r - R_A|^2 as a double-float
struct AtomGeom {
  int atom = -1;
  CartPow cp = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  DFloat d2{0.f, 0.f};
};

// One point's values of the shells that overlap the columns [lo, hi) of a
// half K block, every kStep-th shell from the first one there plus
// `first`.  put(col, v) stages value v at column col - lo; the columns of
// shells out of range for the whole warp keep the zeros the row starts with.
// The shells in the standard Cartesian order (bit 24 of the shell record)
// evaluate their components with compile-time monomials; the others select
// the monomial from the packed exponents.  Both give x^i y^j z^k f1 with the
// same operations in the same order.
template <int kStep, typename Put>
__device__ __forceinline__ void stage_shells(const DevBasis& B, const float2 rg[3], float scale, int lo, int hi,
                                             int first, AtomGeom& g, Put&& put) {
  for (int sh = __ldg(B.f_shell + lo) + first; sh < B.nshells; sh += kStep) {
    const int4 pk = __ldg(B.sh_pack + sh);  // atom, first function, ncomp | npf << 8 | l << 16 | std << 24, first primitive
    const int mu0 = pk.y, ncomp = pk.z & 0xff, np = (pk.z >> 8) & 0xff;
    if (mu0 >= hi) break;  // shells are in function order
    const int c0 = max(0, lo - mu0), c1 = min(ncomp, hi - mu0);
    if (pk.x != g.atom) {
      g.atom = pk.x;
      float s3[3];
      g.d2 = atom_offset_g(rg, B.atom_g, pk.x, s3);
      g.cp = cart_pow(s3[0], s3[1], s3[2]);
    }
    float f1 = 0.f;
    const bool in_range = df_le(g.d2, __ldg(B.sh_rad2_df + sh));
    if (in_range) {
      for (int k = 0; k < np; ++k) {
        const float4 pr = __ldg(B.p_pack + pk.w + k);  // exponent hi, exponent lo, coefficient
        f1 += pr.z * gauss_df(pr.x, pr.y, g.d2.h, g.d2.l);
      }
      f1 *= scale;
    }
    const int col0 = mu0 - lo;
    if (!__any_sync(0xffffffffu, in_range)) continue;  // its columns stay as zeroed
    if ((pk.z >> 24) & 1) {
      const CartPow& cp = g.cp;
      auto comps = [&](auto basec, auto ncc) {
        static_for<0, decltype(ncc)::value>([&](auto kc) {
          constexpr int c = decltype(kc)::value;
          constexpr int code = kCartStdCode[decltype(basec)::value + c];
          constexpr int A = code / 100, Bx = (code / 10) % 10, C = code % 10;
          if (c >= c0 && c < c1) {
            if constexpr (A + Bx + C == 0) put(col0 + c, f1);
            else put(col0 + c, cart_mono<A, Bx, C>(cp) * f1);
          }
        });
      };
      switch ((pk.z >> 16) & 0xff) {
        case 0:
          comps(std::integral_constant<int, 0>{}, std::integral_constant<int, 1>{});
          break;
        case 1:
          comps(std::integral_constant<int, 1>{}, std::integral_constant<int, 3>{});
          break;
        case 2:
          comps(std::integral_constant<int, 4>{}, std::integral_constant<int, 6>{});
          break;
        default:
          comps(std::integral_constant<int, 10>{}, std::integral_constant<int, 10>{});
      }
    } else {
      const float px[4] = {1.f, g.cp.x, g.cp.x2, g.cp.x2 * g.cp.x};
      const float py[4] = {1.f, g.cp.y, g.cp.y2, g.cp.y2 * g.cp.y};
      const float pz[4] = {1.f, g.cp.z, g.cp.z2, g.cp.z2 * g.cp.z};
      for (int c = c0; c < c1; ++c) {
        const int ijk = __ldg(B.f_ijk + mu0 + c);
        const int i = ijk & 15, j = (ijk >> 4) & 15, k = (ijk >> 8) & 15;  // each <= 3
        const float xi = i == 0 ? 1.f : (i == 1 ? px[1] : (i == 2 ? px[2] : px[3]));
        const float yj = j == 0 ? 1.f : (j == 1 ? py[1] : (j == 2 ? py[2] : py[3]));
        const float zk = k == 0 ? 1.f : (k == 1 ? pz[1] : (k == 2 ? pz[2] : pz[3]));
        // the same value as the compile-time forms: a factor 1 is exact
        put(col0 + c, xi * yj * zk * f1);
      }
    }
  }
}

}  // namespace

// kSubs threads per point (thread sub walks the shells sub, sub + kSubs,
// ... of each half block: uniform in a warp, as sub = threadIdx.x / 128),
// the tile's half K blocks split over gridDim.y CTAs.  basis_tile_kernel
// is kSubs = 1 with one CTA per tile; basis_tile_short_kernel (passes with
// fewer tiles than two per SM, where one CTA per SM cannot hide the shell
// walk's latency chain) is kSubs = 4 over several CTAs per tile.  Every
// column of a half block is written by exactly one thread, and the
// arithmetic of a value does not depend on kSubs: both give the same
// operand bit for bit.
template <int kSubs>
__device__ __forceinline__ void basis_tile_body(const CUtensorMap& tm_hi, const CUtensorMap& tm_lo, const DevBasis& B,
                                                const double* __restrict__ pts, int64_t npts,
                                                const int* __restrict__ tiles, int stride,
                                                float* __restrict__ inv_scale, unsigned long long* xneed,
                                                float* s_scale, ScreenSmem* ss, int* screen_out) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base =
      reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  const int row = threadIdx.x & (kBlockM - 1), sub = threadIdx.x >> 7;
  const int64_t m0 = static_cast<int64_t>(blockIdx.x) * kBlockM;
  const int64_t p = min(m0 + row, npts - 1);  // rows past the end compute a copy; the TMA store clips them
  const int nhb = 2 * (B.kpad / kBlockK);
  const int hb0 = static_cast<int>(static_cast<int64_t>(blockIdx.y) * nhb / gridDim.y);
  const int hb1 = static_cast<int>(static_cast<int64_t>(blockIdx.y + 1) * nhb / gridDim.y);
  if (kSubs > 1) {
    // one CTA per SM on cold caches: pull the tables into L1 first
    prefetch_l1(B.sh_pack, B.nshells * sizeof(int4));
    prefetch_l1(B.sh_rad2_df, B.nshells * sizeof(float2));
    prefetch_l1(B.p_pack, B.nprim * sizeof(float4));
    prefetch_l1(B.atom_f4, B.natoms * sizeof(float4));
    prefetch_l1(B.atom_g, B.natoms * 3 * sizeof(float2));
    prefetch_l1(B.f_ijk, B.nbf * sizeof(int));
    prefetch_l1(B.f_shell, B.nbf * sizeof(int));
  }

  // active K blocks of this tile (all when no screening lists are given)
  uint64_t kb_on = ~0ull;
  // Short pass without an earlier tile screen (screen_out): every CTA of the
  // tile screens it (the same lists as tile_screen_kernel, gg_tiles.cuh) and
  // the first writes the lists for the contraction.  The marks are cleared
  // here and the tile's sphere formed by the first warp of the second thread
  // group while the first group computes the row scales; the shells are
  // marked after the row-scale barrier.
  if constexpr (kSubs > 1) {
    if (screen_out) {
      for (int i = threadIdx.x; i < B.nchunk; i += blockDim.x) ss->chunk[i] = 0;
      for (int i = threadIdx.x; i < B.kpad / kBlockK; i += blockDim.x) ss->kb[i] = 0;
      if (threadIdx.x >= kBlockM && threadIdx.x < kBlockM + 32) {
        float cf[3], rf;
        warp_tile_sphere(pts, npts, blockIdx.x, threadIdx.x & 31, cf, &rf);
        if (threadIdx.x == kBlockM) {
          ss->sph[0] = cf[0];
          ss->sph[1] = cf[1];
          ss->sph[2] = cf[2];
          ss->sph[3] = rf;
        }
      }
    }
  }
  if (tiles && !screen_out) {
    const int* tl = tiles + blockIdx.x * static_cast<int64_t>(stride);
    const int nk = tl[1];
    const int* kl = tl + 2 + B.nchunk;
    kb_on = 0;
    for (int i = 0; i < nk; ++i) kb_on |= 1ull << kl[i];
  }

  DFloat r[3];
  for (int c = 0; c < 3; ++c) r[c] = df_split(pts[3 * p + c]);

  // ---- pass 1: log2 of an upper bound of |phi| over the row -------------
  // one table lookup per atom: the envelope of its shells' bounds at the
  // point's distance (shells of K blocks inactive for the tile are out of
  // range of every point of it, so the envelope does not see them); by the
  // first thread of each point
  float scale = 1.f;
  if (sub == 0) {
    float lb = -INFINITY;
    const float* __restrict__ env = B.atom_env;
    const int nb = B.env_bins;
    for (int a = 0; a < B.natoms; ++a) {
      const float4 A = __ldg(B.atom_f4 + a);  // the coordinates rounded to fp32, one 16-byte load
      const float dx = r[0].h - A.x, dy = r[1].h - A.y, dz = r[2].h - A.z;
      const float d2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
      const float t = (__log2f(fmaxf(d2, 1e-30f)) + kEnvOffset) * kEnvPerOctave;
      const int bin = t <= 0.f ? 0 : static_cast<int>(t);
      if (bin < nb) lb = fmaxf(lb, __ldg(env + static_cast<int64_t>(a) * nb + bin));
    }
    if (lb > -INFINITY) {
      // bound < 2^e with e = floor(lb + margin) + 1; scale = 2^(14 - e)
      const int e = static_cast<int>(floorf(lb + 0.05f)) + 1;
      scale = ldexpf(1.f, max(-120, min(120, 14 - e)));
    }
    if (blockIdx.y == 0 && m0 + row < npts) inv_scale[m0 + row] = 1.f / scale;
  }
  if (kSubs > 1) {
    if (sub == 0) s_scale[row] = scale;
    __syncthreads();
    scale = s_scale[row];
  }
  if constexpr (kSubs > 1) {
    if (screen_out) {
      const int nkb = B.kpad / kBlockK;
      const float cf[3] = {ss->sph[0], ss->sph[1], ss->sph[2]};
      for (int sh = threadIdx.x; sh < B.nshells; sh += blockDim.x) mark_shell(B, sh, cf, ss->sph[3], ss->chunk, ss->kb);
      __syncthreads();
      if (blockIdx.y == 0 && threadIdx.x < 32)
        warp_write_lists(B, ss->chunk, ss->kb, screen_out + blockIdx.x * static_cast<int64_t>(stride), threadIdx.x);
      kb_on = 0;
      for (int i = 0; i < nkb; ++i)
        if (ss->kb[i]) kb_on |= 1ull << i;
      // this CTA's half blocks need the cross products until shown small
      // below (no earlier kernel set the mask; the other CTAs of the tile
      // own the other bits)
      if (xneed && threadIdx.x == 0) {
        unsigned long long w0 = 0ull, w1 = 0ull;
        for (int hb = hb0; hb < hb1; ++hb) {
          if (hb < 64) w0 |= 1ull << hb;
          else w1 |= 1ull << (hb - 64);
        }
        if (w0) atomicOr(xneed + 2 * static_cast<int64_t>(blockIdx.x), w0);
        if (w1) atomicOr(xneed + 2 * static_cast<int64_t>(blockIdx.x) + 1, w1);
      }
    }
  }

  // ---- pass 2: values, staged per half K block and stored with TMA --------
  const uint32_t rowoff = static_cast<uint32_t>(row) * 64u, rxs = static_cast<uint32_t>((row >> 1) & 3) << 4;
  float vmax = 0.f;  // largest |value| this thread stages in the current half block
  auto put = [&](int col, float v) {
    vmax = fmaxf(vmax, fabsf(v));
    const uint32_t o = swz_col(rowoff, rxs, col);
    const __half h = __float2half_rn(v);
    const __half l = __float2half_rn(v - __half2float(h));
    *reinterpret_cast<__half*>(base + o) = h;
    *reinterpret_cast<__half*>(base + kStageBytes + o) = l;
  };
  AtomGeom g;
  const float2 rg[3] = {grid_split(r[0]), grid_split(r[1]), grid_split(r[2])};
  for (int hb = hb0; hb < hb1; ++hb) {
    if (!((kb_on >> (hb >> 1)) & 1ull)) continue;  // inactive for the tile: never read
    const int lo = hb * kHalfK, hi = min(lo + kHalfK, B.nbf);
    // the row's 64 bytes of each half start as zeros (16-byte stores; each
    // thread of the point clears its share): the padding columns and the
    // shells out of range for the whole warp are left as they are
    {
      constexpr int kPart = 64 / kSubs;
      const uint32_t o = rowoff + static_cast<uint32_t>(sub * kPart);
#pragma unroll
      for (int b = 0; b < kPart; b += 16) {
        *reinterpret_cast<uint4*>(base + o + b) = make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(base + kStageBytes + o + b) = make_uint4(0u, 0u, 0u, 0u);
      }
      if (kSubs > 1) __syncthreads();  // the other threads of the point write into this share
    }
    if (lo < B.nbf) stage_shells<kSubs>(B, rg, scale, lo, hi, sub, g, put);
    // the half block is complete: write it to HBM, then reuse the buffer;
    // a half block small for every point of the tile needs no cross products
    fence_proxy_async();
    const int small = __syncthreads_and(vmax < kCrossSkipScaled);
    vmax = 0.f;
    if (threadIdx.x == 0 && small && xneed)
      atomicAnd(xneed + 2 * static_cast<int64_t>(blockIdx.x) + (hb >> 6), ~(1ull << (hb & 63)));
    if (threadIdx.x == 0) {
      tma_store_2d(&tm_hi, base, hb * kHalfK, static_cast<int>(m0));
      tma_store_2d(&tm_lo, base + kStageBytes, hb * kHalfK, static_cast<int>(m0));
      bulk_commit();
      bulk_wait_read_0();
    }
    __syncthreads();
  }
  if (threadIdx.x == 0) bulk_wait_all();
}

__global__ void __launch_bounds__(kTileThreads, 10) basis_tile_kernel(const __grid_constant__ CUtensorMap tm_hi,
                                                                  const __grid_constant__ CUtensorMap tm_lo,
                                                                  DevBasis B, const double* __restrict__ pts,
                                                                  int64_t npts, const int* __restrict__ tiles,
                                                                  int stride, float* __restrict__ inv_scale,
                                                                  unsigned long long* __restrict__ xneed) {
  basis_tile_body<1>(tm_hi, tm_lo, B, pts, npts, tiles, stride, inv_scale, xneed, nullptr, nullptr, nullptr);
}

constexpr int kSubs = 4;
constexpr int kShortThreads = kBlockM * kSubs;

__global__ void __launch_bounds__(kShortThreads) basis_tile_short_kernel(
    const __grid_constant__ CUtensorMap tm_hi, const __grid_constant__ CUtensorMap tm_lo, DevBasis B,
    const double* __restrict__ pts, int64_t npts, const int* __restrict__ tiles, int stride,
    float* __restrict__ inv_scale, unsigned long long* __restrict__ xneed, int* screen_out) {
  __shared__ float s_scale[kBlockM];
  __shared__ ScreenSmem ss;
  basis_tile_body<kSubs>(tm_hi, tm_lo, B, pts, npts, tiles, stride, inv_scale, xneed, s_scale, &ss, screen_out);
}

cudaError_t launch_basis_tile(const DevBasis& B, const void* tm_hi, const void* tm_lo, const double* pts,
                              int64_t npts, const int* tiles, int stride, float* inv_scale,
                              unsigned long long* xneed, int* screen_out, cudaStream_t st) {
  if (npts <= 0) return cudaSuccess;
  if (B.kpad / kBlockK > 64) return cudaErrorInvalidValue;  // K-block mask is 64 bits
  if (screen_out && B.nchunk > kMaxScreenChunks) return cudaErrorInvalidValue;
  // the shared-memory attribute (it applies to the current device) and the
  // SM count, once per device
  static PerDevice pd;
  int nsm = 0;
  cudaError_t e = once_per_device(pd, &nsm, [](int dev, int* sms) {
    cudaError_t r = cudaFuncSetAttribute(basis_tile_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTileSmem);
    if (r == cudaSuccess)
      r = cudaFuncSetAttribute(basis_tile_short_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTileSmem);
    if (r != cudaSuccess) return r;
    return cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
  });
  if (e != cudaSuccess) return e;
  const int64_t ntiles = (npts + kBlockM - 1) / kBlockM;
  // fewer tiles than two per SM: split every tile's half K blocks over
  // several CTAs, about two CTAs per SM in all (each CTA walks only the
  // shells of its half blocks; the row-scale pass is repeated per CTA)
  const int nhb = 2 * (B.kpad / kBlockK);
  int kgroups = 1;
  if (nsm > 0 && ntiles < 2 * nsm) kgroups = static_cast<int>(std::min<int64_t>(nhb, (2 * nsm + ntiles - 1) / ntiles));
  const dim3 grid(static_cast<unsigned>(ntiles), static_cast<unsigned>(kgroups));
  if (screen_out && kgroups == 1) return cudaErrorInvalidValue;  // only the short kernel screens its tiles
  if (kgroups > 1)
    basis_tile_short_kernel<<<grid, kShortThreads, kTileSmem, st>>>(*static_cast<const CUtensorMap*>(tm_hi),
                                                                   *static_cast<const CUtensorMap*>(tm_lo), B, pts,
                                                                   npts, tiles, stride, inv_scale, xneed,
                                                                   screen_out);
  else
    basis_tile_kernel<<<grid, kTileThreads, kTileSmem, st>>>(*static_cast<const CUtensorMap*>(tm_hi),
                                                            *static_cast<const CUtensorMap*>(tm_lo), B, pts, npts,
                                                            tiles, stride, inv_scale, xneed);
  return cudaGetLastError();
}

}  // namespace gg
