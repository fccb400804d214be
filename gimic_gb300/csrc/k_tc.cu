// Split-FP16 tensor-core contraction with a fused current-tensor epilogue.
//
// Per CTA: 128 grid points (GEMM rows).  The GEMM computes, chunk by chunk,
//     W[p, (m, nu)] = sum_mu phi_p,mu * M_m[mu, nu],   M = D, C_x, C_y, C_z, P_x, P_y, P_z
// for 32 functions nu at a time (224 columns), as three fp16 tcgen05 MMAs
// per K step (hi*hi + hi*lo + lo*hi of power-of-two scaled operands) with
// fp32 accumulation in TMEM.  The two TMEM accumulators alternate between
// chunks so that the epilogue of chunk c overlaps the MMAs of chunk c+1.
//
// Roles (192 threads):
//   warp 0      TMA producer (A: phi pieces of the tile, B: matrix pieces)
//   warp 1      TMEM owner and MMA issuer
//   warps 2..5  epilogue: for its point (one TMEM lane per thread) it
//               re-evaluates phi, grad phi and the Laplacian of the chunk's 32
//               functions in fp32 (src/libgimic/caos.f90:17-110 semantics)
//               and accumulates the kNDots bilinear forms; fp32 within a
//               chunk, fp64 across chunks; final fp64 combination as in
//               gg_combine.cuh (src/libgimic/jtensor.F90:148-237).
#include <cuda.h>

#include <algorithm>

#include "gg_cart.cuh"
#include "gg_combine.cuh"
#include "gg_kernels.h"

namespace gg {

namespace {
constexpr int kStages = 2;
constexpr int kTileA = kBlockM * kBlockK * 2;          // 16 KiB
constexpr int kTileB = kBlockN * kBlockK * 2;          // 28 KiB
constexpr int kStageBytes = 2 * kTileA + 2 * kTileB;   // 88 KiB
constexpr int kEpiWarps = 8;                           // 2 per TMEM lane quarter
constexpr int kThreads = 32 * (2 + kEpiWarps);
constexpr uint32_t kTmemCols = 512;
constexpr int kAccStride = 256;
constexpr int kMaxTileList = 512;  // ints: 2 + column chunks + K blocks of a tile (nbf <= 10,000)
constexpr int kSmemBytes = kStages * kStageBytes + 1024 + 256 + kMaxTileList * 4;
static_assert(kBlockM * kNDots * 8 <= kStageBytes, "epilogue reduction buffer must fit in one stage");

__device__ __forceinline__ void tmem_ld1(uint32_t taddr, float& v) {
  uint32_t r;
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r) : "r"(taddr) : "memory");
  v = __uint_as_float(r);
}

// wait for this thread's TMEM loads; the registers are in/out operands so
// that no use of them is scheduled before the wait
__device__ __forceinline__ void tmem_wait7(float* v) {
  asm volatile("tcgen05.wait::ld.sync.aligned;"
               : "+f"(v[0]), "+f"(v[1]), "+f"(v[2]), "+f"(v[3]), "+f"(v[4]), "+f"(v[5]), "+f"(v[6])
               :
               : "memory");
}

__device__ __forceinline__ void epi_barrier() { asm volatile("bar.sync 1, %0;" ::"r"(32 * kEpiWarps) : "memory"); }

// error-free fp32 sum: s + e = a + b exactly (Knuth two-sum)
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bp = s - hi;
  const float e = (hi - (s - bp)) + (x - bp);
  hi = s;
  lo += e;
}
}  // namespace

int tc_smem_bytes() { return kSmemBytes; }

// Per chunk the MMAs run in two passes over K into the same accumulator:
// first the two small cross products (hi*lo, lo*hi), then the main product
// (hi*hi).  Tensor-core accumulation truncates each partial sum to fp32; the
// small terms are added while the accumulator is still small, which keeps
// their truncation error negligible (measured: max error of j 1.2e-6 with the
// products interleaved, 4.6e-7 cross-first, for nbf = 720).
__global__ void __launch_bounds__(kThreads, 1)
    tc_fused_kernel(const __grid_constant__ CUtensorMap tm_a_hi, const __grid_constant__ CUtensorMap tm_a_lo,
                    const __grid_constant__ CUtensorMap tm_b_hi, const __grid_constant__ CUtensorMap tm_b_lo,
                    DevBasis Bs, const float* __restrict__ inv_row, const float* __restrict__ inv_col,
                    const double* __restrict__ pts, int64_t npts, Flags fl, Outputs out, int* err,
                    const int* __restrict__ tiles, int tstride, const int* __restrict__ perm,
                    const int* __restrict__ tile_order) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~static_cast<uintptr_t>(1023));
  uint64_t* full = reinterpret_cast<uint64_t*>(base + kStages * kStageBytes);
  uint64_t* empty = full + kStages;
  uint64_t* accfull = empty + kStages;
  uint64_t* accempty = accfull + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accempty + 2);
  int* tlist = reinterpret_cast<int*>(tmem_slot + 4);  // {#chunks, #kblocks, chunk ids, kblock ids}

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int64_t tile = tile_order ? static_cast<int64_t>(tile_order[blockIdx.x]) : static_cast<int64_t>(blockIdx.x);
  const int64_t m0 = tile * kBlockM;
  const int nchunk_all = Bs.nchunk, nkb_all = Bs.kpad / kBlockK;
  // active column chunks and K blocks of this tile (all of them without a
  // screening list)
  if (tiles) {
    for (int i = threadIdx.x; i < tstride; i += blockDim.x) tlist[i] = tiles[tile * tstride + i];
  } else {
    for (int i = threadIdx.x; i < nchunk_all; i += blockDim.x) tlist[2 + i] = i;
    for (int i = threadIdx.x; i < nkb_all; i += blockDim.x) tlist[2 + nchunk_all + i] = i;
    if (threadIdx.x == 0) {
      tlist[0] = nchunk_all;
      tlist[1] = nkb_all;
    }
  }
  const int* clist = tlist + 2;
  const int* klist = tlist + 2 + nchunk_all;
  // epilogue tables: column scales, per-function records (shell << 12 |
  // Cartesian case), shell records, primitives, atoms
  const float* icol = inv_col;
  const int* fpack = Bs.f_pack;
  const int4* shp = Bs.sh_pack;
  const float2* shr = Bs.sh_rad2_df;
  const float4* prm = Bs.p_pack;
  const float2* atm = Bs.atom_df;
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accfull[b], 1);
      mbar_init(&accempty[b], kEpiWarps);
    }
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;
  const int nkb = tlist[1];
  const int nchunk = nkb > 0 ? tlist[0] : 0;
  const int nkb2 = (nkb + 1) / 2;  // main-product stages (two K blocks each)

  if (warp == 0) {
    if (lane == 0) {
      int it = 0;
      for (int ci = 0; ci < nchunk; ++ci) {
        const int c = clist[ci];
        // pass 1: A_hi, A_lo, B_hi, B_lo of one K block per stage
        for (int ki = 0; ki < nkb; ++ki, ++it) {
          const int kb = klist[ki];
          const int s = it % kStages, round = it / kStages;
          if (!mbar_wait(&empty[s], (round & 1) ^ 1, err, 1)) goto done;
          unsigned char* st = base + s * kStageBytes;
          mbar_expect_tx(&full[s], kStageBytes);
          tma_load_2d(st, &tm_a_hi, &full[s], kb * kBlockK, static_cast<int>(m0));
          tma_load_2d(st + kTileA, &tm_a_lo, &full[s], kb * kBlockK, static_cast<int>(m0));
          tma_load_2d(st + 2 * kTileA, &tm_b_hi, &full[s], kb * kBlockK, c * kBlockN);
          tma_load_2d(st + 2 * kTileA + kTileB, &tm_b_lo, &full[s], kb * kBlockK, c * kBlockN);
        }
        // pass 2: A_hi, B_hi of two K blocks per stage (same slots)
        for (int k2 = 0; k2 < nkb2; ++k2, ++it) {
          const int s = it % kStages, round = it / kStages;
          if (!mbar_wait(&empty[s], (round & 1) ^ 1, err, 1)) goto done;
          unsigned char* st = base + s * kStageBytes;
          const int ki0 = 2 * k2, nk = (ki0 + 1 < nkb) ? 2 : 1;
          mbar_expect_tx(&full[s], nk * (kTileA + kTileB));
          for (int j = 0; j < nk; ++j) {
            const int kb = klist[ki0 + j];
            tma_load_2d(st + j * kTileA, &tm_a_hi, &full[s], kb * kBlockK, static_cast<int>(m0));
            tma_load_2d(st + 2 * kTileA + j * kTileB, &tm_b_hi, &full[s], kb * kBlockK, c * kBlockN);
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_f16(kBlockM, kBlockN);
      int it = 0;
      for (int ci = 0; ci < nchunk; ++ci) {
        const int b = ci & 1, rb = ci >> 1;
        if (!mbar_wait(&accempty[b], (rb & 1) ^ 1, err, 2)) goto done;
        tc_fence_after();
        const uint32_t d_tmem = tmem_base + b * kAccStride;
        for (int kb = 0; kb < nkb; ++kb, ++it) {
          const int s = it % kStages, round = it / kStages;
          if (!mbar_wait(&full[s], round & 1, err, 3)) goto done;
          tc_fence_after();
          unsigned char* st = base + s * kStageBytes;
          const uint64_t ah = smem_desc_sw128(st), al = smem_desc_sw128(st + kTileA);
          const uint64_t bh = smem_desc_sw128(st + 2 * kTileA), bl = smem_desc_sw128(st + 2 * kTileA + kTileB);
#pragma unroll
          for (int k = 0; k < kBlockK / 16; ++k) {
            const uint64_t o = static_cast<uint64_t>(k * 32) >> 4;  // 16 fp16 = 32 bytes along K
            mma_f16(d_tmem, ah + o, bl + o, idesc, (kb > 0 || k > 0) ? 1u : 0u);
            mma_f16(d_tmem, al + o, bh + o, idesc, 1u);
          }
          mma_commit(&empty[s]);
        }
        for (int k2 = 0; k2 < nkb2; ++k2, ++it) {
          const int s = it % kStages, round = it / kStages;
          if (!mbar_wait(&full[s], round & 1, err, 3)) goto done;
          tc_fence_after();
          unsigned char* st = base + s * kStageBytes;
          const int nk = (2 * k2 + 1 < nkb) ? 2 : 1;
          for (int j = 0; j < nk; ++j) {
            const uint64_t ah = smem_desc_sw128(st + j * kTileA), bh = smem_desc_sw128(st + 2 * kTileA + j * kTileB);
#pragma unroll
            for (int k = 0; k < kBlockK / 16; ++k) {
              const uint64_t o = static_cast<uint64_t>(k * 32) >> 4;
              mma_f16(d_tmem, ah + o, bh + o, idesc, 1u);
            }
          }
          mma_commit(&empty[s]);
        }
        mma_commit(&accfull[b]);
      }
    }
  } else {
    // ---------------- epilogue: 8 warps ----------------
    // warp w reads TMEM lanes 32*(w%4) .. +31 (its 32 points) and handles
    // half (w-2)/4 of the 32 functions of every chunk.
    const int q = warp & 3;
    const int half = (warp - 2) >> 2;
    const int row = q * 32 + lane;
    const int64_t p = m0 + row;
    const bool valid = p < npts;
    double r[3] = {0.0, 0.0, 0.0};
    if (valid) {
      r[0] = pts[3 * p];
      r[1] = pts[3 * p + 1];
      r[2] = pts[3 * p + 2];
    }
    const DFloat rdf[3] = {df_split(r[0]), df_split(r[1]), df_split(r[2])};
    float thi[kNDots], tlo[kNDots];
#pragma unroll
    for (int i = 0; i < kNDots; ++i) thi[i] = tlo[i] = 0.f;
    int cur_shell = -1, cur_atom = -1;
    float sx = 0.f, sy = 0.f, sz = 0.f, f1 = 0.f, f2 = 0.f, f3 = 0.f;
    CartPow cp = cart_pow(0.f, 0.f, 0.f);
    DFloat d2a{0.f, 0.f};
    bool on = false;
    const uint32_t lane_base = tmem_base + (static_cast<uint32_t>(q * 32) << 16);
    for (int ci = 0; ci < nchunk; ++ci) {
      const int c = clist[ci];
      const int b = ci & 1, rb = ci >> 1;
      if (!mbar_wait(&accfull[b], rb & 1, err, 4)) break;
      tc_fence_after();
      float part[kNDots];
#pragma unroll
      for (int i = 0; i < kNDots; ++i) part[i] = 0.f;
      const int f0 = c * kChunkF;
      const int mb = f0 + half * (kChunkF / 2);
      const int me = min(mb + kChunkF / 2, Bs.nbf);
      const uint32_t tcol = lane_base + b * kAccStride;
#pragma unroll 1
      for (int mu = mb; mu < me; ++mu) {
        const int u = mu - f0;
        const int fp = fpack[mu];
        const int sh = fp >> 12;
        if (sh != cur_shell) {
          cur_shell = sh;
          const int4 pk = shp[sh];  // atom, first function, ncomp | npf << 8 | l << 16, first primitive
          const int a = pk.x;
          if (a != cur_atom) {
            cur_atom = a;
            float s3[3];
            d2a = atom_offset_t(rdf, atm, a, s3);
            sx = s3[0];
            sy = s3[1];
            sz = s3[2];
            cp = cart_pow(sx, sy, sz);
          }
          on = df_le(d2a, shr[sh]);
          f1 = f2 = f3 = 0.f;
          if (on) {
            const int np = (pk.z >> 8) & 0xff;
            for (int k = 0; k < np; ++k) {
              const float4 pr = prm[pk.w + k];  // exponent hi, exponent lo, coefficient
              const float al = pr.x;
              const float e = pr.z * gauss_df(al, pr.y, d2a.h, d2a.l);
              f1 += e;
              f2 += al * e;
              f3 += al * al * e;
            }
          }
        }
        // functions screened for all 32 points of the warp contribute nothing
        if (!__any_sync(0xffffffffu, on)) continue;
        float v[kMats];
#pragma unroll
        for (int m = 0; m < kMats; ++m) tmem_ld1(tcol + m * kChunkF + u, v[m]);
        tmem_wait7(v);
        if (on) {
          float ph, gx, gy, gz, lp;
          cart_case(fp & 0xfff, cp, f1, f2, f3, &ph, &gx, &gy, &gz, &lp);
          const float* cs = icol + c * kBlockN + u;
          const float w0 = v[0] * cs[0];
          const float wc[3] = {v[1] * cs[1 * kChunkF], v[2] * cs[2 * kChunkF], v[3] * cs[3 * kChunkF]};
          const float qq[3] = {v[4] * cs[4 * kChunkF], v[5] * cs[5 * kChunkF], v[6] * cs[6 * kChunkF]};
          const float wp = w0 * ph;
          part[0] = fmaf(w0, ph, part[0]);
          part[1] = fmaf(wp, sx, part[1]);
          part[2] = fmaf(wp, sy, part[2]);
          part[3] = fmaf(wp, sz, part[3]);
          const float wx = w0 * sx, wy = w0 * sy, wz = w0 * sz;
          part[4 + 1] = fmaf(wy, gx, part[4 + 1]);  // E[x][y]
          part[4 + 2] = fmaf(wz, gx, part[4 + 2]);  // E[x][z]
          part[4 + 3] = fmaf(wx, gy, part[4 + 3]);  // E[y][x]
          part[4 + 5] = fmaf(wz, gy, part[4 + 5]);  // E[y][z]
          part[4 + 6] = fmaf(wx, gz, part[4 + 6]);  // E[z][x]
          part[4 + 7] = fmaf(wy, gz, part[4 + 7]);  // E[z][y]
          const float g[3] = {gx, gy, gz};
#pragma unroll
          for (int d = 0; d < 3; ++d) {
#pragma unroll
            for (int m = 0; m < 3; ++m) {
              part[13 + 3 * d + m] = fmaf(wc[d], g[m], part[13 + 3 * d + m]);
              part[25 + 3 * d + m] = fmaf(qq[d], g[m], part[25 + 3 * d + m]);
            }
            part[22 + d] = fmaf(wc[d], lp, part[22 + d]);
            part[34 + d] = fmaf(qq[d], lp, part[34 + d]);
          }
        }
      }
      tc_fence_before();
      __syncwarp();
      if (lane == 0) mbar_arrive(&accempty[b]);
#pragma unroll
      for (int i = 0; i < kNDots; ++i)
        if (i != 4 && i != 8 && i != 12) two_sum_acc(thi[i], tlo[i], part[i]);
    }
    // combine the two halves of every point through shared memory (the
    // pipeline stages are idle once the last accumulator has been read)
    double* red = reinterpret_cast<double*>(base);
    if (half == 1) {
#pragma unroll
      for (int i = 0; i < kNDots; ++i) red[row * kNDots + i] = static_cast<double>(thi[i]) + static_cast<double>(tlo[i]);
    }
    epi_barrier();
    if (half == 0 && valid) {
      double tot[kNDots];
      const double sc = static_cast<double>(inv_row[p]);
#pragma unroll
      for (int i = 0; i < kNDots; ++i)
        tot[i] = ((static_cast<double>(thi[i]) + static_cast<double>(tlo[i])) + red[row * kNDots + i]) * sc;
      double ct[9], dv[3];
      combine_point(tot, r, fl, ct, dv);
      const int64_t o = perm ? static_cast<int64_t>(perm[p]) : p;  // caller's point order
      store_outputs(out, o, ct, tot[0], dv);
    }
  }
done:
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem_base, kTmemCols);
  }
}

cudaError_t launch_tc_fused(const DevBasis& B, const TcArgs& a, cudaStream_t st) {
  if (a.npts <= 0) return cudaSuccess;
  static bool attr_set = false;
  if (!attr_set) {
    cudaError_t e = cudaFuncSetAttribute(tc_fused_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes);
    if (e != cudaSuccess) return e;
    attr_set = true;
  }
  const unsigned grid = static_cast<unsigned>((a.npts + kBlockM - 1) / kBlockM);
  tc_fused_kernel<<<grid, kThreads, kSmemBytes, st>>>(
      *static_cast<const CUtensorMap*>(a.tmap_a_hi), *static_cast<const CUtensorMap*>(a.tmap_a_lo),
      *static_cast<const CUtensorMap*>(a.tmap_b_hi), *static_cast<const CUtensorMap*>(a.tmap_b_lo), B,
      a.inv_row_scale, a.inv_col_scale, a.pts, a.npts, a.flags, a.out, a.err, a.tiles, a.tile_stride, a.perm,
      a.tile_order);
  return cudaGetLastError();
}

}  // namespace gg
