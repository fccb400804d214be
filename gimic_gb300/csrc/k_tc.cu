// Split-FP16 tensor-core contraction with a fused current-tensor epilogue.
//
// Persistent: one CTA per SM takes tiles of 128 grid points (GEMM rows)
// from a global queue in tile order (heaviest first: the producer warp
// draws the next step with an atomic counter and hands it to the MMA and
// epilogue warps through a small ring of mbarrier-guarded slots), so the
// pipeline, the TMEM accumulators and the epilogue run on from one tile
// into the next.  Per
// tile the GEMM computes, chunk by chunk,
//     W[p, (m, nu)] = sum_mu phi_p,mu * M_m[mu, nu],   M = D, C_x, C_y, C_z, P_x, P_y, P_z
// for 32 functions nu at a time (224 columns), as three fp16 tcgen05 MMAs
// per K step (hi*hi + hi*lo + lo*hi of power-of-two scaled operands) with
// fp32 accumulation in TMEM (a four-stage TMA/mbarrier pipeline, one
// operand pair per stage).  The two TMEM accumulators alternate between
// chunks so that the epilogue of chunk c overlaps the MMAs of chunk c+1.
//
// Roles (512 threads, four warpgroups):
//   warp 0      TMA producer (A: phi pieces of the tile, B: matrix pieces)
//   warp 1      TMEM owner and MMA issuer
//   warps 2, 3  none (they complete the first warpgroup, which hands its
//               registers to the epilogue)
//   warps 4..15 epilogue, three warps per TMEM lane quarter, each taking a
//               third of a chunk's functions: for its point (one TMEM lane)
//               it re-evaluates phi, grad phi and the Laplacian of those
//               functions in fp32 (src/libgimic/caos.f90:17-110 semantics)
//               and accumulates the kNDots bilinear forms in fp32 over the
//               tile; the three groups' sums are added as double-floats, and
//               the final combination runs in double-float
//               (gg_combine.cuh, src/libgimic/jtensor.F90:148-237).
#include <cuda.h>

#include <algorithm>
#include <cstring>
#include <type_traits>

#include "gg_cart.cuh"
#include "gg_combine.cuh"
#include "gg_kernels.h"
#include "gg_once.h"

namespace gg {

namespace {
// A stage holds one A piece and one B piece of one K block: (hi, lo) or
// (lo, hi) in the cross pass, (hi, hi) in the main pass.  Four 44 KiB stages
// keep up to 132 KiB of loads in flight while the MMAs read the fourth.
constexpr int kStages = 4;
constexpr int kTileA = kBlockM * kBlockK * 2;          // 16 KiB
constexpr int kTileB = kBlockN * kBlockK * 2;          // 28 KiB
constexpr int kStageBytes = kTileA + kTileB;           // 44 KiB
// Epilogue warps per TMEM lane quarter: each takes one group of a chunk's
// functions (11, 11 and 10 of the 32).  The epilogue is bound by the latency
// of its per-function chains (shell changes, the primitive sums, the
// polynomial), so three warps per quarter issue more of it than two.
constexpr int kEpiGroups = 3;
constexpr int kGroupF = (kChunkF + kEpiGroups - 1) / kEpiGroups;
constexpr int kEpiWarps = 4 * kEpiGroups;
constexpr int kCtlWarps = 4;                           // TMA producer, MMA issuer, two idle: one warpgroup
constexpr int kThreads = 32 * (kCtlWarps + kEpiWarps);
// Register split (setmaxnreg, per warpgroup): the control warpgroup gives
// registers up so that the epilogue warpgroups can hold their accumulators,
// the geometry and the TMEM values of a function without spilling.  The
// shares add up to at most the launch allocation of 128 per thread
// (65,536 / 512), which the launcher checks.
constexpr int kRegsLaunch = 128;
constexpr int kRegsCtl = 56;
constexpr int kRegsEpi = 152;
static_assert(kCtlWarps * kRegsCtl + kEpiWarps * kRegsEpi <= (kCtlWarps + kEpiWarps) * kRegsLaunch,
              "register split exceeds the launch allocation");
constexpr uint32_t kTmemCols = 512;
constexpr int kAccStride = 256;
constexpr int kRedBytes = (kEpiGroups - 1) * kBlockM * kNDots * 4;  // group sums handed to group 0 (fp32)
constexpr int kRing = 4;  // tile steps in flight between the producer and the other roles
constexpr int kSmemBytes = kStages * kStageBytes + kRedBytes + 1024 + 512;  // + alignment, barriers and ring

__device__ __forceinline__ void reg_dealloc_ctl() { asm volatile("setmaxnreg.dec.sync.aligned.u32 %0;" ::"n"(kRegsCtl)); }

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

// the matrix of each of the kNDots sums: 0..12 D (rho, X, E), 13..24 C_d
// (Y_dm at 13 + 3d + m, Laplacian terms at 22 + d), 25..36 P_d (Z_dm at
// 25 + 3d + m, Laplacian terms at 34 + d)
__host__ __device__ constexpr int dot_matrix(int i) {
  return i < 13 ? 0 : i < 22 ? 1 + (i - 13) / 3 : i < 25 ? 1 + (i - 22) : i < 34 ? 4 + (i - 25) / 3 : 4 + (i - 34);
}
static_assert(dot_matrix(12) == 0 && dot_matrix(13) == 1 && dot_matrix(21) == 3 && dot_matrix(24) == 3 &&
                  dot_matrix(25) == 4 && dot_matrix(33) == 6 && dot_matrix(36) == 6 && kNDots == 37,
              "sum layout");

// What a step needs of its job (one pass over one molecule's points): the
// operands' tensor maps and the tile lists for the producer and the MMA
// issuer, the tables, scales, points and outputs for the epilogue.  A
// single-job launch takes them from the kernel parameters, a multi-job
// launch from the job table in global memory.
struct JobView {
  const void *a_hi, *a_lo, *b_hi, *b_lo;  // CUtensorMap
  const int* tiles;
  const unsigned long long* xneed;  // half K blocks that need the cross products (null: all)
  int tstride, nchunk, nkb;
  const int* tile_order;
  int64_t step0, npts;
};
struct EpiView {
  int nbf, nshells;
  const int* fpack;
  const int4* shp;
  const float2* shr;
  const float4* prm;
  const float2* atm;
  const float* icol;
  const float* inv_row;
  const double* pts;
  const int* perm;
  int64_t npts;
  Outputs out;
  int* left;
  unsigned long long* done_ns;
};
}  // namespace

int tc_smem_bytes() { return kSmemBytes; }

// Per chunk the MMAs run in two passes over K into the same accumulator:
// first the two small cross products (hi*lo, lo*hi of each K block), then
// the main product (hi*hi).  Tensor-core accumulation truncates each partial sum to fp32; the
// small terms are added while the accumulator is still small, which keeps
// their truncation error negligible (measured: max error of j 1.2e-6 with the
// products interleaved, 4.6e-7 cross-first, for nbf = 720).
//
// kDiv: the divergence sums (Laplacian terms) are accumulated only when the
// caller asked for div j; without them each function costs 6 FMAs, the
// Laplacian and one FMA per primitive less.
//
// kMulti: one launch over several jobs (the molecules of a batch), whose
// operands and tables come from the job table `jobs` (njobs entries); steps
// are numbered across the jobs in table order (job j owns the steps from
// jobs[j].step0), so the persistent CTAs run on from one molecule into the
// next.  The single-job parameters are then unused.
template <bool kDiv, bool kMulti>
__global__ void __launch_bounds__(kThreads, 1)
    tc_fused_kernel(const __grid_constant__ CUtensorMap tm_a_hi, const __grid_constant__ CUtensorMap tm_a_lo,
                    const __grid_constant__ CUtensorMap tm_b_hi, const __grid_constant__ CUtensorMap tm_b_lo,
                    DevBasis Bs, const float* __restrict__ inv_row, const float* __restrict__ inv_col,
                    const double* __restrict__ pts, int64_t npts, Flags fl, Outputs out, int* err,
                    const int* __restrict__ tiles, int tstride, const int* __restrict__ perm,
                    const int* __restrict__ tile_order, int* __restrict__ tile_counter, int csplit,
                    float2* __restrict__ part, unsigned* __restrict__ tile_done,
                    const unsigned long long* __restrict__ xneed, const TcJob* __restrict__ jobs, int njobs,
                    int64_t multi_steps) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* base = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) &
                                                         ~static_cast<uintptr_t>(1023));
  double* red = reinterpret_cast<double*>(base + kStages * kStageBytes);
  uint64_t* full = reinterpret_cast<uint64_t*>(base + kStages * kStageBytes + kRedBytes);
  uint64_t* empty = full + kStages;
  uint64_t* accfull = empty + kStages;
  uint64_t* accempty = accfull + 2;
  uint64_t* xfull = accempty + 2;   // [4] per lane quarter: groups 1.. have put a tile's sums in `red`
  uint64_t* xempty = xfull + 4;     // [4] group 0 has read them
  uint64_t* ring_full = xempty + 4;          // tile steps handed from the producer to the other roles
  uint64_t* ring_empty = ring_full + kRing;
  uint64_t* drain = ring_empty + kRing;      // the MMA issuer's last MMAs, after an error
  int* ring = reinterpret_cast<int*>(drain + 1);
  int* ring_job = ring + kRing;  // the job of each handed step
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(ring_job + kRing);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // A step is one tile (csplit == 1) or one active chunk of a tile (the
  // chunk split of short passes: step t is chunk t % csplit of tile
  // t / csplit, and csplit is the chunk count of the basis).  A multi-job
  // launch has csplit == 1 and multi_steps tiles over all jobs.
  const int64_t nsteps = kMulti ? multi_steps : ((npts + kBlockM - 1) / kBlockM) * csplit;
  // the job of step t (a binary search over the jobs' first steps)
  auto job_of = [&](int64_t t) -> int {
    if (!kMulti) return 0;
    int lo = 0, hi = njobs - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (jobs[mid].step0 <= t) lo = mid;
      else hi = mid - 1;
    }
    return lo;
  };
  auto view = [&](int j) -> JobView {
    JobView v;
    if (kMulti) {
      const TcJob& J = jobs[j];
      v.a_hi = J.tmap[0];
      v.a_lo = J.tmap[1];
      v.b_hi = J.tmap[2];
      v.b_lo = J.tmap[3];
      v.tiles = J.tiles;
      v.tstride = J.tstride;
      v.nchunk = J.B.nchunk;
      v.nkb = J.B.kpad / kBlockK;
      v.tile_order = J.tile_order;
      v.xneed = J.xneed;
      v.step0 = J.step0;
      v.npts = J.npts;
    } else {
      v.a_hi = &tm_a_hi;
      v.a_lo = &tm_a_lo;
      v.b_hi = &tm_b_hi;
      v.b_lo = &tm_b_lo;
      v.tiles = tiles;
      v.tstride = tstride;
      v.nchunk = Bs.nchunk;
      v.nkb = Bs.kpad / kBlockK;
      v.tile_order = tile_order;
      v.xneed = xneed;
      v.step0 = 0;
      v.npts = npts;
    }
    return v;
  };
  // the tile of step t, and its active column chunks and K blocks (all of
  // them without a screening list; no chunk at all without a K block)
  auto tile_of = [&](const JobView& v, int64_t t) -> int64_t {
    const int64_t u = (t - v.step0) / csplit;
    return v.tile_order ? static_cast<int64_t>(v.tile_order[u]) : u;
  };
  // the chunks [c0, c1) of the tile's active list that step t covers
  auto chunk_span = [&](int64_t t, int nchunk, int* c0, int* c1) {
    if (csplit == 1) {
      *c0 = 0;
      *c1 = nchunk;
    } else {
      const int g = static_cast<int>(t % csplit);
      *c0 = g;
      *c1 = g < nchunk ? g + 1 : g;
    }
  };
  auto n_kb = [&](const JobView& v, int64_t tile) -> int { return v.tiles ? v.tiles[tile * v.tstride + 1] : v.nkb; };
  auto n_chunk = [&](const JobView& v, int64_t tile, int nk) -> int {
    return nk > 0 ? (v.tiles ? v.tiles[tile * v.tstride] : v.nchunk) : 0;
  };
  auto chunk_at = [&](const JobView& v, int64_t tile, int i) -> int {
    return v.tiles ? v.tiles[tile * v.tstride + 2 + i] : i;
  };
  auto kb_at = [&](const JobView& v, int64_t tile, int i) -> int {
    return v.tiles ? v.tiles[tile * v.tstride + 2 + v.nchunk + i] : i;
  };
  // whether K block kb of the tile needs the cross products (either of its
  // two half blocks' bits); the tile's two mask words are read once per step
  auto cross_words = [&](const JobView& v, int64_t tile, unsigned long long* w0, unsigned long long* w1) {
    *w0 = v.xneed ? v.xneed[2 * tile] : ~0ull;
    *w1 = v.xneed ? v.xneed[2 * tile + 1] : ~0ull;
  };
  auto needs_cross = [](unsigned long long w0, unsigned long long w1, int kb) -> bool {
    const int h = 2 * kb;  // both half blocks in one word (h is even)
    return (((h < 64 ? w0 : w1) >> (h & 63)) & 3ull) != 0;
  };
  auto failed = [&]() -> bool { return *reinterpret_cast<volatile int*>(err) != 0; };
  // epilogue tables: matrix scales, per-function records (shell << 12 |
  // Cartesian case), shell records, primitives, atoms; the points, their
  // scales and order, the outputs
  auto epi_view = [&](int j) -> EpiView {
    EpiView e;
    if (kMulti) {
      const TcJob& J = jobs[j];
      e.nbf = J.B.nbf;
      e.nshells = J.B.nshells;
      e.fpack = J.B.f_pack;
      e.shp = J.B.sh_pack;
      e.shr = J.B.sh_rad2_df;
      e.prm = J.B.p_pack;
      e.atm = J.B.atom_g;
      e.icol = J.inv_col;
      e.inv_row = J.inv_row;
      e.pts = J.pts;
      e.perm = J.perm;
      e.npts = J.npts;
      e.out = J.out;
      e.left = J.left;
      e.done_ns = J.done_ns;
    } else {
      e.nbf = Bs.nbf;
      e.nshells = Bs.nshells;
      e.fpack = Bs.f_pack;
      e.shp = Bs.sh_pack;
      e.shr = Bs.sh_rad2_df;
      e.prm = Bs.p_pack;
      e.atm = Bs.atom_g;
      e.icol = inv_col;
      e.inv_row = inv_row;
      e.pts = pts;
      e.perm = perm;
      e.npts = npts;
      e.out = out;
      e.left = nullptr;
      e.done_ns = nullptr;
    }
    return e;
  };
  if (threadIdx.x == 0) {
    for (int s = 0; s < kStages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      mbar_init(&accfull[b], 1);
      mbar_init(&accempty[b], kEpiWarps);
    }
    for (int k = 0; k < 4; ++k) {
      mbar_init(&xfull[k], kEpiGroups - 1);
      mbar_init(&xempty[k], 1);
    }
    for (int k = 0; k < kRing; ++k) {
      mbar_init(&ring_full[k], 1);
      mbar_init(&ring_empty[k], 1 + kEpiWarps);
    }
    mbar_init(drain, 1);
    fence_barrier_init();
  }
  if (warp == 1) tmem_alloc(tmem_slot, kTmemCols);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem_base = *tmem_slot;

  // each role changes its register allocation at its start, so that the
  // compiler allocates every role's code with that role's budget
  if (warp == 0) {
    reg_dealloc_ctl();
    if (lane == 0) {
      int it = 0;  // stages issued
      bool clean = false;
      int cur_job = -1;
      for (int step = 0;; ++step) {
        // next tile step from the global queue, handed to the other roles
        const int slot = step % kRing;
        if (!mbar_wait(&ring_empty[slot], ((step / kRing) & 1) ^ 1, err, 7)) goto producer_exit;
        const int64_t t = failed() ? nsteps : static_cast<int64_t>(atomicAdd(tile_counter, 1));
        const int j = t < nsteps ? job_of(t) : 0;
        ring[slot] = t < nsteps ? static_cast<int>(t) : -1;
        ring_job[slot] = j;
        mbar_arrive(&ring_full[slot]);
        if (t >= nsteps) {
          clean = true;
          break;
        }
        const JobView v = view(j);
        if (kMulti && j != cur_job) {
          // the job's tensor maps live in global memory (written by the
          // host before the launch): acquire them for the TMA unit
          cur_job = j;
          for (const void* m : {v.a_hi, v.a_lo, v.b_hi, v.b_lo})
            asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(m) : "memory");
        }
        const int64_t tile = tile_of(v, t);
        const int m0 = static_cast<int>(tile * kBlockM);
        const int nkb = n_kb(v, tile), nchunk = n_chunk(v, tile, nkb);
        unsigned long long xw0, xw1;
        cross_words(v, tile, &xw0, &xw1);
        int c0, c1;
        chunk_span(t, nchunk, &c0, &c1);
        for (int ci = c0; ci < c1; ++ci) {
          const int c = chunk_at(v, tile, ci);
          // cross pass: (A_hi, B_lo) then (A_lo, B_hi) of every K block that
          // needs them; main pass: (A_hi, B_hi) of every K block; one pair
          // per stage
          for (int q = 0; q < 3 * nkb; ++q) {
            const bool cross = q < 2 * nkb;
            const int kb = kb_at(v, tile, cross ? q >> 1 : q - 2 * nkb);
            if (cross && !needs_cross(xw0, xw1, kb)) continue;
            const bool a_lo = cross && (q & 1), b_lo = cross && !(q & 1);
            const int s = it % kStages, round = it / kStages;
            if (!mbar_wait(&empty[s], (round & 1) ^ 1, err, 1)) goto producer_exit;
            unsigned char* st = base + s * kStageBytes;
            mbar_expect_tx(&full[s], kStageBytes);
            tma_load_2d(st, a_lo ? v.a_lo : v.a_hi, &full[s], kb * kBlockK, m0);
            tma_load_2d(st + kTileA, b_lo ? v.b_lo : v.b_hi, &full[s], kb * kBlockK, c * kBlockN);
            ++it;
          }
        }
      }
    producer_exit:
      // after an error: the loads still in flight (at most one per stage)
      // land before the CTA's shared memory is released
      if (!clean)
        for (int j = max(0, it - kStages); j < it; ++j) mbar_drain(&full[j % kStages], (j / kStages) & 1, kDrainLimitNs);
    }
  } else if (warp == 1) {
    reg_dealloc_ctl();
    if (lane == 0) {
      constexpr uint32_t idesc = idesc_f16(kBlockM, kBlockN);
      int it = 0, acc = 0;
      bool clean = false;
      for (int step = 0;; ++step) {
        const int slot = step % kRing;
        if (!mbar_wait(&ring_full[slot], (step / kRing) & 1, err, 8)) goto mma_exit;
        const int t = ring[slot], j = ring_job[slot];
        mbar_arrive(&ring_empty[slot]);
        if (t < 0) {
          clean = true;
          break;
        }
        const JobView v = view(j);
        const int64_t tile = tile_of(v, t);
        const int nkb = n_kb(v, tile), nchunk = n_chunk(v, tile, nkb);
        // the producer's stage count per chunk: two cross pieces for each K
        // block that needs them, then one main piece for every K block
        unsigned long long xw0, xw1;
        cross_words(v, tile, &xw0, &xw1);
        int nstage = nkb;
        for (int i = 0; i < nkb; ++i)
          if (needs_cross(xw0, xw1, kb_at(v, tile, i))) nstage += 2;
        int c0, c1;
        chunk_span(t, nchunk, &c0, &c1);
        for (int ci = c0; ci < c1; ++ci, ++acc) {
          const int b = acc & 1, rb = acc >> 1;
          if (!mbar_wait(&accempty[b], (rb & 1) ^ 1, err, 2)) goto mma_exit;
          tc_fence_after();
          const uint32_t d_tmem = tmem_base + b * kAccStride;
          for (int q = 0; q < nstage; ++q, ++it) {
            const int s = it % kStages, round = it / kStages;
            if (!mbar_wait(&full[s], round & 1, err, 3)) goto mma_exit;
            tc_fence_after();
            unsigned char* st = base + s * kStageBytes;
            const uint64_t a = smem_desc_sw128(st), b = smem_desc_sw128(st + kTileA);
#pragma unroll
            for (int k = 0; k < kBlockK / 16; ++k) {
              const uint64_t o = static_cast<uint64_t>(k * 32) >> 4;  // 16 fp16 = 32 bytes along K
              mma_f16(d_tmem, a + o, b + o, idesc, (q > 0 || k > 0) ? 1u : 0u);
            }
            mma_commit(&empty[s]);
          }
          mma_commit(&accfull[b]);
        }
      }
    mma_exit:
      // after an error: the MMAs already issued finish before TMEM is freed
      if (!clean) {
        mma_commit(drain);
        mbar_drain(drain, 0, kDrainLimitNs);
      }
    }
  } else if (warp >= kCtlWarps) {
    asm volatile("setmaxnreg.inc.sync.aligned.u32 %0;" ::"n"(kRegsEpi));
    // ---------------- epilogue: kEpiWarps warps ----------------
    // warp w reads TMEM lanes 32*(w%4) .. +31 (its 32 points) and handles
    // function group (w-4)/4 (kGroupF functions) of every chunk.
    const int q = warp & 3;
    const int grp = (warp - kCtlWarps) >> 2;
    const int row = q * 32 + lane;
    const uint32_t lane_base = tmem_base + (static_cast<uint32_t>(q * 32) << 16);
    int acc = 0, tk = 0;
    bool ok = true;
    for (int step = 0; ok; ++step, ++tk) {
      const int slot = step % kRing;
      if (!mbar_wait(&ring_full[slot], (step / kRing) & 1, err, 9)) break;
      const int t = ring[slot], j = ring_job[slot];
      __syncwarp();
      if (lane == 0) mbar_arrive(&ring_empty[slot]);
      if (t < 0) break;
      const JobView v = view(j);
      const EpiView ev = epi_view(j);
      const int64_t tile = tile_of(v, t);
      const int64_t p = tile * kBlockM + row;
      const bool valid = p < ev.npts;
      double r[3] = {0.0, 0.0, 0.0};
      if (valid) {
        r[0] = ev.pts[3 * p];
        r[1] = ev.pts[3 * p + 1];
        r[2] = ev.pts[3 * p + 2];
      }
      const DFloat rdf[3] = {df_split(r[0]), df_split(r[1]), df_split(r[2])};
      const float2 rg[3] = {grid_split(rdf[0]), grid_split(rdf[1]), grid_split(rdf[2])};
      // fp32 running sums over the tile's functions in this group (a
      // compensated sum across chunks changed no digit of the error against
      // the FP64 oracle: it is set by the fp16 products)
      float sum[kNDots];
#pragma unroll
      for (int i = 0; i < kNDots; ++i) sum[i] = 0.f;
      int cur_shell = -1, cur_atom = -1;
      // the next shell's record and its screening radius, loaded when a
      // shell starts (shells are contiguous in function order), so that a
      // shell change does not wait on a chain of dependent loads
      int sh_pre = -1;
      int4 pk_pre = make_int4(0, 0, 0, 0);
      float2 rad_pre = make_float2(0.f, 0.f);
      // the current shell (first function, components, l, whether they are
      // in the standard order) and its radial sums
      int sh_first = 0, sh_ncomp = 0, sh_l = 0;
      bool sh_std = false, warp_on = false;
      float f1 = 0.f, f2 = 0.f, f3 = 0.f, m2f2 = 0.f, lq = 0.f;
      // the current atom: r - R_A (the high parts) and its squared length
      float sx = 0.f, sy = 0.f, sz = 0.f, r2x4 = 0.f;
      CartPow cp = cart_pow(0.f, 0.f, 0.f);
      DFloat d2a{0.f, 0.f};
      // D's terms summed over the current atom's functions: w0 phi and w0
      // grad phi.  The X and E sums carry r - R_A, which is constant per
      // atom, so they take these sums times r - R_A when the atom changes
      // (and at the end of the tile) instead of a product per function.
      float aP = 0.f, aGx = 0.f, aGy = 0.f, aGz = 0.f;
      auto fold_atom = [&]() {
        sum[0] += aP;
        sum[1] = fmaf(sx, aP, sum[1]);
        sum[2] = fmaf(sy, aP, sum[2]);
        sum[3] = fmaf(sz, aP, sum[3]);
        sum[4 + 1] = fmaf(sy, aGx, sum[4 + 1]);  // E[x][y] = sum w0 s_y d/dx phi
        sum[4 + 2] = fmaf(sz, aGx, sum[4 + 2]);  // E[x][z]
        sum[4 + 3] = fmaf(sx, aGy, sum[4 + 3]);  // E[y][x]
        sum[4 + 5] = fmaf(sz, aGy, sum[4 + 5]);  // E[y][z]
        sum[4 + 6] = fmaf(sx, aGz, sum[4 + 6]);  // E[z][x]
        sum[4 + 7] = fmaf(sy, aGz, sum[4 + 7]);  // E[z][y]
        aP = aGx = aGy = aGz = 0.f;
      };
      // one function's terms from its seven TMEM values; the sums stay in
      // the matrices' scaled units until the combination
      auto add_function = [&](const float* v, float ph, float gx, float gy, float gz, float lp) {
        const float w0 = v[0];
        aP = fmaf(w0, ph, aP);
        aGx = fmaf(w0, gx, aGx);
        aGy = fmaf(w0, gy, aGy);
        aGz = fmaf(w0, gz, aGz);
        const float g[3] = {gx, gy, gz};
#pragma unroll
        for (int d = 0; d < 3; ++d) {
#pragma unroll
          for (int m = 0; m < 3; ++m) {
            sum[13 + 3 * d + m] = fmaf(v[1 + d], g[m], sum[13 + 3 * d + m]);
            sum[25 + 3 * d + m] = fmaf(v[4 + d], g[m], sum[25 + 3 * d + m]);
          }
          if (kDiv) {
            sum[22 + d] = fmaf(v[1 + d], lp, sum[22 + d]);
            sum[34 + d] = fmaf(v[4 + d], lp, sum[34 + d]);
          }
        }
      };
      const int nkb = n_kb(v, tile), nchunk = n_chunk(v, tile, nkb);
      int c0, c1;
      chunk_span(t, nchunk, &c0, &c1);
      for (int ci = c0; ci < c1; ++ci, ++acc) {
        const int c = chunk_at(v, tile, ci);
        const int b = acc & 1, rb = acc >> 1;
        if (!mbar_wait(&accfull[b], rb & 1, err, 4)) {
          ok = false;
          break;
        }
        tc_fence_after();
        const int f0 = c * kChunkF;
        const int mb = f0 + grp * kGroupF;
        const int me = min(f0 + min((grp + 1) * kGroupF, kChunkF), ev.nbf);
        const uint32_t tcol = lane_base + b * kAccStride;
        // a function of the current shell at column u: its TMEM loads, then
        // (while they are in flight) its value, gradient and Laplacian (all
        // zero on lanes whose shell is screened: f1 = f2 = f3 = 0 there)
        auto std_function = [&](auto idc, int u) {
          constexpr int kId = decltype(idc)::value;
          float w[kMats];
#pragma unroll
          for (int m = 0; m < kMats; ++m) tmem_ld1(tcol + m * kChunkF + u, w[m]);
          float ph, gx, gy, gz, lp = 0.f;
          cart_std<kId, kDiv>(cp, f1, m2f2, lq, &ph, &gx, &gy, &gz, &lp);
          tmem_wait7(w);
          add_function(w, ph, gx, gy, gz, lp);
        };
        int mu = mb;
#pragma unroll 1
        while (mu < me) {
          // shells are contiguous in function order: after the range's first
          // shell comes the next one
          const int sh = mu == mb ? (ev.fpack[mb] >> 12) : cur_shell + 1;
          if (sh != cur_shell) {
            cur_shell = sh;
            const bool hit = sh == sh_pre;
            // atom, first function, ncomp | npf << 8 | l << 16 | standard order << 24, first primitive
            const int4 pk = hit ? pk_pre : ev.shp[sh];
            const float2 rad = hit ? rad_pre : ev.shr[sh];
            if (sh + 1 < ev.nshells) {
              sh_pre = sh + 1;
              pk_pre = ev.shp[sh + 1];
              rad_pre = ev.shr[sh + 1];
            }
            sh_first = pk.y;
            sh_ncomp = pk.z & 0xff;
            sh_l = (pk.z >> 16) & 0xff;
            sh_std = ((pk.z >> 24) & 1) != 0;
            const int a = pk.x;
            if (a != cur_atom) {
              fold_atom();
              cur_atom = a;
              float s3[3];
              d2a = atom_offset_g(rg, ev.atm, a, s3);
              sx = s3[0];
              sy = s3[1];
              sz = s3[2];
              cp = cart_pow(sx, sy, sz);
              if (kDiv) r2x4 = 4.f * (cp.x2 + cp.y2 + cp.z2);
            }
            const bool on = df_le(d2a, rad);
            // a shell screened for all 32 points of the warp contributes
            // nothing: its functions in this range are skipped
            warp_on = __any_sync(0xffffffffu, on);
            if (warp_on) {
              f1 = f2 = f3 = 0.f;
              if (on) {
                const int np = (pk.z >> 8) & 0xff;
                for (int k = 0; k < np; ++k) {
                  const float4 pr = ev.prm[pk.w + k];  // exponent hi, exponent lo, coefficient
                  const float al = pr.x;
                  const float e = pr.z * gauss_df(al, pr.y, d2a.h, d2a.l);
                  f1 += e;
                  f2 += al * e;
                  if (kDiv) f3 += al * al * e;
                }
              }
              m2f2 = -2.f * f2;
              if (kDiv) lq = fmaf(r2x4, f3, -static_cast<float>(2 * (2 * sh_l + 3)) * f2);
            }
          }
          const int hi = min(me, sh_first + sh_ncomp);
          if (warp_on) {
            if (sh_std) {
              // components cb .. ce-1 of the shell, component k at column u0 + k
              const int cb = mu - sh_first, ce = hi - sh_first, u0 = sh_first - f0;
              auto comps = [&](auto basec, auto ncc) {
                static_for<0, decltype(ncc)::value>([&](auto kc) {
                  constexpr int k = decltype(kc)::value;
                  if (k >= cb && k < ce) std_function(std::integral_constant<int, decltype(basec)::value + k>{}, u0 + k);
                });
              };
              switch (sh_l) {
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
#pragma unroll 1
              for (int f = mu; f < hi; ++f) {
                const int u = f - f0;
                float w[kMats];
#pragma unroll
                for (int m = 0; m < kMats; ++m) tmem_ld1(tcol + m * kChunkF + u, w[m]);
                float ph, gx, gy, gz, lp = 0.f;
                cart_case(ev.fpack[f] & 0xfff, cp, f1, f2, f3, &ph, &gx, &gy, &gz, kDiv ? &lp : nullptr);
                tmem_wait7(w);
                add_function(w, ph, gx, gy, gz, lp);
              }
            }
          }
          mu = hi;
        }
        tc_fence_before();
        __syncwarp();
        if (lane == 0) mbar_arrive(&accempty[b]);
      }
      if (!ok) break;
      fold_atom();
      // combine the groups' sums of every point through `red`: groups 1..
      // write once group 0 of their lane quarter has read the previous
      // tile's sums; group 0 adds them in group order as double-floats
      float* redf = reinterpret_cast<float*>(red);  // [group - 1][sum][row]
      if (grp > 0) {
        if (!mbar_wait(&xempty[q], (tk & 1) ^ 1, err, 5)) break;
        float* dst = redf + (grp - 1) * (kNDots * kBlockM) + row;
#pragma unroll
        for (int i = 0; i < kNDots; ++i) dst[i * kBlockM] = sum[i];
        __syncwarp();
        if (lane == 0) mbar_arrive(&xfull[q]);
      } else {
        if (!mbar_wait(&xfull[q], tk & 1, err, 6)) break;
        float thi[kNDots], tlo[kNDots];
#pragma unroll
        for (int i = 0; i < kNDots; ++i) {
          DFloat a{sum[i], 0.f};
#pragma unroll
          for (int g = 1; g < kEpiGroups; ++g)
            a = df_add(a, DFloat{redf[(g - 1) * (kNDots * kBlockM) + i * kBlockM + row], 0.f});
          thi[i] = a.h;
          tlo[i] = a.l;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&xempty[q]);  // `red` is free for the next tile
        bool finish = true;  // this warp combines and stores its rows now
        if (csplit > 1) {
          // Chunk split: the step's sums of these 32 rows (all groups) go to
          // the tile's partial slot g; the warp that completes this quarter
          // of the tile (the last of the csplit steps to count) adds the
          // slots in chunk order into thi/tlo, so the result does not depend
          // on which step came last.
          const int g = static_cast<int>(t % csplit);
          const int64_t quarter = tile * 4 + q;
          if (g < nchunk) {
            float2* dst = part + (tile * csplit + g) * static_cast<int64_t>(kNDots * kBlockM) + row;
#pragma unroll
            for (int i = 0; i < kNDots; ++i) dst[i * kBlockM] = make_float2(thi[i], tlo[i]);
          }
          __threadfence();
          __syncwarp();
          unsigned last = 0;
          if (lane == 0) last = atomicAdd(tile_done + quarter, 1u) == static_cast<unsigned>(csplit - 1) ? 1u : 0u;
          finish = __shfl_sync(0xffffffffu, last, 0) != 0;
          if (finish) {
            __threadfence();
#pragma unroll
            for (int i = 0; i < kNDots; ++i) thi[i] = tlo[i] = 0.f;
            for (int gg = 0; gg < min(csplit, nchunk); ++gg) {
              const float2* src = part + (tile * csplit + gg) * static_cast<int64_t>(kNDots * kBlockM) + row;
#pragma unroll
              for (int i = 0; i < kNDots; ++i) {
                const float2 v = __ldcg(src + i * kBlockM);
                const DFloat a = df_add(DFloat{thi[i], tlo[i]}, DFloat{v.x, v.y});
                thi[i] = a.h;
                tlo[i] = a.l;
              }
            }
            if (lane == 0) tile_done[quarter] = 0;
          }
        }
        if (finish && valid) {
          // the row scale and the matrix scales are powers of two: scaling
          // a double-float is exact.  Sum i belongs to matrix dot_matrix(i).
          const float sc = ev.inv_row[p];
          float msc[kMats];
#pragma unroll
          for (int m = 0; m < kMats; ++m) msc[m] = sc * ev.icol[m];
          auto tot = [&](int i) -> DFloat {
            const float f = msc[dot_matrix(i)];
            return DFloat{thi[i] * f, tlo[i] * f};
          };
          const int64_t o = ev.perm ? static_cast<int64_t>(ev.perm[p]) : p;  // caller's point order
          if (fl.giao && fl.dia && fl.para) {
            combine_point_df(tot, rdf, [&](int k, DFloat x) { store_output(ev.out, o, k, df_to_double(x)); });
          } else {
            double td[kNDots], ct[9], dv[3];
#pragma unroll
            for (int i = 0; i < kNDots; ++i) td[i] = df_to_double(tot(i));
            combine_point(td, r, fl, ct, dv);
#pragma unroll
            for (int k = 0; k < 9; ++k) store_output(ev.out, o, k, ct[k]);
#pragma unroll
            for (int k = 0; k < 3; ++k) store_output(ev.out, o, 9 + k, dv[k]);
          }
          store_density(ev.out, o, df_to_double(tot(0)));
        }
        if (kMulti && ev.left) {
          // per-job completion time: the last of the job's 4 x ntiles
          // quarter tiles to finish stamps the global timer
          __syncwarp();
          if (lane == 0 && atomicSub(ev.left, 1) == 1) *ev.done_ns = global_ns();
        }
      }
    }
  } else {
    reg_dealloc_ctl();  // warps 2 and 3: no pipeline role
    // They pull the epilogue's tables into L1 while the first operands
    // load: in a short pass each SM sees one or two tiles on cold caches,
    // where every shell change would otherwise wait on a chain of L2 loads.
    const int t = threadIdx.x - 64;
    const DevBasis& PB = kMulti ? jobs[0].B : Bs;
    prefetch_l1(PB.f_pack, PB.nbf * sizeof(int), t, 64);
    prefetch_l1(PB.sh_pack, PB.nshells * sizeof(int4), t, 64);
    prefetch_l1(PB.sh_rad2_df, PB.nshells * sizeof(float2), t, 64);
    prefetch_l1(PB.p_pack, PB.nprim * sizeof(float4), t, 64);
    prefetch_l1(PB.atom_g, PB.natoms * 3 * sizeof(float2), t, 64);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 1) {
    tc_fence_after();
    tmem_dealloc(tmem_base, kTmemCols);
  }
}

namespace {
// Per device and instantiation, once: the shared-memory size attribute and
// the register check (the register split assumes the launch allocation;
// with fewer registers per thread the epilogue's setmaxnreg.inc could never
// be granted).  Stores the device's SM count.
template <bool kDiv, bool kMulti>
cudaError_t tc_kernel_setup(int* nsm) {
  static PerDevice pd;
  return once_per_device(pd, nsm, [](int dev, int* sms) {
    cudaError_t e = cudaFuncSetAttribute(tc_fused_kernel<kDiv, kMulti>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         kSmemBytes);
    if (e != cudaSuccess) return e;
    cudaFuncAttributes fa;
    e = cudaFuncGetAttributes(&fa, tc_fused_kernel<kDiv, kMulti>);
    if (e != cudaSuccess) return e;
    if (fa.numRegs < kRegsLaunch) return cudaErrorInvalidConfiguration;
    return cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
  });
}
}  // namespace

cudaError_t launch_tc_fused(const DevBasis& B, const TcArgs& a, cudaStream_t st) {
  if (a.npts <= 0) return cudaSuccess;
  const bool div = a.out.divt || a.out.divt32;
  int nsm = 0;
  cudaError_t e = div ? tc_kernel_setup<true, false>(&nsm) : tc_kernel_setup<false, false>(&nsm);
  if (e != cudaSuccess) return e;
  if (nsm <= 0) return cudaErrorInvalidDevice;
  const int64_t ntiles = (a.npts + kBlockM - 1) / kBlockM;
  const int csplit = std::max(1, a.csplit);
  if (csplit > 1 && (!a.part || !a.tile_done)) return cudaErrorInvalidValue;
  const unsigned grid = static_cast<unsigned>(std::min<int64_t>(ntiles * csplit, nsm));
  auto kernel = div ? tc_fused_kernel<true, false> : tc_fused_kernel<false, false>;
  kernel<<<grid, kThreads, kSmemBytes, st>>>(
      *static_cast<const CUtensorMap*>(a.tmap_a_hi), *static_cast<const CUtensorMap*>(a.tmap_a_lo),
      *static_cast<const CUtensorMap*>(a.tmap_b_hi), *static_cast<const CUtensorMap*>(a.tmap_b_lo), B,
      a.inv_row_scale, a.inv_col_scale, a.pts, a.npts, a.flags, a.out, a.err, a.tiles, a.tile_stride, a.perm,
      a.tile_order, a.tile_counter, csplit, a.part, a.tile_done, a.xneed, nullptr, 0, 0);
  return cudaGetLastError();
}

cudaError_t launch_tc_fused_multi(const TcJob* jobs, int njobs, int64_t nsteps, Flags flags, bool div, int* err,
                                  int* tile_counter, cudaStream_t st) {
  if (njobs <= 0 || nsteps <= 0) return cudaSuccess;
  if (!jobs || !err || !tile_counter) return cudaErrorInvalidValue;
  int nsm = 0;
  cudaError_t e = div ? tc_kernel_setup<true, true>(&nsm) : tc_kernel_setup<false, true>(&nsm);
  if (e != cudaSuccess) return e;
  if (nsm <= 0) return cudaErrorInvalidDevice;
  const unsigned grid = static_cast<unsigned>(std::min<int64_t>(nsteps, nsm));
  CUtensorMap none;
  std::memset(&none, 0, sizeof(none));
  const DevBasis nob{};
  const Outputs noout{nullptr, nullptr, nullptr};
  auto kernel = div ? tc_fused_kernel<true, true> : tc_fused_kernel<false, true>;
  kernel<<<grid, kThreads, kSmemBytes, st>>>(none, none, none, none, nob, nullptr, nullptr, nullptr, 0, flags,
                                             noout, err, nullptr, 0, nullptr, nullptr, tile_counter, 1, nullptr,
                                             nullptr, nullptr, jobs, njobs, nsteps);
  return cudaGetLastError();
}

}  // namespace gg
