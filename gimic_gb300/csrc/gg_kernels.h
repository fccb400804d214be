// Kernel launchers of the GB300 GIMIC path (host-callable, stream-ordered).
#pragma once
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "gg_device.cuh"

namespace gg {

// Number of per-point bilinear forms produced by the contraction; layout:
//   0 rho = W0.phi           1..3 X_c = W0.(s_c phi)     4..12 E_mc = W0.(s_c g_m)
//   13..21 Y_dm = WC_d.g_m   22..24 YL_d = WC_d.lap      25..33 Z_bm = Q_b.g_m
//   34..36 ZL_b = Q_b.lap
// with W0 = phi^T D, WC_d = phi^T C_d, Q_b = phi^T P_b and s = r - R_atom.
constexpr int kNDots = 37;

// Shell-blocked basis evaluation for the split-FP16 point operand
// (k_basis_tile.cu): one thread per point, the row scale from a log-domain
// bound, K blocks staged in shared memory and written with TMA tensor stores
// through the point operand's own tensor maps; with tile lists, inactive K
// blocks are skipped.
//
// Cross products: xneed (null: none) holds two 64-bit words per tile, one
// bit per half K block (32 functions), all ones on entry.  The kernel
// clears the bit of every half block whose scaled values are all below
// kCrossSkipScaled in magnitude for every point of the tile: 2^-14 of the
// row-scale bound (2^14), itself at least the row's largest value (and
// within 2^7 of it on the seeded bases).  The lo part of an fp16 split is at
// most 2^-11 of the value, so for such a block the two cross products of the
// split (hi*lo, lo*hi) add at most 2^-24 of the row bound times the matrix
// entry per term (tests/test_numerics.py): about one fp32 rounding of the
// products of the row's largest values.  The contraction issues only the
// block's main product (hi*hi).
//
// screen_out (short passes, no more tiles than SMs, only): no tile screen
// ran before; the kernel screens every tile itself, writes the lists to
// screen_out (as launch_tile_screen would, tiles is then ignored) and sets
// the xneed bits it owns before clearing them (xneed need not be set on
// entry).
constexpr float kCrossSkipScaled = 1.0f;
cudaError_t launch_basis_tile(const DevBasis& B, const void* tm_hi, const void* tm_lo, const double* pts,
                              int64_t npts, const int* tiles, int stride, float* inv_scale,
                              unsigned long long* xneed, int* screen_out, cudaStream_t st);
// phi, grad phi and the Laplacian in fp64 for the plain FP64 path.
void launch_basis_fp64(const DevBasis& B, const double* pts, int64_t npts, int64_t ld, double* phi, double* gx,
                       double* gy, double* gz, double* lap, cudaStream_t st);

// C[M][N] = A[M][K] B[K][N], fp64, row-major with leading dimensions.
void launch_dgemm(const double* A, int64_t lda, const double* B, int64_t ldb, double* C, int64_t ldc, int64_t M,
                  int64_t N, int64_t K, cudaStream_t st);
// The same product restricted by tile lists (points in Z order, tiles of 128
// rows): per tile, the columns of its active 32-function chunks of each of
// the 7 matrices (M has ldm = 7 ld columns, block m at column m ld), summed
// over its active 64-function K blocks.  Other columns are not written.
void launch_dgemm_tiles(const double* phi, int64_t ld, const double* M, int64_t ldm, double* W, int64_t ldw,
                        int64_t n, int nbf, const int* tiles, int stride, int nchunk, cudaStream_t st);

// Plain FP64 assembly from W = phi^T [D | C_x C_y C_z | P_x P_y P_z]
// (row stride ldw, block m at column m * nbf) and fp64 basis values.  With
// tile lists only the active chunks of each point's tile are read, and the
// outputs of sorted point p go to perm[p] (null: p).
void launch_assemble_fp64(const DevBasis& B, const double* pts, int64_t npts, const double* W, int64_t ldw,
                          const double* phi, const double* gx, const double* gy, const double* gz, const double* lap,
                          int64_t ld, Flags fl, Outputs out, const int* tiles, int stride, const int* perm,
                          cudaStream_t st);

// Split-FP16 tensor-core path: TMA maps are opaque 128-byte CUtensorMap blobs.
struct TcArgs {
  const void* tmap_a_hi;
  const void* tmap_a_lo;
  const void* tmap_b_hi;
  const void* tmap_b_lo;
  const float* inv_row_scale;  // per point
  const float* inv_col_scale;  // [7]: inverse power-of-two scale of each matrix
  const double* pts;
  int64_t npts;
  Flags flags;
  Outputs out;
  int* err;                    // device error word (0 = ok)
  const int* tiles = nullptr;  // per-tile active chunk / K-block lists (null: all)
  int tile_stride = 0;
  const int* perm = nullptr;   // output index of each (sorted) point (null: identity)
  const int* tile_order = nullptr;  // tile of each queue step (null: step i -> tile i)
  int* tile_counter = nullptr;      // device int, zero at launch: the tile queue
  // Chunk split for short passes (at most one tile per SM): every active
  // chunk of a tile is its own step, on its own SM; csplit = the basis'
  // chunk count, part = ntiles x csplit x kNDots x 128 float2 of partial
  // sums, tile_done = ntiles x 4 counters (zero at launch, zero again after).
  int csplit = 1;
  float2* part = nullptr;
  unsigned* tile_done = nullptr;
  // per tile, the half K blocks that need the cross products (as cleared by
  // launch_basis_tile; null: all of them)
  const unsigned long long* xneed = nullptr;
};
int tc_smem_bytes();

// One job of a multi-job contraction launch: one molecule's pass, with the
// operands, tables and outputs that a single-job launch takes as
// arguments.  Lives in device memory (the tensor maps are read from there
// by the TMA unit).  Steps of all jobs are numbered in table order: job j
// owns its ntiles steps from step0 on.
struct TcJob {
  alignas(64) unsigned char tmap[4][128];  // CUtensorMap: point operand hi, lo; matrix operand hi, lo
  DevBasis B;
  const float* inv_row;
  const float* inv_col;
  const double* pts;
  int64_t npts;
  Outputs out;
  const int* tiles;
  int tstride;
  const unsigned long long* xneed;  // as TcArgs::xneed
  const int* perm;
  const int* tile_order;
  int64_t step0;
  int* left;                    // 4 x ntiles quarter tiles still to finish (null: no timing)
  unsigned long long* done_ns;  // global timer (ns) when the last of them finished
};

// Spatial ordering and tile screening (k_tiles.cu)
int tile_stride(const DevBasis& B);
size_t sort_temp_bytes(int64_t n);
cudaError_t launch_spatial_order(const double* pts, int64_t n, const double lo[3], double cell, uint32_t* keys,
                                 uint32_t* keys_sorted, int* idx, int* perm, void* temp, size_t temp_bytes,
                                 double* pts_sorted, cudaStream_t st);
// xneed (may be null): the cross-product mask of the tiles (TcArgs::xneed),
// set to all ones here for the basis kernel to clear.
void launch_tile_screen(const DevBasis& B, const double* pts_sorted, int64_t n, int* tiles, unsigned long long* xneed,
                        cudaStream_t st);
void launch_tile_work(const int* tiles, int64_t ntiles, int stride, unsigned long long* acc, cudaStream_t st);
// acc += the blocks (chunks x K blocks) of the tiles whose K block needs the
// cross products (xneed as TcArgs::xneed; profiling)
void launch_cross_work(const int* tiles, const unsigned long long* xneed, int64_t ntiles, int stride, int nchunk,
                       unsigned long long* acc, cudaStream_t st);
// Tiles ordered by decreasing GEMM work (blocks = chunks x K blocks), so that
// the heaviest tiles start first and the tail of the launch is short.
size_t tile_order_temp_bytes(int64_t ntiles);
cudaError_t launch_tile_order(const int* tiles, int64_t ntiles, int stride, uint32_t* work, uint32_t* work_sorted,
                              int* ids, int* order, void* temp, size_t temp_bytes, cudaStream_t st);
cudaError_t launch_tc_fused(const DevBasis& B, const TcArgs& a, cudaStream_t st);
// One persistent launch over njobs jobs (device table), nsteps tiles in all;
// div: the jobs' outputs include div j (all jobs alike).
cudaError_t launch_tc_fused_multi(const TcJob* jobs, int njobs, int64_t nsteps, Flags flags, bool div, int* err,
                                  int* tile_counter, cudaStream_t st);

// Many planes at once: plane q owns points [pt_off, pt_off + p1*p2*p3) of jt
// and pts, and weights w[w_off ..] (p1 values, then p2, then p3).
struct PlaneDesc {
  int64_t pt_off;
  int64_t row_off;  // first row of this plane in the flattened row list
  int p1, p2, p3;
  int w_off;
  double center[3];
  double normal[3];
  double radius;
  double origin[3];
  double basv[9];  // basv[3 d + c]: component c of axis d
  int x_off;       // axis coordinates xs[x_off ..] (p1 values, then p2, then p3)
};
// Points of every plane, r(i,j,k) = origin + x1_i basv1 + x2_j basv2 +
// x3_k basv3 in the host's operation order (no fused multiply-adds), one
// block per plane row.  Block 0 also zeroes the nplanes counters `done` of
// the plane reduction that follows on the same stream.
void launch_plane_points(const double* xs, const PlaneDesc* planes, const int* row_plane, int64_t nrows, double* pts,
                         unsigned* done, int nplanes, cudaStream_t st);
// field: the magnetic field vector (3 doubles) in device memory; done:
// nplanes counters, zero at launch (and zero again when it ends).
void launch_plane_batch(const double* jt, const double* pts, const double* w, const PlaneDesc* planes, int nplanes,
                        const int* row_plane, int64_t nrows, const double* field, double* row_out, double* out,
                        unsigned* done, cudaStream_t st);

// Shielding of every centre and magnetizability over a molecular grid whose
// points come in nblocks consecutive blocks [block_off[l], block_off[l+1]):
// sigma_out[(k * nblocks + l) * 5 + q], chi_out[l * 5 + q] with q = the three
// diagonal sums, then the positive and negative parts (k_reduce.cu).
void launch_properties(const double* jt, const double* pts, const double* w, const double* centres, int ncentres,
                       const int64_t* block_off, int nblocks, double* sigma_out, double* chi_out, cudaStream_t st);

// Self-test of the bounded waits (k_diag.cu): one thread waits limit_ns on
// an mbarrier that nothing arrives at and records `code` in *err; the time
// it waited goes to *waited_ns (device memory, may be null).
cudaError_t launch_wait_timeout(int* err, uint64_t limit_ns, int code, unsigned long long* waited_ns,
                                cudaStream_t st);

// One global-timer stamp in *p (k_diag.cu).
cudaError_t launch_stamp(unsigned long long* p, cudaStream_t st);

// Integration proposal network (k_mlp.cu): 5 -> 64 -> 64 -> 1, SiLU.
constexpr int kMlpIn = 5;
constexpr int kMlpHidden = 64;
constexpr int kMlpParams = kMlpHidden * kMlpIn + kMlpHidden + kMlpHidden * kMlpHidden + kMlpHidden + kMlpHidden + 1;
void launch_mlp_train(const float* params, const float* x, const float* t, int n, float* grad, float* loss,
                      cudaStream_t st);
void launch_mlp_adam(float* params, const float* grad, float* m, float* v, float lr, float b1, float b2, float eps, int step,
                     cudaStream_t st);
void launch_mlp_infer(const float* params, const float* x, int n, float* y, cudaStream_t st);
void launch_mlp_features(const DevBasis& B, const double* pts, const double* uv, int64_t n, float* feats,
                         cudaStream_t st);

}  // namespace gg
