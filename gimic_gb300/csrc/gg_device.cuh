// Device-side data layout and sm_103a PTX wrappers (mbarrier, TMA,
// tcgen05/TMEM) shared by the GB300 GIMIC kernels.
#pragma once
#include <cstdint>
#include <cuda_fp16.h>
#include <cuda_runtime.h>

namespace gg {

// Device copy of the basis.  Function arrays are indexed by the basis
// function (atom-major order, as in src/libgimic/bfeval.f90:81-122), shell
// arrays by contraction, primitive arrays by shell.prim .. shell.prim+npf.
struct DevBasis {
  int nbf;        // basis functions
  int natoms;
  int nshells;
  int kpad;       // nbf rounded up to a multiple of 64 (GEMM K extent)
  int nchunk;     // ceil(nbf / 32): 32-function column chunks of the GEMM
  const double* atom_xyz;  // natoms x 3
  const int* f_shell;      // shell of each function
  const int* f_ijk;        // Cartesian exponents packed i | j << 4 | k << 8
  const int* f_pack;       // shell << 12 | Cartesian case id (gg_cart.cuh)
  const int* sh_atom;
  const int* sh_prim;      // first primitive
  const int* sh_npf;
  const int* sh_l;         // angular momentum
  const int* sh_f0;        // first function (functions of a shell are contiguous)
  const int* sh_ncomp;     // number of Cartesian components
  const double* sh_rad2;   // squared screening radius
  const float2* sh_rad2_df;  // the same as a double-float (hi, lo)
  const float2* atom_df;     // natoms x 3 coordinates as double-floats (hi, lo)
  const float2* atom_g;      // natoms x 3 coordinates split on the 2^-12 grid (grid_split)
  const float* p_xp;       // primitive exponents (fp32, rounded)
  const float* p_xplo;     // exponent residuals: p_xpd - p_xp (fp32)
  const float* p_cc;       // normalised contraction coefficients (fp32)
  const float4* p_pack;    // {p_xp, p_xplo, p_cc, 0} per primitive
  int nprim;
  const int4* sh_pack;     // {atom, first function, ncomp | npf << 8 | l << 16 | standard order << 24, first primitive}
  const double* p_xpd;     // same in fp64
  const double* p_ccd;
  // Row-scale envelope: atom_env[a * env_bins + b] bounds log2 |phi| over all
  // in-range shells of atom a at squared distances d2 with
  // floor((log2 d2 + kEnvOffset) * kEnvPerOctave) = b (bin 0 also takes
  // every smaller d2; -inf where no shell of the atom reaches).
  const float* atom_env;
  int env_bins;
  const float4* atom_f4;   // natoms: {x, y, z, 0} in fp32 (tile screening)
  const float* sh_rad;     // screening radius in fp32, rounded up (tile screening)
};
constexpr float kEnvPerOctave = 8.f;
constexpr float kEnvOffset = 14.f;

// Flags of the tensor assembly (src/libgimic/jtensor.F90:148-237 switches)
struct Flags {
  int giao, dia, para;
};

// Per-point outputs; any pointer may be null.  The fp32 set receives the
// same values rounded once from fp64 (for large grids stored in fp32).
struct Outputs {
  double* jt;    // N x 9, column-major 3x3 (t(m,b) at m + 3b)
  double* rho;   // N
  double* divt;  // N x 3: sum_m d/dm t(m,b)
  float* jt32 = nullptr;
  float* rho32 = nullptr;
  float* divt32 = nullptr;
};

__device__ __forceinline__ void store_outputs(const Outputs& out, int64_t o, const double ct[9], double rho,
                                              const double dv[3]) {
  if (out.jt)
    for (int i = 0; i < 9; ++i) out.jt[9 * o + i] = ct[i];
  if (out.rho) out.rho[o] = rho;
  if (out.divt)
    for (int i = 0; i < 3; ++i) out.divt[3 * o + i] = dv[i];
  if (out.jt32)
    for (int i = 0; i < 9; ++i) out.jt32[9 * o + i] = static_cast<float>(ct[i]);
  if (out.rho32) out.rho32[o] = static_cast<float>(rho);
  if (out.divt32)
    for (int i = 0; i < 3; ++i) out.divt32[3 * o + i] = static_cast<float>(dv[i]);
}

// Output k of a point (ct(m, b) at m + 3 b for k < 9, div_b at 9 + b) and
// its density, for whichever of the output arrays are set.
__device__ __forceinline__ void store_output(const Outputs& out, int64_t o, int k, double v) {
  if (k < 9) {
    if (out.jt) out.jt[9 * o + k] = v;
    if (out.jt32) out.jt32[9 * o + k] = static_cast<float>(v);
  } else {
    if (out.divt) out.divt[3 * o + (k - 9)] = v;
    if (out.divt32) out.divt32[3 * o + (k - 9)] = static_cast<float>(v);
  }
}
__device__ __forceinline__ void store_density(const Outputs& out, int64_t o, double rho) {
  if (out.rho) out.rho[o] = rho;
  if (out.rho32) out.rho32[o] = static_cast<float>(rho);
}

// Split-FP16 GEMM geometry
constexpr int kChunkF = 32;              // functions per column chunk
constexpr int kMats = 7;                 // D, C_x, C_y, C_z, P_x, P_y, P_z
constexpr int kBlockN = kMats * kChunkF; // 224 GEMM columns per chunk
constexpr int kBlockM = 128;             // points per CTA tile
constexpr int kBlockK = 64;              // fp16 elements per 128-byte row
constexpr float kScaleTarget = 16384.0f; // |scaled value| < 2^14

// exp(-alpha r^2) in fp32 with the argument carried as a double-float:
// alpha = ah + al, r^2 = rh + rl (both splits of fp64 values).  The product
// error is recovered with an fma and applied to first order, so the result
// is as accurate as expf itself even for large arguments.
__device__ __forceinline__ float gauss_df(float ah, float al, float rh, float rl) {
  const float xh = ah * rh;
  const float xe = fmaf(ah, rh, -xh);
  const float xl = xe + fmaf(ah, rl, al * rh);
  return expf(-xh) * (1.0f - xl);
}

// Double-float arithmetic (value = hi + lo, |lo| <= ulp(hi) / 2) in fp32.
// The FP64 pipe of this GPU issues 64 times fewer operations per cycle than
// the fp32 pipe, so per-function and per-shell geometry (r - R_A, |r - R_A|^2
// and the screening test) is carried this way, with about 44 significant
// bits, and fp64 is kept for per-point work.
struct DFloat {
  float h, l;
};

__device__ __forceinline__ DFloat df_split(double x) {
  const float h = static_cast<float>(x);
  return {h, static_cast<float>(x - static_cast<double>(h))};
}

// Knuth's two-sum: s + e == a + b exactly
__device__ __forceinline__ DFloat two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// Dekker's fast two-sum, |a| >= |b|
__device__ __forceinline__ DFloat fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

__device__ __forceinline__ DFloat df_add(DFloat a, DFloat b) {
  const DFloat s = two_sum(a.h, b.h);
  return fast_two_sum(s.h, __fadd_rn(s.l, __fadd_rn(a.l, b.l)));
}

// (a.h + a.l) * (b.h + b.l), the product error recovered by fmas
__device__ __forceinline__ DFloat df_mul(DFloat a, DFloat b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  return fast_two_sum(p, e);
}

__device__ __forceinline__ DFloat df_sub(DFloat a, DFloat b) { return df_add(a, DFloat{-b.h, -b.l}); }

__device__ __forceinline__ double df_to_double(DFloat a) {
  return static_cast<double>(a.h) + static_cast<double>(a.l);
}

// a <= b for normalised double-floats
__device__ __forceinline__ bool df_le(DFloat a, float2 b) { return a.h < b.x || (a.h == b.x && a.l <= b.y); }

// Grid split of a coordinate: x = g + l with g a multiple of 2^-12 and
// |l| <= 2^-13 + ulp(x) / 2 (for |x| < 2^12 Bohr; beyond, g is x rounded to
// fp32).  Two
// grid-split coordinates below 2^12 in magnitude differ by an exact fp32
// difference of the g parts plus a small one of the l parts, which makes
// r - R_A cheap to form without losing digits.
constexpr float kGridScale = 4096.f;
__device__ __forceinline__ float2 grid_split(DFloat x) {
  const float g = __fmul_rn(rintf(__fmul_rn(x.h, kGridScale)), 1.f / kGridScale);  // exact scalings
  return make_float2(g, __fadd_rn(__fsub_rn(x.h, g), x.l));                       // x.h - g is exact
}

// Position of a point relative to atom a (fp32, rounded once) and its
// squared distance as a double-float, from the grid splits of the point
// (rg) and of the atom table.  d = dh + dl with dh = g_r - g_A exact and
// |dl| about 2^-12 at most; d^2 = dh^2 (exact as p + e) + dl (2 dh + dl).
// The low parts carry about 2^-36 Bohr of rounding, so on random points
// (restated in fp32 on the CPU, tests/test_numerics.py) the error of d^2
// stays below 2^-33 |d| + 2^-45 Bohr^2: a relative 2^-33 once |d| >= 1
// Bohr, far below what the fp32 exponential of alpha d^2 resolves.
__device__ __forceinline__ DFloat atom_offset_g(const float2 rg[3], const float2* atom_g, int a, float s[3]) {
  float dh[3], p[3], lo = 0.f;
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    const float2 A = atom_g[3 * a + c];
    dh[c] = __fsub_rn(rg[c].x, A.x);
    const float dl = __fsub_rn(rg[c].y, A.y);
    s[c] = __fadd_rn(dh[c], dl);
    p[c] = __fmul_rn(dh[c], dh[c]);
    lo = __fadd_rn(lo, fmaf(dh[c], dh[c], -p[c]));
    lo = fmaf(dl, fmaf(2.f, dh[c], dl), lo);
  }
  const DFloat a1 = two_sum(p[0], p[1]);
  const DFloat a2 = two_sum(a1.h, p[2]);
  return two_sum(a2.h, __fadd_rn(__fadd_rn(a1.l, a2.l), lo));
}

__device__ __forceinline__ int ipow_exp(int packed, int axis) { return (packed >> (4 * axis)) & 15; }

template <typename T>
__device__ __forceinline__ T powi(T x, int n) {
  T r = T(1);
  for (int i = 0; i < n; ++i) r *= x;
  return r;
}

// Value, gradient and Laplacian of one Cartesian component
// x^i y^j z^k f(r^2) with f1 = sum c e^{-a r^2}, f2 = sum a c e^{-a r^2},
// f3 = sum a^2 c e^{-a r^2} (gradient as in src/libgimic/caos.f90:39-64).
template <typename T>
__device__ __forceinline__ void cart_eval(int packed, T x, T y, T z, T f1, T f2, T f3, T* phi, T* gx, T* gy, T* gz,
                                          T* lap) {
  const int i = packed & 15, j = (packed >> 4) & 15, k = (packed >> 8) & 15;
  const T xi = powi(x, i), yj = powi(y, j), zk = powi(z, k);
  const T xi1 = i > 0 ? powi(x, i - 1) : T(0);
  const T yj1 = j > 0 ? powi(y, j - 1) : T(0);
  const T zk1 = k > 0 ? powi(z, k - 1) : T(0);
  const T xi2 = i > 1 ? powi(x, i - 2) : T(0);
  const T yj2 = j > 1 ? powi(y, j - 2) : T(0);
  const T zk2 = k > 1 ? powi(z, k - 2) : T(0);
  const T xp1 = xi * x, yp1 = yj * y, zp1 = zk * z;
  const T yz = yj * zk, xz = xi * zk, xy = xi * yj;
  *phi = xi * yz * f1;
  *gx = (T(i) * xi1 * f1 - T(2) * xp1 * f2) * yz;
  *gy = (T(j) * yj1 * f1 - T(2) * yp1 * f2) * xz;
  *gz = (T(k) * zk1 * f1 - T(2) * zp1 * f2) * xy;
  if (lap) {
    const T r2 = x * x + y * y + z * z;
    const T second = T(i * (i - 1)) * xi2 * yz + T(j * (j - 1)) * yj2 * xz + T(k * (k - 1)) * zk2 * xy;
    *lap = second * f1 - T(2 * (2 * (i + j + k) + 3)) * xi * yz * f2 + T(4) * r2 * xi * yz * f3;
  }
}

// --------------------------------------------------------------------------
// PTX wrappers
// --------------------------------------------------------------------------
// Pulls `bytes` of a read-only table into L1, one 128-byte line per thread
// of the CTA at a time (only a hint: no data is returned).
// Thread t of n threads takes lines t, t + n, ...
__device__ __forceinline__ void prefetch_l1(const void* p, size_t bytes, int t, int n) {
  const char* c = static_cast<const char*>(p);
  for (size_t o = static_cast<size_t>(t) * 128; o < bytes; o += static_cast<size_t>(n) * 128)
    asm volatile("prefetch.global.L1 [%0];" ::"l"(c + o));
}
__device__ __forceinline__ void prefetch_l1(const void* p, size_t bytes) {
  prefetch_l1(p, bytes, static_cast<int>(threadIdx.x), static_cast<int>(blockDim.x));
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
  return t;
}

// Bounded wait: gives up after limit_ns (or 2^26 polls), or as soon as
// another thread of the grid has reported an error; sets *err (to `code`,
// unless an error is already recorded) and returns false.
__device__ __forceinline__ bool mbar_wait_for(uint64_t* bar, uint32_t parity, int* err, int code, uint64_t limit_ns) {
  if (mbar_try_wait(bar, parity)) return true;
  const uint64_t t0 = global_ns();
  for (int it = 1; it < (1 << 26); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255) == 0) {
      if (*reinterpret_cast<volatile int*>(err) != 0) return false;
      if (global_ns() - t0 > limit_ns) break;
    }
  }
  atomicCAS(err, 0, code);
  return false;
}

// Bounded wait that ignores the error word, for the way out after an error:
// it lets this thread's own copies or MMAs in flight land before the CTA's
// shared memory and TMEM are released.  Returns false if they did not land
// within limit_ns.
__device__ __forceinline__ bool mbar_drain(uint64_t* bar, uint32_t parity, uint64_t limit_ns) {
  const uint64_t t0 = global_ns();
  for (int it = 0; it < (1 << 26); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if ((it & 255) == 255 && global_ns() - t0 > limit_ns) return false;
  }
  return false;
}
constexpr uint64_t kDrainLimitNs = 1000000000ull;

// The pipeline kernels' wait: about 4 s at most.
constexpr uint64_t kWaitLimitNs = 4000000000ull;
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code) {
  return mbar_wait_for(bar, parity, err, code, kWaitLimitNs);
}

__device__ __forceinline__ void fence_barrier_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void tma_load_2d(void* dst, const void* tmap, uint64_t* bar, int c0, int c1) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::"r"(
          smem_u32(dst)),
      "l"(reinterpret_cast<uint64_t>(tmap)), "r"(smem_u32(bar)), "r"(c0), "r"(c1)
      : "memory");
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
               "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// D[tmem] (+)= A[smem] * B[smem]^T, fp16 inputs, fp32 accumulate
__device__ __forceinline__ void mma_f16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                        uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}

// mbarrier arrives once all previously issued MMAs of this thread complete
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}

// Shared-memory matrix descriptor (tcgen05 format): K-major operand whose
// rows are 128 bytes, 128-byte swizzle, 8-row groups 1024 bytes apart.
__device__ __forceinline__ uint64_t smem_desc_sw128(const void* tile) {
  const uint64_t addr = smem_u32(tile);
  uint64_t d = 0;
  d |= (addr >> 4) & 0x3FFFull;           // start address
  d |= (uint64_t)(16 >> 4) << 16;         // leading byte offset (unused with swizzle)
  d |= (uint64_t)(1024 >> 4) << 32;       // stride byte offset
  d |= 1ull << 46;                        // descriptor version (tcgen05)
  d |= 2ull << 61;                        // SWIZZLE_128B
  return d;
}

// Instruction descriptor: kind::f16, fp16 A/B, fp32 D, K-major A and B.
__host__ __device__ constexpr uint32_t idesc_f16(int m, int n) {
  return (1u << 4)                            // D format: f32
         | (0u << 7) | (0u << 10)             // A, B format: f16
         | (0u << 15) | (0u << 16)            // A, B K-major
         | ((uint32_t)(n >> 3) << 17)         // N
         | ((uint32_t)(m >> 4) << 24);        // M
}

}  // namespace gg
