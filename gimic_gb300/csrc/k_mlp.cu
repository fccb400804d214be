// Learned integration proposal: a 5 -> 64 -> 64 -> 1 multilayer perceptron
// with SiLU activations that predicts log|j . n| on an integration plane from
// cheap geometric features.  The plane integrator uses it to decide where a
// quadtree of Gauss-Lobatto panels is refined; the uniform-grid integral
// stays the judge (no reference counterpart: GIMIC integrates on fixed grids).
//
//  * mlp_train_kernel: forward + backward of a minibatch of samples, one
//    thread per sample, weights in shared memory, gradients reduced per block
//    (hidden activations staged in shared memory) and added to a global fp32
//    gradient buffer; loss = mean (y - t)^2.
//  * mlp_adam_kernel: Adam update of the fp32 master weights.
//  * mlp_infer_kernel: inference with bf16-rounded weights and activations
//    (fp32 arithmetic on bf16 values).
//  * mlp_features_kernel: the five input features of a plane point.
//
// Parameter layout (fp32, kMlpParams values):
//   W1[64][5] b1[64] W2[64][64] b2[64] W3[64] b3[1]
#include <cuda_bf16.h>

#include "gg_kernels.h"

namespace gg {

namespace {
constexpr int kIn = kMlpIn, kH = kMlpHidden;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH, oB3 = oW3 + kH;
constexpr int kTrainThreads = 128;
constexpr int kTrainSmemStage = kMlpParams + kTrainThreads * (kH + 1);
constexpr size_t kTrainSmemBytes = sizeof(float) * (kTrainSmemStage + kTrainThreads * (kH + 1));

// Training uses expf (full fp32 accuracy); bf16 inference the fast __expf.
__device__ __forceinline__ float silu(float z) { return z / (1.f + expf(-z)); }
__device__ __forceinline__ float dsilu(float z) {
  const float s = 1.f / (1.f + expf(-z));
  return s * (1.f + z * (1.f - s));
}
__device__ __forceinline__ float silu_fast(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float bf(float x) { return __bfloat162float(__float2bfloat16_rn(x)); }
}  // namespace

static_assert(oB3 + 1 == kMlpParams, "parameter layout");

__global__ void __launch_bounds__(kTrainThreads) mlp_train_kernel(const float* __restrict__ params,
                                                                  const float* __restrict__ x,
                                                                  const float* __restrict__ target, int n,
                                                                  float* __restrict__ grad, float* __restrict__ loss) {
  extern __shared__ float train_smem[];
  float* w = train_smem;                                                          // kMlpParams
  float(*h1s)[kH + 1] = reinterpret_cast<float(*)[kH + 1]>(w + kMlpParams);       // h1 of each sample
  float(*d2s)[kH + 1] = reinterpret_cast<float(*)[kH + 1]>(w + kTrainSmemStage);  // dL/dz2 of each sample
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) w[i] = params[i];
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool valid = i < n;
  float xin[kIn] = {0, 0, 0, 0, 0};
  if (valid)
    for (int k = 0; k < kIn; ++k) xin[k] = x[static_cast<int64_t>(i) * kIn + k];
  float z1[kH], h1[kH];
#pragma unroll 8
  for (int o = 0; o < kH; ++o) {
    float a = w[oB1 + o];
    for (int k = 0; k < kIn; ++k) a = fmaf(w[oW1 + o * kIn + k], xin[k], a);
    z1[o] = a;
    h1[o] = silu(a);
  }
  float y = w[oB3];
  float d2[kH];
  for (int o = 0; o < kH; ++o) {
    float a = w[oB2 + o];
#pragma unroll 8
    for (int k = 0; k < kH; ++k) a = fmaf(w[oW2 + o * kH + k], h1[k], a);
    d2[o] = a;  // z2 for now
    y = fmaf(w[oW3 + o], silu(a), y);
  }
  const float err = valid ? y - target[i] : 0.f;
  const float dy = valid ? 2.f * err / static_cast<float>(n) : 0.f;
  if (loss) {
    float l = valid ? err * err / static_cast<float>(n) : 0.f;
    for (int off = 16; off > 0; off >>= 1) l += __shfl_xor_sync(0xffffffffu, l, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, l);
  }
  // dL/dW3 = dy h2, dL/db3 = dy, dL/dz2 = dy W3 silu'(z2)
  for (int o = 0; o < kH; ++o) {
    const float z2 = d2[o];
    d2[o] = dy * w[oW3 + o] * dsilu(z2);
    float g3 = dy * silu(z2);
    for (int off = 16; off > 0; off >>= 1) g3 += __shfl_xor_sync(0xffffffffu, g3, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(&grad[oW3 + o], g3);
  }
  {
    float g = dy;
    for (int off = 16; off > 0; off >>= 1) g += __shfl_xor_sync(0xffffffffu, g, off);
    if ((threadIdx.x & 31) == 0) atomicAdd(&grad[oB3], g);
  }
  // dL/dz1 = (W2^T dL/dz2) silu'(z1)
  float d1[kH];
  for (int k = 0; k < kH; ++k) {
    float a = 0.f;
#pragma unroll 8
    for (int o = 0; o < kH; ++o) a = fmaf(w[oW2 + o * kH + k], d2[o], a);
    d1[k] = a * dsilu(z1[k]);
  }
  for (int k = 0; k < kH; ++k) {
    h1s[threadIdx.x][k] = h1[k];
    d2s[threadIdx.x][k] = d2[k];
  }
  // dW1, db1 (per sample, warp-reduced)
  for (int o = 0; o < kH; ++o) {
    float gb = d1[o];
    float gw[kIn];
    for (int k = 0; k < kIn; ++k) gw[k] = d1[o] * xin[k];
    for (int off = 16; off > 0; off >>= 1) {
      gb += __shfl_xor_sync(0xffffffffu, gb, off);
      for (int k = 0; k < kIn; ++k) gw[k] += __shfl_xor_sync(0xffffffffu, gw[k], off);
    }
    if ((threadIdx.x & 31) == 0) {
      atomicAdd(&grad[oB1 + o], gb);
      for (int k = 0; k < kIn; ++k) atomicAdd(&grad[oW1 + o * kIn + k], gw[k]);
    }
  }
  __syncthreads();
  // dW2[o][k] = sum over the block's samples of dz2[o] h1[k], a 4 x 8 tile
  // of it per thread (twelve shared-memory loads feed 32 FMAs per sample;
  // each entry still adds the samples in order); db2[o] = sum dz2[o]
  static_assert(kTrainThreads == 128 && kH == 64, "dW2 tiles: 16 x 8 threads of 4 x 8 entries");
  {
    const int ty = threadIdx.x >> 3, tx = threadIdx.x & 7;
    float acc[4][8];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 8; ++b) acc[a][b] = 0.f;
    for (int s = 0; s < kTrainThreads; ++s) {
      float dv[4], hv[8];
#pragma unroll
      for (int a = 0; a < 4; ++a) dv[a] = d2s[s][4 * ty + a];
#pragma unroll
      for (int b = 0; b < 8; ++b) hv[b] = h1s[s][8 * tx + b];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 8; ++b) acc[a][b] = fmaf(dv[a], hv[b], acc[a][b]);
    }
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
      for (int b = 0; b < 8; ++b) atomicAdd(&grad[oW2 + (4 * ty + a) * kH + 8 * tx + b], acc[a][b]);
  }
  if (threadIdx.x < kH) {
    float a = 0.f;
    for (int s = 0; s < kTrainThreads; ++s) a += d2s[s][threadIdx.x];
    atomicAdd(&grad[oB2 + threadIdx.x], a);
  }
}

__global__ void mlp_adam_kernel(float* __restrict__ params, const float* __restrict__ grad, float* __restrict__ m,
                                float* __restrict__ v, float lr, float beta1, float beta2, float eps, int step) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= kMlpParams) return;
  const float g = grad[i];
  const float mi = beta1 * m[i] + (1.f - beta1) * g;
  const float vi = beta2 * v[i] + (1.f - beta2) * g * g;
  m[i] = mi;
  v[i] = vi;
  const float mh = mi / (1.f - powf(beta1, static_cast<float>(step)));
  const float vh = vi / (1.f - powf(beta2, static_cast<float>(step)));
  params[i] -= lr * mh / (sqrtf(vh) + eps);
}

// bf16 inference: weights and activations rounded to bf16, fp32 arithmetic.
__global__ void __launch_bounds__(256) mlp_infer_kernel(const float* __restrict__ params, const float* __restrict__ x,
                                                        int n, float* __restrict__ y) {
  __shared__ __align__(16) float w[kMlpParams];
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) w[i] = bf(params[i]);
  __syncthreads();
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float xin[kIn];
  for (int k = 0; k < kIn; ++k) xin[k] = bf(x[static_cast<int64_t>(i) * kIn + k]);
  // the hidden activations stay in registers (the layer loops are unrolled,
  // so every index is a constant), and the second layer reads its weights
  // four per shared-memory load; the same FMAs in the same order as a plain
  // loop
  float h1[kH];
#pragma unroll
  for (int o = 0; o < kH; ++o) {
    float a = w[oB1 + o];
#pragma unroll
    for (int k = 0; k < kIn; ++k) a = fmaf(w[oW1 + o * kIn + k], xin[k], a);
    h1[o] = bf(silu_fast(a));
  }
  float out = w[oB3];
  static_assert(oW2 % 4 == 0 && kH % 4 == 0, "16-byte aligned weight rows");
  for (int o = 0; o < kH; ++o) {
    float a = w[oB2 + o];
    const float4* wr = reinterpret_cast<const float4*>(w + oW2 + o * kH);
#pragma unroll
    for (int k4 = 0; k4 < kH / 4; ++k4) {
      const float4 q = wr[k4];
      a = fmaf(q.x, h1[4 * k4], a);
      a = fmaf(q.y, h1[4 * k4 + 1], a);
      a = fmaf(q.z, h1[4 * k4 + 2], a);
      a = fmaf(q.w, h1[4 * k4 + 3], a);
    }
    out = fmaf(w[oW3 + o], bf(silu_fast(a)), out);
  }
  y[i] = out;
}

// Features of a point r on an integration plane with in-plane coordinates
// (u, v) in Bohr:
//   f0 = u / 8, f1 = v / 8;
//   f2, f3 = ln of the distances to the nearest and second-nearest nucleus
//            (Bohr, floored at 0.05);
//   f4 = log10(1e-6 + sum_s sqrt(a_s) exp(-a_s d_s^2)) / 3, the local
//        shell-exponent density: a_s is the smallest exponent of shell s and
//        d_s the distance to its centre.
// All in fp32: the offsets r - R_A from grid splits (exact differences of
// the high parts), |r - R_A|^2 as a double-float and the exponential with a
// double-float argument (gauss_df), so the features agree with the FP64
// formulas to a few fp32 roundings; the FP64 pipe stays idle.
__global__ void __launch_bounds__(256) mlp_features_kernel(DevBasis B, const double* __restrict__ pts,
                                                           const double* __restrict__ uv, int64_t n,
                                                           float* __restrict__ f) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float2 rg[3] = {grid_split(df_split(pts[3 * i])), grid_split(df_split(pts[3 * i + 1])),
                        grid_split(df_split(pts[3 * i + 2]))};
  float n1 = INFINITY, n2 = INFINITY;
  float s3[3];
  for (int a = 0; a < B.natoms; ++a) {
    const float d2 = atom_offset_g(rg, B.atom_g, a, s3).h;
    if (d2 < n1) {
      n2 = n1;
      n1 = d2;
    } else if (d2 < n2) {
      n2 = d2;
    }
  }
  if (B.natoms < 2) n2 = n1;
  DFloat dens{0.f, 0.f};  // a compensated sum over the shells
  int cur = -1;
  DFloat d2a{0.f, 0.f};
  for (int s = 0; s < B.nshells; ++s) {
    const int a = __ldg(B.sh_atom + s), p0 = __ldg(B.sh_prim + s), np = __ldg(B.sh_npf + s);
    if (a != cur) {
      cur = a;
      d2a = atom_offset_g(rg, B.atom_g, a, s3);
    }
    // the smallest exponent of the shell, as its (hi, lo) pair
    float4 pm = __ldg(B.p_pack + p0);
    for (int q = 1; q < np; ++q) {
      const float4 pq = __ldg(B.p_pack + p0 + q);
      if (pq.x + pq.y < pm.x + pm.y) pm = pq;
    }
    dens = df_add(dens, DFloat{sqrtf(pm.x) * gauss_df(pm.x, pm.y, d2a.h, d2a.l), 0.f});
  }
  float* o = f + kMlpIn * i;
  o[0] = static_cast<float>(uv[2 * i]) * 0.125f;
  o[1] = static_cast<float>(uv[2 * i + 1]) * 0.125f;
  o[2] = logf(fmaxf(sqrtf(n1), 0.05f));
  o[3] = logf(fmaxf(sqrtf(n2), 0.05f));
  o[4] = log10f(1e-6f + (dens.h + dens.l)) / 3.f;
}

void launch_mlp_features(const DevBasis& B, const double* pts, const double* uv, int64_t n, float* feats,
                         cudaStream_t st) {
  if (n <= 0) return;
  mlp_features_kernel<<<static_cast<unsigned>((n + 255) / 256), 256, 0, st>>>(B, pts, uv, n, feats);
}

void launch_mlp_train(const float* params, const float* x, const float* t, int n, float* grad, float* loss,
                      cudaStream_t st) {
  if (n <= 0) return;
  if (cudaFuncSetAttribute(mlp_train_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(kTrainSmemBytes)) != cudaSuccess)
    return;  // the launch error is left for cudaGetLastError
  mlp_train_kernel<<<(n + kTrainThreads - 1) / kTrainThreads, kTrainThreads, kTrainSmemBytes, st>>>(params, x, t, n,
                                                                                                 grad, loss);
}

void launch_mlp_adam(float* params, const float* grad, float* m, float* v, float lr, float b1, float b2, float eps, int step,
                     cudaStream_t st) {
  mlp_adam_kernel<<<(kMlpParams + 255) / 256, 256, 0, st>>>(params, grad, m, v, lr, b1, b2, eps, step);
}

void launch_mlp_infer(const float* params, const float* x, int n, float* y, cudaStream_t st) {
  if (n <= 0) return;
  mlp_infer_kernel<<<(n + 255) / 256, 256, 0, st>>>(params, x, n, y);
}

}  // namespace gg
