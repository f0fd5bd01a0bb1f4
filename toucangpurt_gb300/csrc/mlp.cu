// Learned cost model: a 16 -> 64 -> 64 -> 1 FP32 multilayer perceptron (ReLU)
// with hand-written forward, backward and Adam kernels.
//
// It predicts the cost (standardised log of clock64 cycles) of evaluating
// one micro-partition from 16 structural features; the scheduler balances
// warps and blocks on the prediction instead of on gate count.
//
// Parameter layout (floats): W1[64][16], b1[64], W2[64][64], b2[64], W3[64],
// b3[1] -- 5,313 values.  One warp evaluates one sample: lane l owns hidden
// units l and l + 32 of both layers; hidden activations move between lanes
// with shuffles.  Gradients accumulate per warp in shared memory (W2 rows
// padded to 65 floats so the 32 lanes' rows fall in distinct banks) and are
// summed into global memory once per block.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "mlp.h"

namespace tgs {
namespace {

constexpr uint32_t kFull = 0xFFFFFFFFu;
constexpr int kIn = 16, kH = 64;
constexpr int oW1 = 0, oB1 = oW1 + kH * kIn, oW2 = oB1 + kH, oB2 = oW2 + kH * kH, oW3 = oB2 + kH, oB3 = oW3 + kH;
static_assert(oB3 + 1 == kMlpParams, "layout");
constexpr int kWarps = 4;  // warps per block of the gradient kernel
// per-warp gradient accumulator with padded W2 rows
constexpr int gW1 = 0, gB1 = gW1 + kH * kIn, gW2 = gB1 + kH, gB2 = gW2 + kH * 65, gW3 = gB2 + kH, gB3 = gW3 + kH,
              kGradPad = gB3 + 1;

struct Act {
  float h1[2], h2[2], out;
};

// forward of one sample by one warp; w in shared memory
__device__ __forceinline__ Act forwardWarp(const float *__restrict__ w, const float *__restrict__ x, uint32_t lane) {
  Act a;
  float xv = lane < kIn ? x[lane] : 0.f;
#pragma unroll
  for (int u = 0; u < 2; ++u) {
    const int j = lane + 32 * u;
    float s = w[oB1 + j];
#pragma unroll
    for (int m = 0; m < kIn; ++m) s += w[oW1 + j * kIn + m] * __shfl_sync(kFull, xv, m);
    a.h1[u] = fmaxf(s, 0.f);
  }
  float s2[2] = {w[oB2 + lane], w[oB2 + lane + 32]};
#pragma unroll 8
  for (int k = 0; k < kH; ++k) {
    const float hk = __shfl_sync(kFull, a.h1[k >> 5], k & 31);
    s2[0] += w[oW2 + lane * kH + k] * hk;
    s2[1] += w[oW2 + (lane + 32) * kH + k] * hk;
  }
  a.h2[0] = fmaxf(s2[0], 0.f);
  a.h2[1] = fmaxf(s2[1], 0.f);
  float o = w[oW3 + lane] * a.h2[0] + w[oW3 + lane + 32] * a.h2[1];
  for (int off = 16; off > 0; off >>= 1) o += __shfl_xor_sync(kFull, o, off);
  a.out = o + w[oB3];
  return a;
}

__global__ void __launch_bounds__(128) mlpForwardKernel(const float *__restrict__ params, const float *__restrict__ X,
                                                        uint32_t n, float *__restrict__ out) {
  __shared__ float w[kMlpParams];
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) w[i] = params[i];
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  for (uint32_t s = blockIdx.x * (blockDim.x >> 5) + warp; s < n; s += gridDim.x * (blockDim.x >> 5)) {
    Act a = forwardWarp(w, X + size_t(s) * kIn, lane);
    if (lane == 0) out[s] = a.out;
  }
}

// Gradient of mean squared error over the samples idx[0..n) (idx null: 0..n).
__global__ void __launch_bounds__(32 * kWarps) mlpGradKernel(const float *__restrict__ params, const float *__restrict__ X,
                                                             const float *__restrict__ y, const uint32_t *__restrict__ idx,
                                                             uint32_t n, float scale, float *__restrict__ grad,
                                                             float *__restrict__ loss) {
  extern __shared__ float sm[];
  float *w = sm;
  float *gacc = sm + kMlpParams;  // [kWarps][kGradPad]
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) w[i] = params[i];
  for (int i = threadIdx.x; i < kWarps * kGradPad; i += blockDim.x) gacc[i] = 0.f;
  __syncthreads();
  const uint32_t lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  float *g = gacc + warp * kGradPad;
  float lossAcc = 0.f;
  for (uint32_t t = blockIdx.x * kWarps + warp; t < n; t += gridDim.x * kWarps) {
    const uint32_t s = idx ? idx[t] : t;
    const float *x = X + size_t(s) * kIn;
    const Act a = forwardWarp(w, x, lane);
    const float d = a.out - y[s];
    lossAcc += d * d;
    const float dy = 2.f * d * scale;
    // output layer
    float dh2[2];
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int j = lane + 32 * u;
      g[gW3 + j] += dy * a.h2[u];
      dh2[u] = a.h2[u] > 0.f ? dy * w[oW3 + j] : 0.f;
      g[gB2 + j] += dh2[u];
    }
    if (lane == 0) g[gB3] += dy;
    // second layer: dW2[j][k] = dh2[j] * h1[k]; dh1[k] = sum_j dh2[j] W2[j][k]
#pragma unroll 8
    for (int k = 0; k < kH; ++k) {
      const float hk = __shfl_sync(kFull, a.h1[k >> 5], k & 31);
      g[gW2 + lane * 65 + k] += dh2[0] * hk;
      g[gW2 + (lane + 32) * 65 + k] += dh2[1] * hk;
    }
    float dh1[2] = {0.f, 0.f};
#pragma unroll 8
    for (int j = 0; j < kH; ++j) {
      const float dj = __shfl_sync(kFull, dh2[j >> 5], j & 31);
      dh1[0] += dj * w[oW2 + j * kH + lane];
      dh1[1] += dj * w[oW2 + j * kH + lane + 32];
    }
    const float xv = lane < kIn ? x[lane] : 0.f;
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      const int k = lane + 32 * u;
      const float dk = a.h1[u] > 0.f ? dh1[u] : 0.f;
      g[gB1 + k] += dk;
#pragma unroll
      for (int m = 0; m < kIn; ++m) g[gW1 + k * kIn + m] += dk * __shfl_sync(kFull, xv, m);
    }
  }
  __syncthreads();
  // sum the warps' accumulators and add to the global gradient
  for (int i = threadIdx.x; i < kMlpParams; i += blockDim.x) {
    int src;
    if (i < oW2) src = i;                                   // W1, b1 share offsets
    else if (i < oB2) src = gW2 + ((i - oW2) / kH) * 65 + (i - oW2) % kH;
    else src = gB2 + (i - oB2);                             // b2, W3, b3 follow
    float s = 0.f;
    for (int wv = 0; wv < kWarps; ++wv) s += gacc[wv * kGradPad + src];
    atomicAdd(grad + i, s);
  }
  // every lane of a warp holds the same output, so lane 0's sum is the warp's
  if (lane == 0 && loss) atomicAdd(loss, lossAcc);
}

__global__ void adamKernel(float *__restrict__ p, float *__restrict__ m, float *__restrict__ v,
                           const float *__restrict__ g, uint32_t n, float lr, float b1, float b2, float eps,
                           float c1, float c2) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
  }
}

}  // namespace

size_t mlpGradSmem() { return (size_t(kMlpParams) + size_t(kWarps) * kGradPad) * sizeof(float); }

cudaError_t mlpForward(const float *params, const float *X, uint32_t n, float *out, cudaStream_t st) {
  if (!n) return cudaSuccess;
  const uint32_t blocks = std::min<uint32_t>(2048, (n + 3) / 4);
  mlpForwardKernel<<<blocks, 128, 0, st>>>(params, X, n, out);
  return cudaGetLastError();
}

cudaError_t mlpGrad(const float *params, const float *X, const float *y, const uint32_t *idx, uint32_t n, float scale,
                    float *grad, float *loss, cudaStream_t st) {
  if (!n) return cudaSuccess;
  // set on every call: the attribute belongs to the current device's context
  // (another device, or a context re-created after a reset, starts without it)
  cudaError_t e = cudaFuncSetAttribute(mlpGradKernel, cudaFuncAttributeMaxDynamicSharedMemorySize, int(mlpGradSmem()));
  if (e != cudaSuccess) return e;
  const uint32_t blocks = std::min<uint32_t>(304, (n + kWarps - 1) / kWarps);
  mlpGradKernel<<<blocks, 32 * kWarps, mlpGradSmem(), st>>>(params, X, y, idx, n, scale, grad, loss);
  return cudaGetLastError();
}

cudaError_t adamStep(float *params, float *m, float *v, const float *grad, uint32_t n, float lr, float b1, float b2,
                     float eps, uint32_t t, cudaStream_t st) {
  float c1 = 1.f, c2 = 1.f;
  for (uint32_t i = 0; i < t; ++i) {
    c1 *= b1;
    c2 *= b2;
  }
  adamKernel<<<(n + 255) / 256, 256, 0, st>>>(params, m, v, grad, n, lr, b1, b2, eps, 1.f - c1, 1.f - c2);
  return cudaGetLastError();
}

}  // namespace tgs
