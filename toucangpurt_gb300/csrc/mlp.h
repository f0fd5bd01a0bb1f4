// Launch wrappers of the cost-model kernels (mlp.cu).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>

namespace tgs {

constexpr int kMlpParams = 64 * 16 + 64 + 64 * 64 + 64 + 64 + 1;  // 5,313

size_t mlpGradSmem();
// out[i] = network(X[i]) for n samples of 16 features (device pointers)
cudaError_t mlpForward(const float *params, const float *X, uint32_t n, float *out, cudaStream_t st);
// grad += d/dparams of scale * sum_i (network(X[idx[i]]) - y[idx[i]])^2 ; loss += the sum of squares
cudaError_t mlpGrad(const float *params, const float *X, const float *y, const uint32_t *idx, uint32_t n, float scale,
                    float *grad, float *loss, cudaStream_t st);
cudaError_t adamStep(float *params, float *m, float *v, const float *grad, uint32_t n, float lr, float b1, float b2,
                     float eps, uint32_t t, cudaStream_t st);

}  // namespace tgs
