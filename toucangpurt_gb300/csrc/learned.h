// Learned cost model of micro-partitions: features, training and inference
// (kernels in mlp.cu).
#pragma once
#include <cstdint>
#include <vector>

#include "emit.h"
#include "mlp.h"

namespace tgs {

constexpr int kFeatures = 16;
void featureVector(const MPartFeat &f, float *out);

struct TrainResult {
  float trainMse = 0, valMse = 0, valCorr = 0, gateCorr = 0;
  uint32_t samples = 0, epochs = 0;
  double ms = 0;
};

class CostModel {
 public:
  bool trained() const { return trained_; }
  // cost[part][level][i] (predicted cycles) for every micro-partition of the image
  void predictAll(const DeviceImage &img, std::vector<std::vector<std::vector<float>>> &cost) const;
  // predicted cycles for n feature rows (GPU, current device)
  void predict(const float *X, uint32_t n, float *cycles) const;
  // trains on (features, measured cycles) with Adam on the GPU
  TrainResult train(const float *X, const float *cycles, uint32_t n, uint32_t epochs, uint32_t batch, float lr,
                    uint64_t seed, float valFrac);
  // parameters followed by the target scale (mean, std of log cycles)
  std::vector<float> state() const;
  void setState(const std::vector<float> &s);

 private:
  bool trained_ = false;
  std::vector<float> w_;
  float mu_ = 0, sigma_ = 1;
};

}  // namespace tgs
