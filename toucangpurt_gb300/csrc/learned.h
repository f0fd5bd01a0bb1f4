// Learned cost model of micro-partitions (see learned.cpp / mlp_kernels.cu).
#pragma once
#include <cstdint>
#include <vector>

#include "emit.h"

namespace tgs {

constexpr int kFeatures = 16;
void featureVector(const MPartFeat &f, float *out);

class CostModel {
 public:
  bool trained() const { return trained_; }
  // cost[part][level][i] for every micro-partition of the image
  void predictAll(const DeviceImage &img, std::vector<std::vector<std::vector<float>>> &cost) const;
  // host-side forward pass of the 16-64-64-1 network
  float predict(const float *x) const;
  void setWeights(const std::vector<float> &w);
  const std::vector<float> &weights() const { return w_; }

 private:
  bool trained_ = false;
  std::vector<float> w_;
};

}  // namespace tgs
