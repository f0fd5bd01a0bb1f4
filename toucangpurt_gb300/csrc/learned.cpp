// Learned cost model: host side (features, inference for scheduling).
#include "learned.h"

#include <algorithm>
#include <cmath>

namespace tgs {

// 16 structural features of a micro-partition, log-scaled counts.
void featureVector(const MPartFeat &f, float *x) {
  auto l = [](double v) { return float(std::log1p(v)); };
  x[0] = f.kind == kMPLut;
  x[1] = f.kind == kMPVecRead;
  x[2] = f.kind == kMPVecOp;
  x[3] = f.kind == kMPMemRead;
  x[4] = l(f.lanes);
  x[5] = l(f.depth);
  x[6] = l(f.ops);
  x[7] = l(f.nops);
  x[8] = l(f.threeOp);
  x[9] = l(f.vpReads);
  x[10] = l(f.writes);
  x[11] = l(f.memPorts);
  x[12] = l(f.vecNibbles);
  x[13] = l(f.fanIn);
  x[14] = l(f.fanOut);
  x[15] = l(f.partLevels);
}

void CostModel::setWeights(const std::vector<float> &w) {
  w_ = w;
  trained_ = !w.empty();
}

// Layout of w_: W1[64][16], b1[64], W2[64][64], b2[64], W3[64], b3[1];
// prediction = exp(output) (the network regresses log cycles).
float CostModel::predict(const float *x) const {
  const float *W1 = w_.data(), *b1 = W1 + 64 * 16, *W2 = b1 + 64, *b2 = W2 + 64 * 64, *W3 = b2 + 64, *b3 = W3 + 64;
  float h1[64], h2[64];
  for (int j = 0; j < 64; ++j) {
    float s = b1[j];
    for (int i = 0; i < 16; ++i) s += W1[j * 16 + i] * x[i];
    h1[j] = s > 0 ? s : 0;
  }
  for (int j = 0; j < 64; ++j) {
    float s = b2[j];
    for (int i = 0; i < 64; ++i) s += W2[j * 64 + i] * h1[i];
    h2[j] = s > 0 ? s : 0;
  }
  float o = b3[0];
  for (int i = 0; i < 64; ++i) o += W3[i] * h2[i];
  return std::exp(std::min(o, 30.0f));
}

void CostModel::predictAll(const DeviceImage &img, std::vector<std::vector<std::vector<float>>> &cost) const {
  cost.resize(img.mp.size());
  for (size_t p = 0; p < img.mp.size(); ++p) {
    cost[p].resize(img.mp[p].size());
    for (size_t l = 0; l < img.mp[p].size(); ++l) {
      cost[p][l].resize(img.mp[p][l].size());
      for (size_t i = 0; i < img.mp[p][l].size(); ++i) {
        float x[kFeatures];
        featureVector(img.mp[p][l][i].feat, x);
        cost[p][l][i] = predict(x);
      }
    }
  }
}

}  // namespace tgs
