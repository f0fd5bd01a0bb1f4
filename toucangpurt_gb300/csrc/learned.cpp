// Learned cost model: features, training loop and batch inference.
//
// Target: standardised log of the clock64 cycles one evaluation of a
// micro-partition takes (recorded by the cycle kernel's profiling mode).  The
// 16-64-64-1 network is trained with Adam by the hand-written kernels of
// mlp.cu; the scheduler then balances warps and blocks on exp(prediction).
#include "learned.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <string>

#include "tgs_internal.h"

namespace tgs {

namespace {

#define TGS_CK(call)                                                                                      \
  do {                                                                                                    \
    cudaError_t e_ = (call);                                                                              \
    if (e_ != cudaSuccess) throw Error(TGS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

template <typename T>
struct Dev {
  T *p = nullptr;
  explicit Dev(size_t n) { TGS_CK(cudaMalloc(&p, std::max<size_t>(1, n) * sizeof(T))); }
  ~Dev() {
    if (p) cudaFree(p);
  }
  Dev(const Dev &) = delete;
  Dev &operator=(const Dev &) = delete;
};

uint64_t splitmix(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
float uniform(uint64_t &s) { return float(splitmix(s) >> 40) * (1.0f / 16777216.0f); }

float corr(const std::vector<float> &a, const std::vector<float> &b) {
  const size_t n = a.size();
  if (n < 2) return 0;
  double ma = 0, mb = 0;
  for (size_t i = 0; i < n; ++i) ma += a[i], mb += b[i];
  ma /= n, mb /= n;
  double sab = 0, saa = 0, sbb = 0;
  for (size_t i = 0; i < n; ++i) {
    sab += (a[i] - ma) * (b[i] - mb);
    saa += (a[i] - ma) * (a[i] - ma);
    sbb += (b[i] - mb) * (b[i] - mb);
  }
  return saa > 0 && sbb > 0 ? float(sab / std::sqrt(saa * sbb)) : 0.f;
}

}  // namespace

// 16 structural features of a micro-partition, log-scaled counts.
void featureVector(const MPartFeat &f, float *x) {
  auto l = [](double v) { return float(std::log1p(v)); };
  x[0] = l(f.fastOps);  // LUT ops computed word-wide (kind LUT: x[1..3] all zero)
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

std::vector<float> CostModel::state() const {
  std::vector<float> s = w_;
  s.push_back(mu_);
  s.push_back(sigma_);
  return s;
}

void CostModel::setState(const std::vector<float> &s) {
  if (s.size() != size_t(kMlpParams) + 2) throw Error(TGS_ERR_ARG, "cost model state must hold 5,315 floats");
  w_.assign(s.begin(), s.begin() + kMlpParams);
  mu_ = s[kMlpParams];
  sigma_ = s[kMlpParams + 1];
  trained_ = true;
}

void CostModel::predict(const float *X, uint32_t n, float *cycles) const {
  if (!trained_) throw Error(TGS_ERR_STATE, "cost model not trained");
  Dev<float> dw(kMlpParams), dx(size_t(n) * kFeatures), dy(n);
  TGS_CK(cudaMemcpy(dw.p, w_.data(), kMlpParams * 4, cudaMemcpyHostToDevice));
  TGS_CK(cudaMemcpy(dx.p, X, size_t(n) * kFeatures * 4, cudaMemcpyHostToDevice));
  TGS_CK(mlpForward(dw.p, dx.p, n, dy.p, nullptr));
  TGS_CK(cudaMemcpy(cycles, dy.p, size_t(n) * 4, cudaMemcpyDeviceToHost));
  for (uint32_t i = 0; i < n; ++i) cycles[i] = std::exp(std::min(mu_ + sigma_ * cycles[i], 40.f));
}

void CostModel::predictAll(const DeviceImage &img, std::vector<std::vector<std::vector<float>>> &cost) const {
  std::vector<float> X;
  for (auto &p : img.mp)
    for (auto &l : p)
      for (auto &r : l) {
        float x[kFeatures];
        featureVector(r.feat, x);
        X.insert(X.end(), x, x + kFeatures);
      }
  const uint32_t n = uint32_t(X.size() / kFeatures);
  std::vector<float> y(n);
  if (n) predict(X.data(), n, y.data());
  size_t k = 0;
  cost.resize(img.mp.size());
  for (size_t p = 0; p < img.mp.size(); ++p) {
    cost[p].resize(img.mp[p].size());
    for (size_t l = 0; l < img.mp[p].size(); ++l) {
      cost[p][l].resize(img.mp[p][l].size());
      for (size_t i = 0; i < img.mp[p][l].size(); ++i) cost[p][l][i] = y[k++];
    }
  }
}

TrainResult CostModel::train(const float *X, const float *cyc, uint32_t n, uint32_t epochs, uint32_t batch, float lr,
                             uint64_t seed, float valFrac) {
  if (n < 8) throw Error(TGS_ERR_ARG, "need at least 8 training samples");
  auto t0 = std::chrono::steady_clock::now();
  TrainResult r;
  // split (seeded permutation) and standardised log targets
  std::vector<uint32_t> perm(n);
  std::iota(perm.begin(), perm.end(), 0u);
  uint64_t rs = seed ^ 0x7EA1ull;
  for (uint32_t i = n - 1; i > 0; --i) std::swap(perm[i], perm[uint32_t(splitmix(rs) % (i + 1))]);
  const uint32_t nVal = std::min<uint32_t>(n - 1, uint32_t(double(n) * std::max(0.f, std::min(valFrac, 0.5f))));
  const uint32_t nTr = n - nVal;
  std::vector<float> t(n);
  for (uint32_t i = 0; i < n; ++i) t[i] = std::log(std::max(1.0f, cyc[i]));
  double m = 0, v = 0;
  for (uint32_t i = 0; i < nTr; ++i) m += t[perm[i]];
  m /= nTr;
  for (uint32_t i = 0; i < nTr; ++i) v += (t[perm[i]] - m) * (t[perm[i]] - m);
  const float mu = float(m), sigma = float(std::max(1e-3, std::sqrt(v / nTr)));
  std::vector<float> y(n);
  for (uint32_t i = 0; i < n; ++i) y[i] = (t[i] - mu) / sigma;
  // He-uniform initialisation
  std::vector<float> w(kMlpParams, 0.f);
  uint64_t ws = seed;
  auto fill = [&](int off, int cnt, int fanIn) {
    const float a = std::sqrt(6.f / fanIn);
    for (int i = 0; i < cnt; ++i) w[off + i] = (2.f * uniform(ws) - 1.f) * a;
  };
  fill(0, 64 * 16, 16);
  fill(64 * 16 + 64, 64 * 64, 64);
  fill(64 * 16 + 64 + 64 * 64 + 64, 64, 64);
  Dev<float> dw(kMlpParams), dm(kMlpParams), dv(kMlpParams), dg(kMlpParams), dx(size_t(n) * kFeatures), dy(n), dl(1);
  Dev<uint32_t> di(n);
  TGS_CK(cudaMemcpy(dw.p, w.data(), kMlpParams * 4, cudaMemcpyHostToDevice));
  TGS_CK(cudaMemset(dm.p, 0, kMlpParams * 4));
  TGS_CK(cudaMemset(dv.p, 0, kMlpParams * 4));
  TGS_CK(cudaMemcpy(dx.p, X, size_t(n) * kFeatures * 4, cudaMemcpyHostToDevice));
  TGS_CK(cudaMemcpy(dy.p, y.data(), size_t(n) * 4, cudaMemcpyHostToDevice));
  batch = std::max<uint32_t>(32, std::min(batch, nTr));
  uint32_t step = 0;
  std::vector<uint32_t> order(perm.begin(), perm.begin() + nTr);
  for (uint32_t e = 0; e < epochs; ++e) {
    for (uint32_t i = nTr - 1; i > 0; --i) std::swap(order[i], order[uint32_t(splitmix(rs) % (i + 1))]);
    TGS_CK(cudaMemcpy(di.p, order.data(), size_t(nTr) * 4, cudaMemcpyHostToDevice));
    for (uint32_t b = 0; b < nTr; b += batch) {
      const uint32_t cnt = std::min(batch, nTr - b);
      TGS_CK(cudaMemsetAsync(dg.p, 0, kMlpParams * 4, nullptr));
      TGS_CK(mlpGrad(dw.p, dx.p, dy.p, di.p + b, cnt, 1.f / float(cnt), dg.p, nullptr, nullptr));
      TGS_CK(adamStep(dw.p, dm.p, dv.p, dg.p, kMlpParams, lr, 0.9f, 0.999f, 1e-8f, ++step, nullptr));
    }
  }
  TGS_CK(cudaDeviceSynchronize());
  TGS_CK(cudaMemcpy(w.data(), dw.p, kMlpParams * 4, cudaMemcpyDeviceToHost));
  // report: MSE (standardised log space) and correlations on the held-out set
  auto mse = [&](uint32_t lo, uint32_t hi) {
    if (hi <= lo) return 0.f;
    std::vector<uint32_t> ids(perm.begin() + lo, perm.begin() + hi);
    TGS_CK(cudaMemcpy(di.p, ids.data(), ids.size() * 4, cudaMemcpyHostToDevice));
    TGS_CK(cudaMemset(dl.p, 0, 4));
    TGS_CK(cudaMemset(dg.p, 0, kMlpParams * 4));
    TGS_CK(mlpGrad(dw.p, dx.p, dy.p, di.p, uint32_t(ids.size()), 1.f, dg.p, dl.p, nullptr));
    float l = 0;
    TGS_CK(cudaMemcpy(&l, dl.p, 4, cudaMemcpyDeviceToHost));
    return l / float(ids.size());
  };
  r.trainMse = mse(0, nTr);
  r.valMse = mse(nTr, n);
  w_ = w;
  mu_ = mu;
  sigma_ = sigma;
  trained_ = true;
  if (nVal >= 2) {
    std::vector<float> xv, pred(nVal), truth(nVal), gate(nVal);
    for (uint32_t i = 0; i < nVal; ++i) {
      const uint32_t k = perm[nTr + i];
      xv.insert(xv.end(), X + size_t(k) * kFeatures, X + size_t(k + 1) * kFeatures);
      truth[i] = t[k];
      gate[i] = std::log(std::max(1.0f, std::expm1(X[size_t(k) * kFeatures + 6])));  // log op count
    }
    predict(xv.data(), nVal, pred.data());
    for (auto &p : pred) p = std::log(std::max(1e-6f, p));
    r.valCorr = corr(pred, truth);
    r.gateCorr = corr(gate, truth);
  }
  r.samples = n;
  r.epochs = epochs;
  r.ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return r;
}

}  // namespace tgs
