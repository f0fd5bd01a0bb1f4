// Seeded synthetic designs in the reference's design-file format.
//
// The reference ships neither designs nor the LLVM-based compiler that writes
// them (include/ToucanGPUGenDataTypes.h:285-286 only hints at it), so this
// file produces legal SimDesignInfo / SimDebugInfo pairs directly, with the
// structure the reference runtime requires:
//   * exactly two regions per cycle (src/SimEval.cu:1292-1310): region-0
//     partitions read registers (L0 RegRead) and end in one exchange block
//     copy; region-1 partitions read the exchange pool (L0 ExgRead) and end in
//     one register block copy plus memory writes (SimEval.cu:1183: a partition
//     reads either registers or exchange, never both);
//   * micro-partitions of <= 32 lanes per level and <= 158 middle levels
//     (SimEval.cu:92-97), operands < 16 immediate at the top level and lanes
//     32..63 in middle levels (SimEval.cu:345-347, 388-404);
//   * every value-pool slot written before it is read in the same partition,
//     and no two micro-partitions of one exec level touching a slot the other
//     writes, so results do not depend on the schedule;
//   * block copies word aligned (SimEval.cu:658-665): partition outputs are
//     4-nibble aligned and a multiple of 4 nibbles long;
//   * memory reads in region 0 and writes in region 1 (reads see the previous
//     cycle's contents), write ports of one memory on disjoint addresses.
//
// Truth tables are windows into the design-global 4,642-byte table
// (SimEval.cu:33,190): a few fixed palette windows (AND/OR/XOR/EQ/ULT/MUX/ADD/
// SUB and single-operand "force low bits" windows for port addresses) inside
// seeded random nibbles; a generic 2-operand LUT is a random 256-entry window,
// a generic 3-operand LUT a random 4,096-entry window.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <fstream>
#include <functional>
#include <numeric>
#include <string>
#include <vector>

#include "tgs_internal.h"

namespace tgs {
namespace {

using namespace toucanGPUSim;

// palette window bases (256 entries indexed by (b << 4) | c with a = 0).  MUX
// is at base 1 so that even a select operand read from a slot (any nibble)
// keeps the full 4,096-entry window inside the table; its rows a = 0 and
// a = 1 hold the mux function.
constexpr uint16_t kMux = 1, kAdd = 520, kSub = 776, kAnd = 1032, kOr = 1288, kXor = 1544, kEq = 1800, kUlt = 2056;
constexpr uint16_t kForceBase = 2600;  // 16-entry windows: (c & ~(P-1)) | p

// Records are written to the file as raw bytes, padding included.  A copy
// of a struct may skip its padding, so every padded record is zeroed in
// place inside its vector before its fields are set: files are reproducible.
template <typename T>
T &addZeroed(std::vector<T> &v) {
  v.emplace_back();
  T &t = v.back();
  std::memset(static_cast<void *>(&t), 0, sizeof(T));
  return t;
}
void addRegRead(std::vector<CGRegReadMetaInfo> &v, uint32_t reg, uint16_t slot) {
  auto &r = addZeroed(v);
  r.reg = reg;
  r.result = slot;
}
void addExgRead(std::vector<CGExchangeReadMetaInfo> &v, uint32_t e, uint16_t slot) {
  auto &r = addZeroed(v);
  r.exchange = e;
  r.result = slot;
}
void addWriteBack(std::vector<CGMicroPartLUTLastLevelWriteBack> &v, uint8_t src, uint16_t slot) {
  auto &r = addZeroed(v);
  r.shuffleId = src;
  r.result = slot;
}

struct Rng {
  uint64_t s;
  explicit Rng(uint64_t seed) : s(mix64(seed ^ 0x5EEDull)) {}
  uint64_t next() { return mix64(s += 0x9E3779B97F4A7C15ull); }
  uint32_t below(uint32_t n) { return n ? uint32_t((next() >> 32) * n >> 32) : 0; }
};

uint16_t forceWindow(uint32_t ports, uint32_t p) {
  // ports 2 -> windows 0,1 ; ports 4 -> windows 2..5
  uint32_t idx = ports == 2 ? p : 2 + p;
  return uint16_t(kForceBase + 16 * idx);
}

std::vector<uint8_t> buildLut(Rng &rng) {
  std::vector<uint8_t> lut(kLutSize);
  for (auto &v : lut) v = uint8_t(rng.next() & 0xF);
  for (uint32_t b = 0; b < 16; ++b)
    for (uint32_t c = 0; c < 16; ++c) {
      uint32_t i = (b << 4) | c;
      lut[kAdd + i] = uint8_t((b + c) & 0xF);
      lut[kSub + i] = uint8_t((b - c) & 0xF);
      lut[kAnd + i] = uint8_t(b & c);
      lut[kOr + i] = uint8_t(b | c);
      lut[kXor + i] = uint8_t(b ^ c);
      lut[kEq + i] = uint8_t(b == c);
      lut[kUlt + i] = uint8_t(b < c);
      lut[kMux + i] = uint8_t(c);          // select 0 -> c
      lut[kMux + 256 + i] = uint8_t(b);    // select 1 -> b
    }
  const uint32_t portsList[6][2] = {{2, 0}, {2, 1}, {4, 0}, {4, 1}, {4, 2}, {4, 3}};
  for (auto &pp : portsList)
    for (uint32_t c = 0; c < 16; ++c) lut[forceWindow(pp[0], pp[1]) + c] = uint8_t((c & ~(pp[0] - 1) & 0xF) | pp[1]);
  return lut;
}

// Register / exchange layout shared by the generator and tgs_gen_inputs.
struct Layout {
  uint32_t nParts = 1;                   // partitions per region
  std::vector<uint32_t> ffStart, ffCount;  // per region-1 partition, 4-aligned blocks
  uint32_t ffTotal = 0, piStart = 0, piCount = 0, resetCount = 0, regPool = 0;
};

Layout makeLayout(const tgs_gen_config &c) {
  Layout L;
  uint64_t perRegion = std::max<uint64_t>(1, c.n_lut / 2);
  uint32_t lpp = std::max<uint32_t>(32, c.luts_per_part);
  L.nParts = uint32_t(std::max<uint64_t>(1, (perRegion + lpp - 1) / lpp));
  uint32_t ffNib = (c.ff_bits + 3) / 4;
  uint32_t per = (ffNib + L.nParts - 1) / L.nParts;
  per = std::max<uint32_t>(4, (per + 3) & ~3u);
  uint32_t at = 0;
  for (uint32_t k = 0; k < L.nParts; ++k) {
    L.ffStart.push_back(at);
    L.ffCount.push_back(per);
    at += per;
  }
  L.ffTotal = at;
  L.piStart = at;
  L.piCount = (c.pi_bits + 3) / 4;
  L.resetCount = c.reset_inputs;
  L.regPool = (L.piStart + L.piCount + L.resetCount + 3) & ~3u;
  return L;
}

struct Val {
  uint16_t slot;
  bool bit;  // value known to be 0/1 (select operand for MUX)
};

struct Band {
  std::vector<Val> vals;
  std::vector<uint64_t> cum;  // prefix sums of popularity weights
};

struct PartKind {
  uint32_t width = 32, depth = 1, operands = 2, palettePct = 0;
  double alpha = 0;
  uint32_t maxFan = 4096;
};

struct Counts {
  uint64_t lut = 0, nop = 0, mparts = 0, memR = 0, memW = 0, vec = 0, l0 = 0;
};

class PartGen {
 public:
  PartGen(Rng &rng, SimPartitionInfo &P, Counts &cnt, const PartKind &k) : rng_(rng), P_(P), cnt_(cnt), k_(k) {}

  // Inputs: L0 reads into consecutive slots starting at 16.
  uint16_t addInput(uint32_t src, bool exchange) {
    uint16_t s = slot(1);
    if (exchange)
      addExgRead(P_.ops_l0_exchangeRead, src, s);
    else
      addRegRead(P_.ops_l0_regRead, src, s);
    ++cnt_.l0;
    inputs_.vals.push_back({s, false});
    return s;
  }
  void finishInputs() { weigh(inputs_); }

  uint16_t slot(uint32_t n, uint32_t align = 1) {
    next_ = (next_ + align - 1) / align * align;
    uint32_t s = next_;
    next_ += n;
    if (next_ > 65000) throw DesignError("generator: value pool over 65,000 slots; lower luts_per_part");
    return uint16_t(s);
  }

  // Builds `bands` levels of micro-partitions with `width` values each.
  // Final band writes into [outBase, outBase + nOut).
  void build(uint32_t levels, uint32_t width, uint32_t nOut, uint16_t outBase, uint32_t memReadBand,
             const std::function<void(uint32_t band)> &afterBand) {
    uint32_t d = std::max<uint32_t>(1, std::min(k_.depth, levels));
    uint32_t bands = (levels + d - 1) / d;
    uint32_t w = std::max<uint32_t>(1, std::min<uint32_t>(32, k_.width));
    width = std::max(width, 1u);
    const uint32_t R = 3;
    uint32_t ringBlock = ((std::max(width, nOut) + 3) & ~3u);
    std::vector<uint16_t> ring(R + 2);
    for (auto &r : ring) r = slot(ringBlock, 4);
    (void)memReadBand;
    for (uint32_t b = 0; b < bands; ++b) {
      bool last = b + 1 == bands;
      uint32_t levelsHere = std::min(d, levels - b * d);
      uint32_t nVals = last ? std::max(width, nOut) : width;
      Band band;
      std::vector<CGMicroPartInfo> mparts;
      uint32_t made = 0;
      while (made < nVals) {
        uint32_t lanes = std::min(w, nVals - made);
        CGMicroPartInfo m;
        m.isLUTPart = true;
        bool bit[32];
        for (uint32_t l = 0; l < lanes; ++l) m.topLevel.push_back(topOp(b, bit[l]));
        for (uint32_t lv = 1; lv < levelsHere; ++lv) {
          std::vector<CGMicroPartLUTMiddleLevelOp> ops;
          for (uint32_t l = 0; l < lanes; ++l) ops.push_back(midOp(lanes, bit[l]));
          m.middleLevels.push_back(std::move(ops));
        }
        for (uint32_t l = 0; l < lanes; ++l) {
          uint32_t idx = made + l;
          uint16_t dst = (last && idx < nOut) ? uint16_t(outBase + idx) : uint16_t(ring[b % (R + 2)] + (idx % ringBlock));
          addWriteBack(m.lastLevel, uint8_t(32 + l), dst);
          band.vals.push_back({dst, bit[l]});
        }
        made += lanes;
        mparts.push_back(std::move(m));
        ++cnt_.mparts;
      }
      P_.exec_mParts.push_back(std::move(mparts));
      weigh(band);
      bands_.push_back(std::move(band));
      if (afterBand) afterBand(b);
    }
  }

  // Extra exec level with one micro-partition producing 8 contiguous address
  // nibbles: masked values of the latest band, constant zero above.
  uint16_t addressGen(uint32_t addrBits, uint32_t ports, uint32_t port, std::vector<CGMicroPartInfo> &level) {
    uint16_t base = slot(8, 4);
    CGMicroPartInfo m;
    m.isLUTPart = true;
    for (uint32_t j = 0; j < 8; ++j) {
      uint32_t bits = addrBits > 4 * j ? std::min<uint32_t>(4, addrBits - 4 * j) : 0;
      CGMicroPartLUTTopLevelOp op{0, 0, 0, 0};
      if (bits == 0) {
        op = {0, 0, 0, 0};  // move of immediate 0
        ++cnt_.nop;
      } else {
        uint16_t src = pick(uint32_t(bands_.size()), false).slot;
        if (j == 0 && ports > 1) {
          op = {forceWindow(ports, port), 0, 0, src};
          ++cnt_.lut;
        } else if (bits < 4) {
          op = {kAnd, 0, src, uint16_t((1u << bits) - 1)};
          ++cnt_.lut;
        } else {
          op = {0, 0, 0, src};
          ++cnt_.nop;
        }
      }
      m.topLevel.push_back(op);
      addWriteBack(m.lastLevel, uint8_t(32 + j), uint16_t(base + j));
    }
    level.push_back(std::move(m));
    ++cnt_.mparts;
    return base;
  }

  // Value of the latest band (or inputs) for memory-write data etc.
  uint16_t anyRecent() { return pick(uint32_t(bands_.size()), false).slot; }

  // Extra exec level with one micro-partition: a recent value compared with
  // a constant nibble (EQ window), nonzero in about one cycle in 16.
  uint16_t rareFlag(std::vector<CGMicroPartInfo> &level) {
    const uint16_t out = slot(1);
    CGMicroPartInfo m;
    m.isLUTPart = true;
    m.topLevel.push_back({kEq, 0, anyRecent(), uint16_t(1 + rng_.below(15))});
    ++cnt_.lut;
    addWriteBack(m.lastLevel, uint8_t(32), out);
    level.push_back(std::move(m));
    ++cnt_.mparts;
    return out;
  }

  void addBandValues(const std::vector<uint16_t> &slots) {
    if (bands_.empty()) {
      for (auto s : slots) inputs_.vals.push_back({s, false});
      weigh(inputs_);
    } else {
      for (auto s : slots) bands_.back().vals.push_back({s, false});
      weigh(bands_.back());
    }
  }

  uint32_t valuePoolSize() const { return (next_ + 15) & ~15u; }
  Counts &counts() { return cnt_; }

 private:
  // Popularity weights follow a discrete power law: weight 2^k with
  // P(k) proportional to 2^(-k (alpha - 1)), k = 0 .. log2(maxFan), so that
  // P(weight >= x) ~ x^-(alpha - 1).  Only integers after one rounding of the
  // exponent to 1/64: integer arithmetic only, so designs are identical on every
  // host (x86-64 and aarch64 libm / FMA contraction would otherwise differ).
  void weigh(Band &b) {
    b.cum.resize(b.vals.size());
    uint64_t acc = 0;
    for (size_t i = 0; i < b.vals.size(); ++i) {
      acc += k_.alpha > 1.0 ? (uint64_t(1) << weightClass()) : 1u;
      b.cum[i] = acc;
    }
  }

  uint32_t weightClass() {
    if (classThr_.empty()) {
      uint32_t kmax = 0;
      while ((2u << kmax) <= std::max<uint32_t>(1, k_.maxFan)) ++kmax;
      // ratio = 2^-(alpha - 1) in Q32 as (2^-1/64)^steps, alpha - 1 rounded to 1/64
      constexpr uint64_t kTwoPowMinusSixtyFourth = 4248701965ull;  // 2^(-1/64) in Q32
      const int64_t steps = std::max<int64_t>(0, (int64_t)((k_.alpha - 1.0) * 64.0 + 0.5));
      uint64_t ratio = uint64_t(1) << 32;
      for (int64_t i = 0; i < steps; ++i) ratio = (ratio * kTwoPowMinusSixtyFourth) >> 32;
      std::vector<uint64_t> p(kmax + 1);
      p[0] = uint64_t(1) << 32;
      for (uint32_t k = 1; k <= kmax; ++k) p[k] = (p[k - 1] * ratio) >> 32;
      uint64_t total = 0;
      for (auto v : p) total += v;
      uint64_t run = 0;
      for (uint32_t k = 0; k <= kmax; ++k) {
        run += p[k];
        classThr_.push_back(uint64_t((unsigned __int128)run * 0xFFFFFFFFull / total));
      }
      classThr_.back() = 0xFFFFFFFFull;
    }
    const uint64_t u = rng_.next() >> 32;
    uint32_t k = 0;
    while (k + 1 < classThr_.size() && u > classThr_[k]) ++k;
    return k;
  }

  // Operand for band b: uniformly one of the previous 1-3 bands (inputs
  // before band 0), then a value by popularity weight.
  Val pick(uint32_t b, bool wantBit) {
    const Band *src = &inputs_;
    uint32_t back = 1 + rng_.below(3);
    if (b >= back) src = &bands_[b - back];
    if (src->vals.empty()) src = bands_.empty() ? &inputs_ : &bands_.back();
    if (src->vals.empty()) throw DesignError("generator: partition without inputs");
    if (wantBit) {
      for (int t = 0; t < 8; ++t) {
        const Val &v = src->vals[rng_.below(uint32_t(src->vals.size()))];
        if (v.bit) return v;
      }
    }
    const uint64_t r = 1 + uint64_t((unsigned __int128)(rng_.next()) * src->cum.back() >> 64);
    size_t i = std::lower_bound(src->cum.begin(), src->cum.end(), r) - src->cum.begin();
    return src->vals[std::min(i, src->vals.size() - 1)];
  }

  // Choice of function: palette (AND/OR/XOR/MUX) with palettePct, a few
  // comparators (bit-valued, feed MUX selects), else a random window.
  void chooseFn(uint16_t &lut, bool &threeOp, bool &isMux, bool &bitOut) {
    threeOp = k_.operands >= 3;
    isMux = false;
    bitOut = false;
    uint32_t r = rng_.below(100);
    if (r < k_.palettePct) {
      switch (rng_.below(4)) {
        case 0: lut = kAnd; break;
        case 1: lut = kOr; break;
        case 2: lut = kXor; break;
        default: lut = kMux; isMux = true; break;
      }
      threeOp = isMux;
      return;
    }
    if (k_.palettePct && r < k_.palettePct + 5) {
      lut = rng_.below(2) ? kEq : kUlt;
      threeOp = false;
      bitOut = true;
      return;
    }
    lut = threeOp ? uint16_t(1 + rng_.below(kLutSize - 4096)) : uint16_t(1 + rng_.below(kLutSize - 256));
  }

  CGMicroPartLUTTopLevelOp topOp(uint32_t b, bool &bitOut) {
    uint16_t lut;
    bool three, mux;
    chooseFn(lut, three, mux, bitOut);
    CGMicroPartLUTTopLevelOp op;
    op.lutIndex = lut;
    op.op0 = 0;
    if (mux) {
      Val sel = pick(b, true);
      op.op0 = sel.bit ? sel.slot : uint16_t(rng_.below(2));  // immediate select when no 0/1 value is at hand
    } else if (three) {
      op.op0 = pick(b, false).slot;
    }
    op.op1 = pick(b, false).slot;
    op.op2 = pick(b, false).slot;
    ++cnt_.lut;
    return op;
  }

  CGMicroPartLUTMiddleLevelOp midOp(uint32_t lanes, bool &bitOut) {
    uint16_t lut;
    bool three, mux;
    chooseFn(lut, three, mux, bitOut);
    auto lane = [&]() { return uint8_t(32 + rng_.below(lanes)); };
    uint8_t a = 0;
    if (mux)
      a = uint8_t(rng_.below(2));  // lanes are not tracked as 0/1 values: immediate select
    else if (three)
      a = lane();
    ++cnt_.lut;
    // draws in a fixed order (argument evaluation order is unspecified)
    const uint8_t b = lane();
    const uint8_t c = lane();
    return CGMicroPartLUTMiddleLevelOp(lut, a, b, c);
  }

  Rng &rng_;
  SimPartitionInfo &P_;
  Counts &cnt_;
  PartKind k_;
  uint32_t next_ = 16;
  Band inputs_;
  std::vector<Band> bands_;
  std::vector<uint64_t> classThr_;
};

struct MemPlan {
  uint32_t nibbles, addrBits;
  std::vector<uint64_t> nibBase;  // memBase per nibble memory
  bool multi;
};

}  // namespace

void generateDesign(const tgs_gen_config &c, SimDesignInfo &d, SimDebugInfo &s, tgs_gen_info *info) {
  if (c.levels < 2) throw Error(TGS_ERR_ARG, "levels must be >= 2");
  Rng rng(c.seed);
  Layout L = makeLayout(c);
  d = SimDesignInfo();
  s = SimDebugInfo();
  d.lut = buildLut(rng);
  d.shouldStop = false;
  d.regPoolSize = L.regPool;
  Counts cnt;

  // ---- memories ---------------------------------------------------------
  std::vector<MemPlan> mems;
  uint64_t memAt = 0;
  for (uint32_t m = 0; m < c.n_mems; ++m) {
    MemPlan mp;
    mp.nibbles = (std::max(1u, c.mem_width) + 3) / 4;
    mp.addrBits = 0;
    while ((1ull << mp.addrBits) < std::max(1u, c.mem_depth)) ++mp.addrBits;
    mp.multi = c.mem_multi_writer != 0;
    std::vector<std::tuple<uint32_t, uint32_t, uint32_t>> sym;
    if (mp.multi) {
      for (uint32_t j = 0; j < mp.nibbles; ++j) mp.nibBase.push_back(memAt + (j / 4) * 4ull * c.mem_depth + (j % 4));
      for (uint32_t q = 0; q < (mp.nibbles + 3) / 4; ++q)
        sym.emplace_back(uint32_t(memAt + q * 4ull * c.mem_depth), 4u, 4u * c.mem_depth);
      memAt += ((mp.nibbles + 3) / 4) * 4ull * c.mem_depth;
    } else {
      for (uint32_t j = 0; j < mp.nibbles; ++j) {
        mp.nibBase.push_back(memAt);
        sym.emplace_back(uint32_t(memAt), 4u, c.mem_depth);
        memAt += c.mem_depth;
      }
    }
    if (memAt > 0xFFFFFFF0ull) throw Error(TGS_ERR_RANGE, "memories exceed 4 GiB nibble pool");
    s.memDebugInfo["mem_" + std::to_string(m)] = std::move(sym);
    mems.push_back(std::move(mp));
  }
  d.memPoolSize = uint32_t((memAt + 3) & ~3ull);

  // ---- registers ---------------------------------------------------------
  for (uint32_t k = 0, id = 0; id < L.ffTotal; ++k) {
    std::vector<std::tuple<uint32_t, uint32_t>> nib;
    for (uint32_t j = 0; j < 8 && id < L.ffTotal; ++j, ++id) nib.emplace_back(id, 4u);
    std::reverse(nib.begin(), nib.end());  // most significant nibble first
    s.regDebugInfo["ff_" + std::to_string(k)] = std::move(nib);
  }
  for (uint32_t k = 0, i = 0; i < L.piCount; ++k) {
    std::vector<std::tuple<uint32_t, uint32_t>> nib;
    for (uint32_t j = 0; j < 8 && i < L.piCount; ++j, ++i) {
      uint32_t bits = (i + 1 == L.piCount && c.pi_bits % 4) ? c.pi_bits % 4 : 4;
      nib.emplace_back(L.piStart + i, bits);
    }
    std::reverse(nib.begin(), nib.end());
    s.regDebugInfo["pi_" + std::to_string(k)] = std::move(nib);
  }
  for (uint32_t r = 0; r < L.resetCount; ++r)
    s.regDebugInfo["rst_" + std::to_string(r)] = {std::make_tuple(L.piStart + L.piCount + r, 1u)};

  // ---- partitions ------------------------------------------------------
  const uint32_t P = L.nParts;
  const uint32_t lv0 = c.levels / 2, lv1 = c.levels - lv0;
  const uint64_t perPart = std::max<uint64_t>(1, c.n_lut / 2 / P);
  std::vector<uint32_t> exStart(P), exCount(P);
  d.parts.resize(2 * P);

  auto kindFor = [&](uint32_t k) {
    PartKind pk;
    pk.width = c.mpart_width ? c.mpart_width : 32;
    pk.depth = c.cone_depth ? c.cone_depth : 1;
    pk.operands = c.operands;
    pk.palettePct = c.palette_pct;
    pk.alpha = c.fanout_alpha;
    pk.maxFan = c.max_fanout ? c.max_fanout : 4096;
    if (c.mixed) {
      uint32_t r = uint32_t(mix64(c.seed ^ (0xABCull + k)) % 100);
      if (r < 40) {         // wide datapath cones, depth 8-12, 3 operands
        pk.width = 32; pk.depth = 8 + uint32_t(mix64(k * 7 + 1) % 5); pk.operands = 3;
      } else if (r < 70) {  // deep narrow control cones, depth 32-64
        pk.width = 4 + 4 * uint32_t(mix64(k * 7 + 2) % 2); pk.depth = 32 + uint32_t(mix64(k * 7 + 3) % 33);
      } else if (r < 90) {  // memory-heavy: shallow logic
        pk.width = 32; pk.depth = 1;
      } else {              // high fan-out nets
        pk.width = 32; pk.depth = 2; pk.alpha = 1.6; pk.maxFan = 65536;
      }
    }
    return pk;
  };
  auto memHeavy = [&](uint32_t k) { return c.mixed && (mix64(c.seed ^ (0xABCull + k)) % 100) >= 70 && (mix64(c.seed ^ (0xABCull + k)) % 100) < 90; };

  // Memory ports to partitions: reads to region 0, writes to region 1.
  std::vector<std::vector<std::pair<uint32_t, uint32_t>>> readsOf(P), writesOf(P);
  {
    std::vector<uint32_t> heavy;
    for (uint32_t k = 0; k < P; ++k)
      if (memHeavy(k)) heavy.push_back(k);
    for (uint32_t m = 0; m < c.n_mems; ++m) {
      uint32_t nr = c.mem_read_ports, nw = c.mem_write_ports;
      if (c.mixed) { nr = 1 + uint32_t(mix64(m * 3 + 11) % 4); nw = 1; }
      for (uint32_t r = 0; r < nr; ++r) {
        uint32_t k = heavy.empty() ? rng.below(P) : heavy[rng.below(uint32_t(heavy.size()))];
        readsOf[k].push_back({m, r});
      }
      for (uint32_t w = 0; w < nw; ++w) writesOf[rng.below(P)].push_back({m, w});
    }
  }
  const uint32_t writePorts = c.mixed ? 1 : std::max(1u, c.mem_write_ports);
  if (writePorts != 1 && writePorts != 2 && writePorts != 4) throw Error(TGS_ERR_ARG, "mem_write_ports must be 1, 2 or 4");

  // Vector ops to region-0 partitions.
  std::vector<uint32_t> vecOf(P, 0);
  for (uint32_t v = 0; v < c.n_vec_ops; ++v) vecOf[rng.below(P)]++;
  const uint32_t vn = std::max(1u, std::min(31u, c.vec_nibbles ? c.vec_nibbles : 8));

  // ---- region 0 -----------------------------------------------------------
  uint32_t exAt = 0;
  for (uint32_t k = 0; k < P; ++k) {
    SimPartitionInfo &part = d.parts[k];
    PartKind pk = kindFor(k);
    PartGen g(rng, part, cnt, pk);
    uint32_t width = uint32_t(std::max<uint64_t>(1, perPart / lv0));
    // vector-op operands: contiguous register groups read into contiguous slots
    std::vector<std::pair<uint16_t, uint16_t>> vecGroups;  // (slotA, slotB)
    std::vector<uint32_t> readRegs;
    uint32_t nVec = vecOf[k];
    for (uint32_t v = 0; v < nVec; ++v) {
      uint16_t sa = 0, sb = 0;
      for (int opd = 0; opd < 2; ++opd) {
        uint32_t grp = L.ffTotal >= vn ? rng.below(L.ffTotal - vn + 1) : 0;
        uint16_t first = 0;
        for (uint32_t j = 0; j < vn; ++j) {
          uint16_t sl = g.addInput(std::min(grp + j, L.regPool - 1), false);
          if (j == 0) first = sl;
        }
        (opd ? sb : sa) = first;
      }
      vecGroups.push_back({sa, sb});
    }
    // scalar inputs: own feedback block, then random registers and inputs
    uint32_t nIn = std::max<uint32_t>(8, std::min<uint32_t>(width + 8, 4096));
    for (uint32_t j = 0; j < L.ffCount[k] && readRegs.size() < nIn; ++j) readRegs.push_back(L.ffStart[k] + j);
    for (uint32_t j = 0; j < L.piCount + L.resetCount; ++j)
      if (P == 1 || rng.below(P) < 2) readRegs.push_back(L.piStart + j);
    while (readRegs.size() < nIn) readRegs.push_back(rng.below(L.ffTotal));
    for (uint32_t r : readRegs) g.addInput(r, false);
    g.finishInputs();

    uint32_t nOut = std::max<uint32_t>(4, (std::min<uint32_t>(width, 4096) + 3) & ~3u);
    uint16_t outBase = g.slot(nOut, 4);

    // vector ops as exec level 0 (read inputs only)
    std::vector<uint16_t> vecResults;
    if (!vecGroups.empty()) {
      std::vector<CGMicroPartInfo> lvl;
      for (size_t v0 = 0; v0 < vecGroups.size(); v0 += 32) {
        CGMicroPartInfo m;
        m.isLUTPart = false;
        for (size_t v = v0; v < std::min(vecGroups.size(), v0 + 32); ++v) {
          auto &op = addZeroed(m.vecArithAndLogic);
          op.vec1Base = vecGroups[v].first;
          op.vec2Base = vecGroups[v].second;
          op.vecLength = uint16_t(vn);
          uint32_t r = rng.below(8);
          op.opName = uint8_t(r < 3 ? VEC_ARITH_ADD : r < 4 ? VEC_ARITH_SUB : r < 5 ? VEC_ARITH_MUL : r < 6 ? VEC_LOGIC_EQ : r < 7 ? VEC_LOGIC_LT : VEC_LOGIC_LE);
          op.isV1V2Const = 0;
          bool isVec = op.opName <= VEC_ARITH_MUL;
          op.result = g.slot(isVec ? vn : 1);
          if (isVec)
            for (uint32_t j = 0; j < vn; ++j) vecResults.push_back(uint16_t(op.result + j));
          else
            vecResults.push_back(op.result);
          ++cnt.vec;
        }
        lvl.push_back(std::move(m));
        ++cnt.mparts;
      }
      part.exec_mParts.push_back(std::move(lvl));
      g.addBandValues(vecResults);
    }

    // memory-read ports: address generation after a random band, then reads
    std::vector<uint32_t> readBand(readsOf[k].size());
    uint32_t bandsR0 = (lv0 + std::max(1u, std::min(pk.depth, lv0)) - 1) / std::max(1u, std::min(pk.depth, lv0));
    for (auto &rb : readBand) rb = bandsR0 > 1 ? rng.below(bandsR0 - 1) : 0;
    bool vecReadDone = nVec == 0;
    g.build(lv0, width, nOut, outBase, 0, [&](uint32_t b) {
      std::vector<CGMicroPartInfo> addrLvl, readLvl, vrLvl;
      std::vector<uint16_t> produced;
      for (size_t i = 0; i < readsOf[k].size(); ++i) {
        if (readBand[i] != b) continue;
        const MemPlan &mp = mems[readsOf[k][i].first];
        uint16_t addr = g.addressGen(mp.addrBits, 1, 0, addrLvl);
        for (uint32_t j0 = 0; j0 < mp.nibbles; j0 += 32) {
          CGMicroPartInfo m;
          m.isLUTPart = false;
          for (uint32_t j = j0; j < std::min(mp.nibbles, j0 + 32); ++j) {
            auto &op = addZeroed(m.memRead);
            op.hasMultipleWriter = mp.multi;
            op.memBase = mp.nibBase[j];
            op.en = 1;
            op.addrVec = addr;
            op.result = g.slot(1);
            produced.push_back(op.result);
            ++cnt.memR;
          }
          readLvl.push_back(std::move(m));
          ++cnt.mparts;
        }
      }
      // shifts lowered to dynamic vector reads (one per vector op)
      if (!vecReadDone && b == 0 && !vecGroups.empty()) {
        CGMicroPartInfo m;
        m.isLUTPart = false;
        for (size_t v = 0; v < vecGroups.size() && v < 32; ++v) {
          auto &op = addZeroed(m.vecRead);
          op.vecBase = vecGroups[v].first;
          op.vecLength = uint16_t(vn);
          op.offset = uint16_t(rng.below(4));
          op.isConstVec = false;
          op.index0 = op.index1 = op.index2 = 0;
          op.index3 = g.anyRecent();
          op.outRangeValue = 0;
          op.result = g.slot(1);
          produced.push_back(op.result);
        }
        vrLvl.push_back(std::move(m));
        ++cnt.mparts;
        vecReadDone = true;
      }
      if (!addrLvl.empty()) part.exec_mParts.push_back(std::move(addrLvl));
      if (!readLvl.empty()) part.exec_mParts.push_back(std::move(readLvl));
      if (!vrLvl.empty()) part.exec_mParts.push_back(std::move(vrLvl));
      if (!produced.empty()) g.addBandValues(produced);
    });
    exStart[k] = exAt;
    exCount[k] = nOut;
    exAt += nOut;
    part.op_last_exchangeWrite = {exStart[k], outBase, uint16_t(nOut)};
    part.op_last_regWrite = {0, 0, 0};
    part.valuePoolSize = g.valuePoolSize();
  }
  d.exchangePoolSize = exAt;

  // ---- region 1 -----------------------------------------------------------
  for (uint32_t k = 0; k < P; ++k) {
    SimPartitionInfo &part = d.parts[P + k];
    PartKind pk = kindFor(P + k);
    PartGen g(rng, part, cnt, pk);
    uint32_t width = uint32_t(std::max<uint64_t>(1, perPart / lv1));
    uint32_t nIn = std::max<uint32_t>(8, std::min<uint32_t>(width + 8, 4096));
    std::vector<uint32_t> ins;
    for (uint32_t j = 0; j < exCount[k] && ins.size() < nIn; ++j) ins.push_back(exStart[k] + j);
    while (ins.size() < nIn) ins.push_back(rng.below(exAt));
    for (uint32_t e : ins) g.addInput(e, true);
    g.finishInputs();
    uint32_t nOut = L.ffCount[k];
    uint16_t outBase = g.slot(nOut, 4);
    bool stopHere = c.with_stop && k == 0;
    g.build(lv1, width, nOut, outBase, 0, [&](uint32_t b) {
      uint32_t d1 = std::max(1u, std::min(pk.depth, lv1));
      uint32_t bands = (lv1 + d1 - 1) / d1;
      if (b + 2 != bands && bands > 1) return;
      if (bands == 1 && b != 0) return;
      // memory writes: address and data from the band before the last
      std::vector<CGMicroPartInfo> addrLvl;
      for (auto &mw : writesOf[k]) {
        const MemPlan &mp = mems[mw.first];
        uint16_t addr = g.addressGen(mp.addrBits, writePorts, mw.second, addrLvl);
        for (uint32_t j = 0; j < mp.nibbles; ++j) {
          auto &op = addZeroed(part.ops_last_memWrite);
          op.hasMultipleWriter = mp.multi;
          op.memBase = mp.nibBase[j];
          op.addrVec = addr;
          op.dat = g.anyRecent();
          op.en = 1;
          ++cnt.memW;
        }
      }
      if (!addrLvl.empty()) part.exec_mParts.push_back(std::move(addrLvl));
      if (stopHere) {
        std::vector<CGMicroPartInfo> flagLvl;
        const uint16_t en = c.with_stop == 2 ? g.rareFlag(flagLvl) : g.anyRecent();
        if (!flagLvl.empty()) part.exec_mParts.push_back(std::move(flagLvl));
        part.ops_last_stop.push_back({en});
        part.ops_last_print.push_back({en, 0});
      }
    });
    part.op_last_regWrite = {L.ffStart[k], outBase, uint16_t(nOut)};
    part.op_last_exchangeWrite = {0, 0, 0};
    part.valuePoolSize = g.valuePoolSize();
  }
  if (c.with_stop) d.printMsgs.push_back("stop condition reached\n");

  d.regionPartitionIds.resize(2);
  for (uint32_t k = 0; k < P; ++k) d.regionPartitionIds[0].push_back(k);
  for (uint32_t k = 0; k < P; ++k) d.regionPartitionIds[1].push_back(P + k);

  // internal signals: 1-4 sections of value-pool slots written by a LUT
  // write-back of the partition (drawn from their own generator, so designs
  // without signals stay as they were)
  if (c.signals) {
    Rng srng(c.seed ^ 0x5167A15ull);
    std::vector<std::vector<uint16_t>> written(d.parts.size());
    for (size_t pid = 0; pid < d.parts.size(); ++pid) {
      for (auto &lvl : d.parts[pid].exec_mParts)
        for (auto &m : lvl)
          for (auto &w : m.lastLevel) written[pid].push_back(w.result);
      std::sort(written[pid].begin(), written[pid].end());
      written[pid].erase(std::unique(written[pid].begin(), written[pid].end()), written[pid].end());
    }
    for (uint32_t i = 0; i < c.signals; ++i) {
      uint32_t pid = srng.below(uint32_t(d.parts.size()));
      for (uint32_t tries = 0; written[pid].empty() && tries < d.parts.size(); ++tries) pid = (pid + 1) % d.parts.size();
      if (written[pid].empty()) break;
      const uint32_t nsec = 1 + srng.below(4);
      std::vector<std::tuple<uint32_t, uint32_t, uint32_t>> secs;
      for (uint32_t k = 0; k < nsec; ++k) {
        const uint16_t slot = written[pid][srng.below(uint32_t(written[pid].size()))];
        const uint32_t width = (k == 0) ? 1 + srng.below(4) : 4;
        secs.emplace_back(pid, slot, width);
      }
      s.signalDebugInfo["sig_" + std::to_string(i)] = std::move(secs);
    }
  }

  if (info) {
    std::memset(info, 0, sizeof(*info));
    info->lut_ops = cnt.lut;
    info->nop_ops = cnt.nop;
    info->mparts = cnt.mparts;
    info->partitions = 2ull * P;
    info->mem_read_ops = cnt.memR;
    info->mem_write_ops = cnt.memW;
    info->vec_ops = cnt.vec;
    info->l0_ops = cnt.l0;
    info->reg_pool = d.regPoolSize;
    info->mem_pool = d.memPoolSize;
    info->exchange_pool = d.exchangePoolSize;
    uint32_t mv = 0;
    for (auto &p : d.parts) mv = std::max(mv, p.valuePoolSize);
    info->max_value_pool = mv;
    info->n_pi_nibbles = L.piCount + L.resetCount;
  }
}

}  // namespace tgs

extern "C" int tgs_gen_inputs(const tgs_gen_config *cfg, uint32_t *ids, uint8_t *bits, uint32_t n) {
  if (!cfg) return TGS_ERR_ARG;
  tgs::Layout L = tgs::makeLayout(*cfg);
  if (n != L.piCount + L.resetCount) {
    tgs::setLastError("tgs_gen_inputs: n must equal the primary-input nibble count");
    return TGS_ERR_ARG;
  }
  for (uint32_t i = 0; i < L.piCount; ++i) {
    ids[i] = L.piStart + i;
    bits[i] = uint8_t((i + 1 == L.piCount && cfg->pi_bits % 4) ? cfg->pi_bits % 4 : 4);
  }
  for (uint32_t r = 0; r < L.resetCount; ++r) {
    ids[L.piCount + r] = L.piStart + L.piCount + r;
    bits[L.piCount + r] = 1;
  }
  return TGS_OK;
}
