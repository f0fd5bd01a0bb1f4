// Design -> device image, and the static schedule.
//
// The image replaces the reference's copy_netlist_to_gpu / copyMicroPartToNetlist
// (src/SimEval.cu:69-148,1114-1343): instead of per-level pointer arrays and
// a magic-tagged byte stream per micro-partition, every micro-partition is a
// 16-byte aligned record of lane-major 32-bit words (devimage.h), and the
// order in which warps take micro-partitions is fixed here instead of by the
// shared-memory atomic counter of SimEval.cu:818-843.  The schedule is the
// only thing the greedy and the learned cost models change: values do not
// depend on it for designs that pass the static checks.
#include <algorithm>
#include <cstring>
#include <numeric>
#include <queue>
#include <vector>

#include "emit.h"
#include "slotalloc.h"

namespace tgs {

using namespace toucanGPUSim;

namespace {

void align4(std::vector<uint32_t> &v) {
  while (v.size() % 4) v.push_back(0);
}

}  // namespace

// ---- word-wide evaluation of palette LUT ops -------------------------------
FastLuts::FastLuts(const std::vector<uint8_t> &lut) : lut_(lut), rowCode_(lut.size(), -2), muxCode_(lut.size(), -2) {}

// The 2-input function of a 256-entry row (index b << 4 | c), as the 4-bit
// truth table g of one output bit (bit (x << 1 | y) = g(b bit x, c bit y)),
// when every entry is that function applied to each of the 4 bits; else -1.
int FastLuts::rowCode(uint32_t row) {
  if (row + 256 > lut_.size()) return -1;
  int &memo = rowCode_[row];
  if (memo != -2) return memo;
  memo = -1;
  const uint32_t v01 = lut_[row + 0x0F], v10 = lut_[row + 0xF0], v11 = lut_[row + 0xFF], v00 = lut_[row];
  for (uint32_t v : {v00, v01, v10, v11})
    if (v != 0 && v != 15) return memo;
  const uint32_t g = (v00 & 1u) | ((v01 & 1u) << 1) | ((v10 & 1u) << 2) | ((v11 & 1u) << 3);
  for (uint32_t b = 0; b < 16; ++b)
    for (uint32_t c = 0; c < 16; ++c) {
      uint32_t want = 0;
      for (uint32_t i = 0; i < 4; ++i) want |= ((g >> ((((b >> i) & 1u) << 1) | ((c >> i) & 1u))) & 1u) << i;
      if (lut_[row + (b << 4 | c)] != want) return memo;
    }
  return memo = int(g);
}

// A 4,096-entry window whose rows a = 0 and a = 1 pass one operand each: 1
// for a ? b : c, 2 for a ? c : b, else 0.
int FastLuts::muxCode(uint32_t base) {
  if (base >= 1u << 13 || base + 4096 > lut_.size()) return 0;
  int &memo = muxCode_[base];
  if (memo != -2) return memo;
  const int r0 = rowCode(base), r1 = rowCode(base + 256);
  memo = r0 == kGPassC && r1 == kGPassB ? 1 : r0 == kGPassB && r1 == kGPassC ? 2 : 0;
  return memo;
}

uint16_t FastLuts::code(const CGMicroPartLUTTopLevelOp &o) {
  if (o.lutIndex == 0) return uint16_t(kFastOp | kGPassC);  // a move passes op2
  if (o.op0 < 16) {
    const int g = rowCode(uint32_t(o.lutIndex) + (uint32_t(o.op0) << 8));
    return g < 0 ? 0 : uint16_t(kFastOp | uint32_t(g));
  }
  const int k = muxCode(o.lutIndex);
  return k ? uint16_t(kFastOp | (uint32_t(k) << kFastKindShift) | o.lutIndex) : 0;
}

namespace {

uint32_t emitLut(const CGMicroPartInfo &m, std::vector<uint32_t> &net, MPartFeat &f, FastLuts *fast) {
  uint32_t W = uint32_t(m.topLevel.size());
  for (auto &l : m.middleLevels) W = std::max<uint32_t>(W, uint32_t(l.size()));
  W = std::max<uint32_t>(W, uint32_t(m.lastLevel.size()));
  W = std::max<uint32_t>(W, 1);
  uint32_t nMid = uint32_t(m.middleLevels.size());
  bool direct = true;
  for (size_t l = 0; l < m.lastLevel.size(); ++l) direct = direct && m.lastLevel[l].shuffleId == 32 + l;
  // word-wide top level: every top op (and idle lane) has a fast form
  std::vector<uint16_t> codes;
  bool fastTop = fast != nullptr && !m.topLevel.empty(), sel = false;
  for (size_t l = 0; fastTop && l < m.topLevel.size(); ++l) {
    codes.push_back(fast->code(m.topLevel[l]));
    fastTop = codes.back() != 0;
    sel = sel || ((codes.back() >> kFastKindShift) & 3u) != 0;
  }
  // compact lanes (one word pair per op, the write-back slot inside it): a
  // single-level record whose entry l writes lane l's value, with every slot
  // below 4096 (renumbered value pools are far smaller)
  bool compact = nMid == 0 && direct && !m.topLevel.empty() && m.lastLevel.size() == m.topLevel.size();
  for (size_t l = 0; compact && l < m.topLevel.size(); ++l) {
    const auto &o = m.topLevel[l];
    compact = o.op0 < 4096 && o.op1 < 4096 && o.op2 < 4096 && m.lastLevel[l].result < 4096;
  }
  align4(net);
  uint32_t off = uint32_t(net.size());
  net.push_back(kMPLut | (W << 2) | (nMid << 8) | (uint32_t(m.lastLevel.size()) << 16) |
                (uint32_t(m.topLevel.size()) << 24) | (direct ? kMPDirectWB : 0u) | (fastTop ? kMPFastTop : 0u) |
                (fastTop && sel ? kMPFastSel : 0u) | (compact ? kMPCompact : 0u));
  net.push_back(0);
  net.push_back(0);
  net.push_back(0);
  for (uint32_t l = 0; l < W; ++l) {
    if (l < m.topLevel.size()) {
      const auto &o = m.topLevel[l];
      uint32_t lutW = o.lutIndex, aW = o.op0;
      if (fastTop) {
        // the table form stays readable (single streams evaluate by lookups):
        // lutIndex in bits 0..12, and for kind 0 op0 in bits 0..3 of the op0
        // field with g above it (a move's op0 is never read)
        const uint32_t kind = (codes[l] >> kFastKindShift) & 3u;
        lutW = o.lutIndex | kFastOp | (kind << kFastKindShift);
        if (kind == 0) aW = (o.lutIndex ? o.op0 & 15u : 0u) | ((codes[l] & 15u) << 4);
      }
      if (compact) {
        const uint32_t c = o.op2, res = m.lastLevel[l].result;
        net.push_back(aW | (uint32_t(o.op1) << 12) | ((c & 0xFFu) << 24));
        net.push_back((c >> 8) | (res << 4) | (lutW << 16));
      } else {
        net.push_back(lutW | (aW << 16));
        net.push_back(uint32_t(o.op1) | (uint32_t(o.op2) << 16));
      }
      f.fastOps += fastTop && o.lutIndex != 0;
      f.ops += 1;
      f.nops += o.lutIndex == 0;
      f.vpReads += (o.op0 >= 16) + (o.op1 >= 16) + (o.op2 >= 16);
      f.threeOp += o.op0 >= 16;
    } else {
      net.push_back(0);
      net.push_back(0);
    }
  }
  for (auto &lvl : m.middleLevels)
    for (uint32_t l = 0; l < W; ++l) {
      uint32_t w = l < lvl.size() ? lvl[l].getPacked() : 0u;
      net.push_back(w);
      if (l < lvl.size()) {
        f.ops += 1;
        f.nops += (w >> 18) == 0;
        f.threeOp += ((w >> 12) & 63) >= 32;
      }
    }
  for (uint32_t l = 0; l < W && !compact; ++l) {
    if (l < m.lastLevel.size())
      net.push_back(uint32_t(m.lastLevel[l].shuffleId) | (uint32_t(m.lastLevel[l].result) << 16));
    else
      net.push_back(0);
  }
  f.kind = kMPLut;
  f.fastTop = fastTop ? 1u : 0u;
  f.lanes = W;
  f.depth = nMid + 1;
  f.writes = uint32_t(m.lastLevel.size());
  return off;
}

// ---- lane packing of narrow LUT micro-partitions --------------------------
// A LUT micro-partition of W lanes occupies a whole warp for its top level,
// its middle levels and its write-back.  Narrow ones (W <= kPackMaxLanes) of
// one exec level are laid side by side into 32-lane micro-partitions: member
// k keeps its ops on lanes [off_k, off_k + W_k), its lane references (middle
// operands 32..63, write-back shuffle ids >= 32) move by off_k, a member with
// fewer middle levels carries its values through the extra levels with
// moves of its own lane (lut 0 passes op2, SimEval.cu:350-352), and idle
// lanes keep the zero ops that give them the value 0 as before.  Members
// touch disjoint value-pool slots (micro-partitions of one level do), so the
// packed one computes exactly what the members did.  A member qualifies only
// if every lane it references lies inside its own W lanes.
constexpr uint32_t kPackMaxLanes = 16;

uint32_t lutWidth(const CGMicroPartInfo &m) {
  uint32_t W = uint32_t(m.topLevel.size());
  for (auto &l : m.middleLevels) W = std::max<uint32_t>(W, uint32_t(l.size()));
  return std::max<uint32_t>(std::max<uint32_t>(W, uint32_t(m.lastLevel.size())), 1);
}

bool packable(const CGMicroPartInfo &m) {
  if (!m.isLUTPart || m.lastLevel.empty()) return false;
  const uint32_t W = lutWidth(m);
  if (W > kPackMaxLanes) return false;
  for (auto &lvl : m.middleLevels)
    for (auto &op : lvl)
      for (uint32_t x : {uint32_t(op.op0()), uint32_t(op.op1()), uint32_t(op.op2())})
        if (x >= 32 && x - 32 >= W) return false;
  for (auto &w : m.lastLevel)
    if (w.shuffleId >= 32 && (w.shuffleId & 31u) >= W) return false;
  return true;
}

CGMicroPartInfo packMembers(const std::vector<CGMicroPartInfo> &in, const std::vector<uint32_t> &members) {
  CGMicroPartInfo out;
  out.isLUTPart = true;
  uint32_t nMid = 0, lanes = 0;
  for (uint32_t i : members) {
    nMid = std::max<uint32_t>(nMid, uint32_t(in[i].middleLevels.size()));
    lanes += lutWidth(in[i]);
  }
  out.topLevel.assign(lanes, CGMicroPartLUTTopLevelOp{0, 0, 0, 0});
  out.middleLevels.assign(nMid, std::vector<CGMicroPartLUTMiddleLevelOp>(lanes));
  auto lane = [](uint32_t x, uint32_t off) { return uint8_t(x >= 32 ? 32 + off + (x & 31u) : x); };
  uint32_t off = 0;
  for (size_t k = 0; k < members.size(); ++k) {
    const CGMicroPartInfo &m = in[members[k]];
    const uint32_t W = lutWidth(m);
    for (size_t l = 0; l < m.topLevel.size(); ++l) out.topLevel[off + l] = m.topLevel[l];
    for (uint32_t lv = 0; lv < nMid; ++lv)
      for (uint32_t l = 0; l < W; ++l) {
        auto &dst = out.middleLevels[lv][off + l];
        if (lv < m.middleLevels.size()) {
          if (l < m.middleLevels[lv].size()) {
            const auto &op = m.middleLevels[lv][l];
            dst = CGMicroPartLUTMiddleLevelOp(op.lutIndex(), lane(op.op0(), off), lane(op.op1(), off), lane(op.op2(), off));
          }  // else a zero op, as the member's idle lane had
        } else {
          dst = CGMicroPartLUTMiddleLevelOp(0, 0, 0, uint8_t(32 + off + l));  // carry the lane's value
        }
      }
    // write-back entry l sits on lane l: the member's entries on its lanes;
    // lanes between its entries and the next member repeat its last entry
    // (the same value into the same slot)
    const uint32_t nWB = uint32_t(m.lastLevel.size());
    const bool last = k + 1 == members.size();
    for (uint32_t l = 0; l < (last ? nWB : W); ++l) {
      CGMicroPartLUTLastLevelWriteBack w = m.lastLevel[std::min(l, nWB - 1)];
      w.shuffleId = lane(w.shuffleId >= 64 ? 32u + (w.shuffleId & 31u) : w.shuffleId, off);
      out.lastLevel.push_back(w);
    }
    off += W;
  }
  return out;
}

}  // namespace

// The exec level with its narrow LUT micro-partitions packed (first fit,
// deepest and widest first, so members of a packed one have similar depth).
std::vector<CGMicroPartInfo> packLevel(const std::vector<CGMicroPartInfo> &in) {
  std::vector<uint32_t> cand, out;
  std::vector<CGMicroPartInfo> res;
  for (uint32_t i = 0; i < in.size(); ++i) (packable(in[i]) ? cand : out).push_back(i);
  if (cand.size() < 2) return in;
  std::stable_sort(cand.begin(), cand.end(), [&](uint32_t a, uint32_t b) {
    const size_t da = in[a].middleLevels.size(), db = in[b].middleLevels.size();
    return da != db ? da > db : lutWidth(in[a]) > lutWidth(in[b]);
  });
  std::vector<std::vector<uint32_t>> bins;
  std::vector<uint32_t> used;
  for (uint32_t i : cand) {
    const uint32_t W = lutWidth(in[i]);
    size_t b = 0;
    while (b < bins.size() && used[b] + W > 32) ++b;
    if (b == bins.size()) {
      bins.emplace_back();
      used.push_back(0);
    }
    bins[b].push_back(i);
    used[b] += W;
  }
  for (uint32_t i : out) res.push_back(in[i]);
  for (auto &b : bins) res.push_back(b.size() == 1 ? in[b[0]] : packMembers(in, b));
  return res;
}

// Regrouping of single-level LUT micro-partitions (see emit.h).
std::vector<CGMicroPartInfo> regroupLevel(const std::vector<CGMicroPartInfo> &in, FastLuts *fast) {
  std::vector<uint32_t> cand;
  for (uint32_t i = 0; i < in.size(); ++i)
    if (in[i].isLUTPart && in[i].middleLevels.empty() && !in[i].lastLevel.empty()) cand.push_back(i);
  if (cand.empty()) return in;
  struct Item {
    CGMicroPartLUTTopLevelOp op;
    std::vector<uint16_t> results;  // slots that take the op's value
    uint32_t cls;                   // 0 word-wide, 1 word-wide multiplexer, 2 table
  };
  std::vector<Item> items;
  std::vector<std::pair<uint8_t, uint16_t>> imm;  // (immediate value, slot)
  std::vector<int32_t> writer;                    // slot -> item (or -2 for an immediate), -1 none
  std::vector<uint8_t> readSlot;
  auto grow = [&](uint32_t s) {
    if (s >= writer.size()) {
      writer.resize(s + 1, -1);
      readSlot.resize(s + 1, 0);
    }
  };
  // the value an entry takes: (item, -1) for a lane, (-1, value) for an immediate
  for (uint32_t i : cand) {
    const CGMicroPartInfo &m = in[i];
    const uint32_t base = uint32_t(items.size()), nTop = uint32_t(m.topLevel.size());
    for (auto &o : m.topLevel) {
      const uint16_t code = fast ? fast->code(o) : 0;
      const uint32_t cls = code == 0 ? 2u : ((code >> kFastKindShift) & 3u) ? 1u : 0u;
      items.push_back({o, {}, cls});
      for (uint16_t s : {o.op0, o.op1, o.op2})
        if (s >= 16) {
          grow(s);
          readSlot[s] = 1;
        }
    }
    for (auto &w : m.lastLevel) {
      int32_t src = -2;  // immediate
      uint8_t val = w.shuffleId;
      if (w.shuffleId >= 32) {
        const uint32_t lane = w.shuffleId & 31u;
        if (lane < nTop) src = int32_t(base + lane);
        else val = 0;  // an idle lane holds 0
      }
      grow(w.result);
      if (writer[w.result] != -1) {
        // the same value into the same slot again is harmless; anything else
        // leaves the level as it is
        const bool same = src >= 0 ? writer[w.result] == src
                                   : writer[w.result] == -2 &&
                                         std::any_of(imm.begin(), imm.end(), [&](auto &e) { return e.second == w.result && e.first == val; });
        if (!same) return in;
        continue;
      }
      writer[w.result] = src;
      if (src >= 0) items[size_t(src)].results.push_back(w.result);
      else imm.push_back({val, w.result});
    }
  }
  for (size_t s = 0; s < writer.size(); ++s)
    if (writer[s] != -1 && readSlot[s]) return in;  // an op reads a slot the level writes
  for (const Item &it : items)
    if (it.results.size() > 32) return in;  // more write-back entries than one micro-partition holds
  std::stable_sort(items.begin(), items.end(), [](const Item &a, const Item &b) { return a.cls < b.cls; });
  // a partial word-wide micro-partition that would add a warp pass to the
  // level (its ops fit in the partial table one) joins the table ops instead
  {
    const size_t F = size_t(std::count_if(items.begin(), items.end(), [](const Item &it) { return it.cls < 2; }));
    const size_t T = items.size() - F;
    if (F % 32 && T % 32 && F % 32 + T % 32 <= 32)
      for (size_t i = F - F % 32; i < F; ++i) items[i].cls = 2;
  }
  std::vector<CGMicroPartInfo> out;
  for (uint32_t i = 0; i < in.size(); ++i)
    if (!(in[i].isLUTPart && in[i].middleLevels.empty() && !in[i].lastLevel.empty())) out.push_back(in[i]);
  CGMicroPartInfo cur;
  uint32_t curCls = 0;
  auto flush = [&]() {
    if (!cur.topLevel.empty() || !cur.lastLevel.empty()) out.push_back(std::move(cur));
    cur = CGMicroPartInfo();
    cur.isLUTPart = true;
  };
  cur.isLUTPart = true;
  for (const Item &it : items) {
    const bool table = it.cls == 2;
    if (!cur.topLevel.empty() && ((curCls == 2) != table || cur.topLevel.size() == 32 ||
                                  cur.lastLevel.size() + it.results.size() > 32))
      flush();
    curCls = it.cls;
    const uint8_t lane = uint8_t(32 + cur.topLevel.size());
    cur.topLevel.push_back(it.op);
    for (uint16_t r : it.results) cur.lastLevel.push_back({lane, r});
  }
  for (auto &e : imm) {
    if (cur.lastLevel.size() == 32) flush();
    cur.lastLevel.push_back({e.first, e.second});
  }
  flush();
  return out;
}

namespace {

uint32_t emitSpecial(const CGMicroPartInfo &m, std::vector<uint32_t> &net, MPartFeat &f) {
  align4(net);
  uint32_t off = uint32_t(net.size());
  if (!m.vecRead.empty()) {
    uint32_t n = uint32_t(m.vecRead.size());
    net.push_back(kMPVecRead | (n << 2));
    net.push_back(0); net.push_back(0); net.push_back(0);
    for (auto &o : m.vecRead) {
      net.push_back(uint32_t(o.vecBase) | (uint32_t(o.vecLength) << 16));
      net.push_back(uint32_t(o.offset) | (uint32_t(o.isConstVec ? 1 : 0) << 16));
      net.push_back(uint32_t(o.index0) | (uint32_t(o.index1) << 16));
      net.push_back(uint32_t(o.index2) | (uint32_t(o.index3) << 16));
      net.push_back(uint32_t(o.outRangeValue) | (uint32_t(o.result) << 16));
    }
    f.kind = kMPVecRead;
    f.lanes = n;
    f.ops = n;
    f.vpReads = 5 * n;
    f.writes = n;
  } else if (!m.vecArithAndLogic.empty()) {
    uint32_t n = uint32_t(m.vecArithAndLogic.size());
    net.push_back(kMPVecOp | (n << 2));
    net.push_back(0); net.push_back(0); net.push_back(0);
    for (auto &o : m.vecArithAndLogic) {
      net.push_back(uint32_t(o.vec1Base) | (uint32_t(o.vec2Base) << 16));
      net.push_back(uint32_t(o.vecLength) | (uint32_t(o.opName) << 16) | (uint32_t(o.isV1V2Const) << 24));
      net.push_back(uint32_t(o.result));
      f.vecNibbles += o.vecLength;
      f.writes += o.opName <= VEC_ARITH_MUL ? o.vecLength : 1;
    }
    f.kind = kMPVecOp;
    f.lanes = n;
    f.ops = n;
    f.vpReads = 2 * f.vecNibbles;
  } else {
    uint32_t n = uint32_t(m.memRead.size());
    net.push_back(kMPMemRead | (n << 2));
    net.push_back(0); net.push_back(0); net.push_back(0);
    for (auto &o : m.memRead) {
      net.push_back(uint32_t(o.memBase & 0xFFFFFFFFu));
      net.push_back(uint32_t((o.memBase >> 32) & 0x7FFFFFFFu) | (o.hasMultipleWriter ? 0x80000000u : 0u));
      net.push_back(uint32_t(o.en) | (uint32_t(o.addrVec) << 16));
      net.push_back(uint32_t(o.result));
    }
    f.kind = kMPMemRead;
    f.lanes = n;
    f.ops = n;
    f.memPorts = n;
    f.vpReads = 9 * n;
    f.writes = n;
  }
  f.depth = 1;
  return off;
}

// Slots read / written by a micro-partition (for barrier placement).
void accessOf(const CGMicroPartInfo &m, std::vector<uint32_t> &rd, std::vector<uint32_t> &wr) {
  if (m.isLUTPart) {
    for (auto &o : m.topLevel) {
      if (o.op0 >= 16) rd.push_back(o.op0);
      if (o.op1 >= 16) rd.push_back(o.op1);
      if (o.op2 >= 16) rd.push_back(o.op2);
    }
    for (auto &w : m.lastLevel) wr.push_back(w.result);
  } else if (!m.vecRead.empty()) {
    for (auto &o : m.vecRead) {
      for (uint16_t s : {o.index0, o.index1, o.index2, o.index3})
        if (s >= 16) rd.push_back(s);
      if (o.outRangeValue >= 16) rd.push_back(o.outRangeValue);
      if (!o.isConstVec)
        for (uint32_t i = 0; i < o.vecLength; ++i) rd.push_back(o.vecBase + i);
      wr.push_back(o.result);
    }
  } else if (!m.vecArithAndLogic.empty()) {
    for (auto &o : m.vecArithAndLogic) {
      if (!(o.isV1V2Const & 2))
        for (uint32_t i = 0; i < o.vecLength; ++i) rd.push_back(o.vec1Base + i);
      if (!(o.isV1V2Const & 1))
        for (uint32_t i = 0; i < o.vecLength; ++i) rd.push_back(o.vec2Base + i);
      uint32_t n = o.opName <= VEC_ARITH_MUL ? o.vecLength : 1;
      for (uint32_t i = 0; i < n; ++i) wr.push_back(uint16_t(o.result + i));
    }
  } else {
    for (auto &o : m.memRead) {
      if (o.en >= 16) rd.push_back(o.en);
      for (uint32_t j = 0; j < 8; ++j) rd.push_back(o.addrVec + j);
      if (o.en != 0) wr.push_back(o.result);
    }
  }
}

}  // namespace

void buildImage(const SimDesignInfo &d, DeviceImage &img, bool compactSlots, const ProbeList *probes, bool packLanes,
                bool fastLuts) {
  img = DeviceImage();
  FastLuts fl(d.lut);
  FastLuts *fast = fastLuts && d.lut.size() == kLutSize ? &fl : nullptr;
  img.parts.resize(d.parts.size());
  img.mp.resize(d.parts.size());
  img.partRegion.assign(d.parts.size(), 0);
  for (size_t r = 0; r < d.regionPartitionIds.size(); ++r)
    for (uint32_t id : d.regionPartitionIds[r]) img.partRegion[id] = uint32_t(r);
  auto &net = img.net;
  img.renumbered = compactSlots;
  for (uint32_t pid = 0; pid < d.parts.size(); ++pid) {
    const SimPartitionInfo &orig = d.parts[pid];
    SimPartitionInfo renamed;
    const SimPartitionInfo *pp = &orig;
    std::vector<uint32_t> keep, newOf;
    if (probes && pid < probes->size())
      for (auto &pr : (*probes)[pid]) keep.push_back(pr.first);
    if (compactSlots) {
      const uint32_t n = planSlots(orig, newOf, keep.empty() ? nullptr : &keep);
      if (n <= 65534) {
        renamed = orig;
        renameSlots(renamed, newOf, n);
        pp = &renamed;
      } else {
        newOf.clear();
        img.renumbered = false;
      }
    }
    const SimPartitionInfo &p = *pp;
    PartDesc &pd = img.parts[pid];
    std::memset(&pd, 0, sizeof(pd));
    pd.vpSlots = (std::max<uint32_t>(p.valuePoolSize, 16) + 3) & ~3u;
    pd.region = img.partRegion[pid];
    // L0 reads
    bool exg = !p.ops_l0_exchangeRead.empty();
    pd.l0Exchange = exg ? 1 : 0;
    pd.l0Count = uint32_t(exg ? p.ops_l0_exchangeRead.size() : p.ops_l0_regRead.size());
    align4(net);
    pd.l0Off = uint32_t(net.size());
    for (uint32_t i = 0; i < pd.l0Count; ++i) net.push_back(exg ? p.ops_l0_exchangeRead[i].exchange : p.ops_l0_regRead[i].reg);
    for (uint32_t i = 0; i < pd.l0Count; i += 2) {
      auto dst = [&](uint32_t k) -> uint32_t {
        if (k >= pd.l0Count) return 0;
        return exg ? p.ops_l0_exchangeRead[k].result : p.ops_l0_regRead[k].result;
      };
      net.push_back(dst(i) | (dst(i + 1) << 16));
    }
    // micro-partitions
    pd.nLevels = uint32_t(p.exec_mParts.size());
    img.mp[pid].resize(pd.nLevels);
    for (uint32_t lv = 0; lv < pd.nLevels; ++lv) {
      std::vector<CGMicroPartInfo> packed;
      if (packLanes) packed = packLevel(p.exec_mParts[lv]);
      if (fast) packed = regroupLevel(packLanes ? packed : p.exec_mParts[lv], fast);
      for (const auto &m : (packLanes || fast) ? packed : p.exec_mParts[lv]) {
        MPartRef ref;
        ref.feat.partLevels = pd.nLevels;
        ref.off = m.isLUTPart ? emitLut(m, net, ref.feat, fast) : emitSpecial(m, net, ref.feat);
        ref.words = uint32_t((net.size() + 3) / 4 * 4) - ref.off;
        ref.id = img.nMParts++;
        net[ref.off + 1] = ref.id;  // header word 1: design-wide micro-partition id (profiling)
        accessOf(m, ref.reads, ref.writes);
        std::sort(ref.reads.begin(), ref.reads.end());
        ref.reads.erase(std::unique(ref.reads.begin(), ref.reads.end()), ref.reads.end());
        ref.feat.fanIn = uint32_t(ref.reads.size());
        img.mp[pid][lv].push_back(std::move(ref));
      }
    }
    // fan-out: later reads of each micro-partition's outputs within the partition
    {
      std::vector<int64_t> writer(std::max<uint32_t>(p.valuePoolSize, 16) + 64, -1);
      std::vector<MPartRef *> flat;
      for (auto &lvl : img.mp[pid])
        for (auto &r : lvl) flat.push_back(&r);
      size_t idx = 0;
      for (auto &lvl : img.mp[pid]) {
        const size_t first = idx;
        for (auto &r : lvl) {
          for (uint32_t sl : r.reads)
            if (sl < writer.size() && writer[sl] >= 0) flat[size_t(writer[sl])]->feat.fanOut++;
          ++idx;
        }
        idx = first;
        for (auto &r : lvl) {
          for (uint32_t sl : r.writes)
            if (sl < writer.size()) writer[sl] = int64_t(idx);
          ++idx;
        }
      }
    }
    // last level
    if (p.op_last_exchangeWrite.count != 0) {
      auto op = lastLevelExchangeOp(p);
      pd.copyKind = 2;
      pd.copySrc = op.dat & ~3u;
      pd.copyDst = op.exchange & ~3u;
      pd.copySlots = (uint32_t(op.count) + 3) / 4 * 4;
    } else {
      if (p.op_last_regWrite.count != 0) {
        pd.copyKind = 1;
        pd.copySrc = p.op_last_regWrite.dat & ~3u;
        pd.copyDst = p.op_last_regWrite.reg & ~3u;
        pd.copySlots = (uint32_t(p.op_last_regWrite.count) + 3) / 4 * 4;
      }
      align4(net);
      pd.memWCount = uint32_t(p.ops_last_memWrite.size());
      pd.memWOff = uint32_t(net.size());
      for (auto &w : p.ops_last_memWrite) {
        net.push_back(uint32_t(w.memBase & 0xFFFFFFFFu));
        net.push_back(uint32_t((w.memBase >> 32) & 0x7FFFFFFFu) | (w.hasMultipleWriter ? 0x80000000u : 0u));
        net.push_back(uint32_t(w.addrVec) | (uint32_t(w.dat) << 16));
        net.push_back(uint32_t(w.en));
      }
      pd.printCount = uint32_t(p.ops_last_print.size());
      pd.printOff = uint32_t(net.size());
      for (auto &pr : p.ops_last_print) net.push_back(uint32_t(pr.en) | (uint32_t(pr.msg) << 16));
      pd.stopCount = uint32_t(p.ops_last_stop.size());
      pd.stopOff = uint32_t(net.size());
      // enable slot | the design file's number of it (for the stop diagnostic)
      for (size_t i = 0; i < p.ops_last_stop.size(); ++i)
        net.push_back(uint32_t(p.ops_last_stop[i].en) | (uint32_t(orig.ops_last_stop[i].en) << 16));
    }
    // signal probes: (slot in the image's numbering, probe index)
    align4(net);
    pd.probeOff = uint32_t(net.size());
    if (probes && pid < probes->size())
      for (auto &pr : (*probes)[pid]) {
        uint32_t slot = pr.first;
        if (!newOf.empty()) slot = slot < newOf.size() ? newOf[slot] : kNoSlot;
        if (slot == kNoSlot || slot >= pd.vpSlots) continue;  // never written here: no value to record
        net.push_back(slot);
        net.push_back(pr.second);
        ++pd.probeCount;
      }
    pd.constOff = uint32_t(img.constVec.size());
    pd.constLen = uint32_t(p.constVecPool.size());
    img.constVec.insert(img.constVec.end(), p.constVecPool.begin(), p.constVecPool.end());
    while (img.constVec.size() % 16) img.constVec.push_back(0);
    img.maxVpSlots = std::max(img.maxVpSlots, pd.vpSlots);
  }
  align4(net);
  if (net.empty()) net.resize(4, 0);
  if (img.constVec.empty()) img.constVec.resize(16, 0);
}

// Greedy gate-count cost of a micro-partition (the fallback cost model).
float gateCost(const MPartFeat &f) { return float(std::max<uint32_t>(1, f.ops)); }

namespace {

// Union-find over micro-partitions (fusing exec levels).
struct Dsu {
  std::vector<uint32_t> p;
  explicit Dsu(size_t n) : p(n) { std::iota(p.begin(), p.end(), 0u); }
  uint32_t find(uint32_t x) {
    while (p[x] != x) x = p[x] = p[p[x]];
    return x;
  }
  void join(uint32_t a, uint32_t b) { p[find(a)] = find(b); }
};

}  // namespace

void buildSchedule(const SimDesignInfo &d, DeviceImage &img, uint32_t NW, uint32_t G,
                   const std::vector<std::vector<std::vector<float>>> *cost, uint32_t nBlocks, uint32_t nGroupBlocks,
                   Schedule &out, const SchedOpts &so) {
  out = Schedule();
  out.NW = NW;
  out.partCost.assign(d.parts.size(), 0.0);
  auto &sw = out.words;
  const uint32_t bundle = std::max<uint32_t>(1, so.unitLanes / 32);
  const uint32_t lpb = std::max<uint32_t>(1, so.levelsPerBarrier);
  // a unit of work: micro-partition i of exec level lv, stream groups [g0, g0 + gn)
  struct Unit {
    uint32_t lv, i, g0, gn;
    double c;
  };
  using Plan = std::vector<std::vector<Unit>>;  // units per warp, in execution order
  for (uint32_t pid = 0; pid < d.parts.size(); ++pid) {
    PartDesc &pd = img.parts[pid];
    const auto &levels = img.mp[pid];
    const uint32_t nLv = uint32_t(levels.size());
    pd.schedOff = uint32_t(out.levelDesc.size() / 2);
    double total = 0;
    auto costOf = [&](uint32_t lv, uint32_t i) {
      return cost ? double((*cost)[pid][lv][i]) : double(gateCost(levels[lv][i].feat));
    };
    // One exec level on its own: a LUT micro-partition runs every group of the
    // item in one warp (its lanes share the operand loads), a special one is
    // split into one unit per group (a level holding one of them keeps G warps
    // busy); LUT units go to warps in bundles of `bundle` (micro-partitions of
    // 32 x bundle LUTs per warp), largest cost first onto the least loaded warp.
    auto planLevel = [&](uint32_t lv, Plan &plan) {
      const auto &mps = levels[lv];
      std::vector<std::vector<Unit>> items;  // LPT items: bundles of units
      std::vector<Unit> luts;
      for (uint32_t i = 0; i < mps.size(); ++i) {
        if (mps[i].feat.kind != kMPLut && G > 1)
          for (uint32_t g = 0; g < G; ++g) items.push_back({{lv, i, g, 1, costOf(lv, i) / G}});
        else
          luts.push_back({lv, i, 0, G, costOf(lv, i)});
      }
      std::stable_sort(luts.begin(), luts.end(), [](const Unit &a, const Unit &b) { return a.c > b.c; });
      for (size_t k = 0; k < luts.size(); k += bundle)
        items.emplace_back(luts.begin() + k, luts.begin() + std::min(luts.size(), k + bundle));
      std::vector<double> ic(items.size(), 0.0);
      for (size_t k = 0; k < items.size(); ++k)
        for (auto &u : items[k]) ic[k] += u.c;
      std::vector<uint32_t> order(items.size());
      std::iota(order.begin(), order.end(), 0u);
      std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return ic[a] > ic[b]; });
      std::vector<double> load(NW, 0.0);
      plan.assign(NW, {});
      for (uint32_t k : order) {
        const uint32_t w = uint32_t(std::min_element(load.begin(), load.end()) - load.begin());
        load[w] += ic[k];
        plan[w].insert(plan[w].end(), items[k].begin(), items[k].end());
      }
      return *std::max_element(load.begin(), load.end());
    };
    // Exec levels [lv, lv + m) as one block without barriers inside: micro-
    // partitions that touch a slot one of them writes (across the levels)
    // form one component, a component runs on one warp level by level, and
    // components go to warps largest first.  Special micro-partitions run
    // every group in one unit.
    auto planFused = [&](uint32_t lv, uint32_t m, Plan &plan) {
      std::vector<std::pair<uint32_t, uint32_t>> ids;  // (level, i)
      for (uint32_t l = lv; l < lv + m; ++l)
        for (uint32_t i = 0; i < levels[l].size(); ++i) ids.push_back({l, i});
      Dsu dsu(ids.size());
      std::vector<int32_t> lastW(pd.vpSlots + 64, -1);
      std::vector<std::vector<uint32_t>> readers(pd.vpSlots + 64);
      size_t at = 0;
      for (uint32_t l = lv; l < lv + m; ++l) {
        const size_t first = at;
        for (uint32_t i = 0; i < levels[l].size(); ++i, ++at) {
          const MPartRef &r = levels[l][i];
          for (uint32_t s : r.reads)
            if (lastW[s] >= 0) dsu.join(uint32_t(at), uint32_t(lastW[s]));
          for (uint32_t s : r.writes) {
            if (lastW[s] >= 0) dsu.join(uint32_t(at), uint32_t(lastW[s]));
            for (uint32_t x : readers[s]) dsu.join(uint32_t(at), x);
          }
        }
        // the level's own accesses count from the next level on (micro-
        // partitions of one level touch disjoint slots)
        for (size_t k = first; k < at; ++k) {
          const MPartRef &r = levels[ids[k].first][ids[k].second];
          for (uint32_t s : r.reads) readers[s].push_back(uint32_t(k));
          for (uint32_t s : r.writes) {
            lastW[s] = int32_t(k);
            readers[s].clear();
          }
        }
      }
      std::vector<double> cc(ids.size(), 0.0);
      std::vector<std::vector<uint32_t>> members(ids.size());
      for (size_t k = 0; k < ids.size(); ++k) {
        const uint32_t root = dsu.find(uint32_t(k));
        cc[root] += costOf(ids[k].first, ids[k].second);
        members[root].push_back(uint32_t(k));
      }
      std::vector<uint32_t> roots;
      for (uint32_t k = 0; k < ids.size(); ++k)
        if (!members[k].empty()) roots.push_back(k);
      std::stable_sort(roots.begin(), roots.end(), [&](uint32_t a, uint32_t b) { return cc[a] > cc[b]; });
      std::vector<double> load(NW, 0.0);
      plan.assign(NW, {});
      for (uint32_t rt : roots) {
        const uint32_t w = uint32_t(std::min_element(load.begin(), load.end()) - load.begin());
        load[w] += cc[rt];
        for (uint32_t k : members[rt])
          plan[w].push_back({ids[k].first, ids[k].second, 0, G, costOf(ids[k].first, ids[k].second)});
      }
      for (auto &wu : plan)
        std::stable_sort(wu.begin(), wu.end(), [](const Unit &a, const Unit &b) { return a.lv < b.lv; });
      return *std::max_element(load.begin(), load.end());
    };

    // barrier placement: hazards since the last block barrier, tracked per slot
    std::vector<int32_t> lastWriter(pd.vpSlots + 64, -1);  // warp of last write since the barrier
    std::vector<uint32_t> readersMask(pd.vpSlots + 64, 0);  // warps that read since the barrier
    std::vector<uint32_t> touched;
    uint32_t blocks = 0;
    for (uint32_t lv = 0; lv < nLv;) {
      Plan plan;
      double mk = planLevel(lv, plan);
      uint32_t n = 1;
      if (lpb > 1) {
        // fuse as many levels (up to lpb) as run no longer on their warps
        // than the same levels with a barrier between each
        std::vector<double> single;
        for (uint32_t l = lv; l < std::min(nLv, lv + lpb); ++l) {
          Plan tmp;
          single.push_back(l == lv ? mk : planLevel(l, tmp));
        }
        for (uint32_t m = uint32_t(single.size()); m >= 2; --m) {
          Plan fused;
          const double fmk = planFused(lv, m, fused);
          double sep = 0;
          for (uint32_t k = 0; k < m; ++k) sep += single[k];
          if (fmk <= sep) {
            plan = std::move(fused);
            mk = fmk;
            n = m;
            break;
          }
        }
      }
      total += mk;
      {
        double wsum = 0, umax = 0;
        for (const auto &wu : plan)
          for (const Unit &un : wu) {
            wsum += un.c;
            umax = std::max(umax, un.c);
          }
        out.planMakespan += mk;
        out.planWork += wsum;
        out.planLower += std::max(wsum / NW, umax);
        out.planUpper += wsum / NW + umax;
      }
      // does this block need a block barrier first?
      bool need = lv == 0;
      if (!need) {
        for (uint32_t w = 0; w < NW && !need; ++w)
          for (const Unit &un : plan[w]) {
            const MPartRef &r = levels[un.lv][un.i];
            for (uint32_t s : r.reads)
              if (lastWriter[s] >= 0 && lastWriter[s] != int32_t(w)) { need = true; break; }
            if (need) break;
            for (uint32_t s : r.writes)
              if ((lastWriter[s] >= 0 && lastWriter[s] != int32_t(w)) || (readersMask[s] & ~(1u << w))) { need = true; break; }
            if (need) break;
          }
      }
      if (need) {
        for (uint32_t s : touched) { lastWriter[s] = -1; readersMask[s] = 0; }
        touched.clear();
        out.barriers++;
      }
      // a slot written by units of one micro-partition on several warps
      // counts as written by each of them (the last one recorded): every
      // later access from another warp then needs a barrier
      for (uint32_t w = 0; w < NW; ++w)
        for (const Unit &un : plan[w]) {
          const MPartRef &r = levels[un.lv][un.i];
          for (uint32_t s : r.reads) { readersMask[s] |= 1u << w; touched.push_back(s); }
          for (uint32_t s : r.writes) {
            if (lastWriter[s] >= 0 && lastWriter[s] != int32_t(w)) lastWriter[s] = int32_t(NW);  // several warps
            else lastWriter[s] = int32_t(w);
            touched.push_back(s);
          }
        }
      out.levels++;
      // level block: [flags][NW + 1 prefix offsets][unit offsets][pad][micro-partitions in warp order]
      while (sw.size() % 4) sw.push_back(0);
      const uint32_t blk = uint32_t(sw.size());
      uint32_t nUnits = 0;
      for (uint32_t w = 0; w < NW; ++w) nUnits += uint32_t(plan[w].size());
      sw.push_back(need ? 1u : 0u);
      uint32_t acc = 0;
      for (uint32_t w = 0; w < NW; ++w) {
        sw.push_back(acc);
        acc += uint32_t(plan[w].size());
      }
      sw.push_back(acc);
      const uint32_t unitBase = uint32_t(sw.size());
      sw.resize(sw.size() + nUnits, 0);
      while (sw.size() % 4) sw.push_back(0);
      uint32_t u = 0;
      std::vector<std::vector<uint32_t>> recordAt(n);  // one record per micro-partition
      for (uint32_t k = 0; k < n; ++k) recordAt[k].assign(levels[lv + k].size(), UINT32_MAX);
      for (uint32_t w = 0; w < NW; ++w)
        for (const Unit &un : plan[w]) {
          uint32_t &ra = recordAt[un.lv - lv][un.i];
          if (ra == UINT32_MAX) {
            ra = uint32_t(sw.size()) - blk;
            const MPartRef &r = levels[un.lv][un.i];
            sw.insert(sw.end(), img.net.begin() + r.off, img.net.begin() + r.off + r.words);
            while (sw.size() % 4) sw.push_back(0);
          }
          if (ra > kUnitOffsetMask) throw Error(TGS_ERR_RESOURCES, "exec level too large");
          sw[unitBase + u++] = ra | (un.g0 << 24) | ((un.gn - 1) << 27);
        }
      const uint32_t words = uint32_t(sw.size()) - blk;
      out.levelDesc.push_back(blk);
      out.levelDesc.push_back(words);
      out.maxLevelWords = std::max(out.maxLevelWords, words);
      out.fusedLevels += n - 1;
      ++blocks;
      lv += n;
    }
    pd.nLevels = blocks;  // exec-level blocks the kernel runs
    // L0 and last level scale with their op counts spread over the block
    total += double(pd.l0Count + pd.copySlots + 8 * pd.memWCount) / double(32 * NW) + 1.0;
    out.partCost[pid] = total;
  }
  while (sw.size() % 4 || sw.empty()) sw.push_back(0);
  if (out.levelDesc.empty()) out.levelDesc.assign(2, 0);

  // items (partition, group block) onto blocks, per region, LPT by cost
  out.items.clear();
  out.itemBegin.assign(2 * (nBlocks + 1), 0);
  for (uint32_t r = 0; r < 2; ++r) {
    std::vector<std::pair<double, uint32_t>> it;
    for (uint32_t pid : d.regionPartitionIds[r])
      for (uint32_t gb = 0; gb < nGroupBlocks; ++gb) it.push_back({out.partCost[pid], pid | (gb << 20)});
    std::stable_sort(it.begin(), it.end(), [](auto &a, auto &b) { return a.first > b.first; });
    using E = std::pair<double, uint32_t>;
    std::priority_queue<E, std::vector<E>, std::greater<E>> pq;
    for (uint32_t b = 0; b < nBlocks; ++b) pq.push({0.0, b});
    std::vector<std::vector<uint32_t>> perBlock(nBlocks);
    double mk = 0;
    for (auto &e : it) {
      auto top = pq.top();
      pq.pop();
      perBlock[top.second].push_back(e.second);
      top.first += e.first;
      mk = std::max(mk, top.first);
      pq.push(top);
    }
    out.makespan[r] = mk;
    uint32_t base = uint32_t(out.items.size());
    for (uint32_t b = 0; b < nBlocks; ++b) {
      out.itemBegin[r * (nBlocks + 1) + b] = base;
      for (uint32_t x : perBlock[b]) out.items.push_back(x);
      base = uint32_t(out.items.size());
    }
    out.itemBegin[r * (nBlocks + 1) + nBlocks] = base;
  }
  if (out.items.empty()) out.items.push_back(0);
}

}  // namespace tgs
