// Design / symbol file (de)serialization, byte-compatible with the reference
// Serializer (src/Serializer.cpp:25-446, ucsc-vama/toucanGPURT).
//
// File grammar (little endian, no magic, no version):
//   prim<T>      := sizeof(T) raw bytes
//   vec<T>       := u64 count, count * sizeof(T) raw struct bytes (padding included)
//   string       := vec<char>
//   design       := u32 regPoolSize, u32 memPoolSize, u32 exchangePoolSize, bool shouldStop,
//                   vec<u8> lut, vec<u8> regPool, vec<u8> memPool,
//                   u64 nParts, partition*, u64 nRegions, vec<u32>*, u64 nMsgs, string*
//                   (Serializer.cpp:199-223)
//   partition    := vec<u8> valuePool, u32 valuePoolSize, vec<u8> constVecPool,
//                   vec<RegRead>, vec<ExgRead>, u64 nLevels, (u64 nMParts, mpart*)*,
//                   RegWrite, vec<MemWrite>, vec<Print>, vec<Stop>, ExgWrite
//                   (Serializer.cpp:147-166)
//   mpart        := bool isLUT, LUT: vec<Top>, u64 nMid, vec<Mid>*, vec<WriteBack>
//                   else: vec<VecRead>, vec<VecOp>, vec<MemRead>   (Serializer.cpp:106-121)
//   symbols      := 3 maps of (string, u64 n, n raw tuples of u32)  (Serializer.cpp:264-300)
//
// Unlike the reference's per-element istream::read, the loader reads the
// whole stream into memory and copies POD vectors in bulk, with every count
// checked against the bytes left, so a truncated or corrupt file is an error
// instead of an unbounded allocation.
#include <cstring>
#include <istream>
#include <iterator>
#include <ostream>
#include <sstream>
#include <stdexcept>

#include "ToucanGPUGenDataTypes.h"
#include "tgs_internal.h"

namespace toucanGPUSim {

namespace {

class Reader {
 public:
  Reader(const uint8_t *p, size_t n) : p_(p), n_(n) {}

  template <typename T>
  void prim(T &v) {
    need(sizeof(T));
    std::memcpy(&v, p_ + off_, sizeof(T));
    off_ += sizeof(T);
  }
  uint64_t count(size_t elem) {
    uint64_t c;
    prim(c);
    if (elem && c > (n_ - off_) / elem) throw tgs::FormatError("vector count exceeds file size");
    return c;
  }
  template <typename T>
  void vec(std::vector<T> &v) {
    uint64_t c = count(sizeof(T));
    v.resize(c);
    if (c) {
      std::memcpy(static_cast<void *>(v.data()), p_ + off_, c * sizeof(T));
      off_ += c * sizeof(T);
    }
  }
  void str(std::string &s) {
    uint64_t c = count(1);
    s.assign(reinterpret_cast<const char *>(p_ + off_), c);
    off_ += c;
  }
  size_t remaining() const { return n_ - off_; }

 private:
  void need(size_t k) {
    if (k > n_ - off_) throw tgs::FormatError("truncated design/symbol stream");
  }
  const uint8_t *p_;
  size_t n_;
  size_t off_ = 0;
};

class Writer {
 public:
  explicit Writer(std::ostream &o) : o_(o) {}
  template <typename T>
  void prim(const T &v) {
    o_.write(reinterpret_cast<const char *>(&v), sizeof(T));
  }
  template <typename T>
  void vec(const std::vector<T> &v) {
    prim<uint64_t>(v.size());
    if (!v.empty()) o_.write(reinterpret_cast<const char *>(v.data()), v.size() * sizeof(T));
  }
  void str(const std::string &s) {
    prim<uint64_t>(s.size());
    o_.write(s.data(), s.size());
  }

 private:
  std::ostream &o_;
};

void readMPart(Reader &r, CGMicroPartInfo &m) {
  r.prim(m.isLUTPart);
  m.topLevel.clear();
  m.middleLevels.clear();
  m.lastLevel.clear();
  m.vecRead.clear();
  m.vecArithAndLogic.clear();
  m.memRead.clear();
  if (m.isLUTPart) {
    r.vec(m.topLevel);
    uint64_t nMid = r.count(8);
    m.middleLevels.resize(nMid);
    for (auto &lvl : m.middleLevels) r.vec(lvl);
    r.vec(m.lastLevel);
  } else {
    r.vec(m.vecRead);
    r.vec(m.vecArithAndLogic);
    r.vec(m.memRead);
  }
}

void writeMPart(Writer &w, const CGMicroPartInfo &m) {
  w.prim(m.isLUTPart);
  if (m.isLUTPart) {
    w.vec(m.topLevel);
    w.prim<uint64_t>(m.middleLevels.size());
    for (const auto &lvl : m.middleLevels) w.vec(lvl);
    w.vec(m.lastLevel);
  } else {
    w.vec(m.vecRead);
    w.vec(m.vecArithAndLogic);
    w.vec(m.memRead);
  }
}

void readPart(Reader &r, SimPartitionInfo &p) {
  r.vec(p.valuePool);
  r.prim(p.valuePoolSize);
  r.vec(p.constVecPool);
  r.vec(p.ops_l0_regRead);
  r.vec(p.ops_l0_exchangeRead);
  uint64_t nLevels = r.count(8);
  p.exec_mParts.resize(nLevels);
  for (auto &lvl : p.exec_mParts) {
    uint64_t n = r.count(1);
    lvl.resize(n);
    for (auto &m : lvl) readMPart(r, m);
  }
  r.prim(p.op_last_regWrite);
  r.vec(p.ops_last_memWrite);
  r.vec(p.ops_last_print);
  r.vec(p.ops_last_stop);
  r.prim(p.op_last_exchangeWrite);
}

void writePart(Writer &w, const SimPartitionInfo &p) {
  w.vec(p.valuePool);
  w.prim(p.valuePoolSize);
  w.vec(p.constVecPool);
  w.vec(p.ops_l0_regRead);
  w.vec(p.ops_l0_exchangeRead);
  w.prim<uint64_t>(p.exec_mParts.size());
  for (const auto &lvl : p.exec_mParts) {
    w.prim<uint64_t>(lvl.size());
    for (const auto &m : lvl) writeMPart(w, m);
  }
  w.prim(p.op_last_regWrite);
  w.vec(p.ops_last_memWrite);
  w.vec(p.ops_last_print);
  w.vec(p.ops_last_stop);
  w.prim(p.op_last_exchangeWrite);
}

template <typename Tuple>
void readSymbolMap(Reader &r, std::unordered_map<std::string, std::vector<Tuple>> &m) {
  uint64_t n = r.count(16);
  for (uint64_t i = 0; i < n; ++i) {
    std::string key;
    r.str(key);
    uint64_t k = r.count(sizeof(uint32_t) * std::tuple_size<Tuple>::value);
    std::vector<Tuple> v(k);
    for (auto &t : v) {
      if constexpr (std::tuple_size<Tuple>::value == 2) {
        r.prim(std::get<0>(t));
        r.prim(std::get<1>(t));
      } else {
        r.prim(std::get<0>(t));
        r.prim(std::get<1>(t));
        r.prim(std::get<2>(t));
      }
    }
    m[key] = std::move(v);
  }
}

template <typename Tuple>
void writeSymbolMap(Writer &w, const std::unordered_map<std::string, std::vector<Tuple>> &m) {
  w.prim<uint64_t>(m.size());
  for (const auto &kv : m) {
    w.str(kv.first);
    w.prim<uint64_t>(kv.second.size());
    for (const auto &t : kv.second) {
      w.prim(std::get<0>(t));
      w.prim(std::get<1>(t));
      if constexpr (std::tuple_size<Tuple>::value == 3) w.prim(std::get<2>(t));
    }
  }
}

std::vector<uint8_t> slurp(std::istream &in) {
  return std::vector<uint8_t>(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
}

}  // namespace

}  // namespace toucanGPUSim

namespace tgs {

void parseDesign(const uint8_t *data, size_t n, toucanGPUSim::SimDesignInfo &d) {
  using namespace toucanGPUSim;
  Reader r(data, n);
  r.prim(d.regPoolSize);
  r.prim(d.memPoolSize);
  r.prim(d.exchangePoolSize);
  r.prim(d.shouldStop);
  r.vec(d.lut);
  r.vec(d.regPool);
  r.vec(d.memPool);
  uint64_t nParts = r.count(8);
  d.parts.resize(nParts);
  for (auto &p : d.parts) readPart(r, p);
  uint64_t nRegions = r.count(8);
  d.regionPartitionIds.resize(nRegions);
  for (auto &ids : d.regionPartitionIds) r.vec(ids);
  uint64_t nMsgs = r.count(8);
  d.printMsgs.resize(nMsgs);
  for (auto &s : d.printMsgs) r.str(s);
}

void parseSymbols(const uint8_t *data, size_t n, toucanGPUSim::SimDebugInfo &s) {
  using namespace toucanGPUSim;
  Reader r(data, n);
  toucanGPUSim::readSymbolMap(r, s.regDebugInfo);
  toucanGPUSim::readSymbolMap(r, s.signalDebugInfo);
  toucanGPUSim::readSymbolMap(r, s.memDebugInfo);
}

}  // namespace tgs

namespace toucanGPUSim {

void serializeSimDesignInfo(std::ostream &out, const SimDesignInfo &d) {
  Writer w(out);
  w.prim(d.regPoolSize);
  w.prim(d.memPoolSize);
  w.prim(d.exchangePoolSize);
  w.prim(d.shouldStop);
  w.vec(d.lut);
  w.vec(d.regPool);
  w.vec(d.memPool);
  w.prim<uint64_t>(d.parts.size());
  for (const auto &p : d.parts) writePart(w, p);
  w.prim<uint64_t>(d.regionPartitionIds.size());
  for (const auto &ids : d.regionPartitionIds) w.vec(ids);
  w.prim<uint64_t>(d.printMsgs.size());
  for (const auto &s : d.printMsgs) w.str(s);
}

void deserializeSimDesignInfo(std::istream &in, SimDesignInfo &d) {
  std::vector<uint8_t> buf = slurp(in);
  tgs::parseDesign(buf.data(), buf.size(), d);
}

void serializeSimDebugInfo(std::ostream &out, const SimDebugInfo &s) {
  Writer w(out);
  writeSymbolMap(w, s.regDebugInfo);
  writeSymbolMap(w, s.signalDebugInfo);
  writeSymbolMap(w, s.memDebugInfo);
}

void deserializeSimDebugInfo(std::istream &in, SimDebugInfo &s) {
  std::vector<uint8_t> buf = slurp(in);
  tgs::parseSymbols(buf.data(), buf.size(), s);
}

namespace {
template <typename T>
bool sameBytes(const std::vector<T> &a, const std::vector<T> &b) {
  return a.size() == b.size() && (a.empty() || std::memcmp(a.data(), b.data(), a.size() * sizeof(T)) == 0);
}
template <typename T>
bool samePod(const T &a, const T &b) {
  return std::memcmp(&a, &b, sizeof(T)) == 0;
}
bool sameMPart(const CGMicroPartInfo &a, const CGMicroPartInfo &b) {
  if (a.isLUTPart != b.isLUTPart || a.middleLevels.size() != b.middleLevels.size()) return false;
  for (size_t i = 0; i < a.middleLevels.size(); ++i)
    if (!sameBytes(a.middleLevels[i], b.middleLevels[i])) return false;
  return sameBytes(a.topLevel, b.topLevel) && sameBytes(a.lastLevel, b.lastLevel) && sameBytes(a.vecRead, b.vecRead) &&
         sameBytes(a.vecArithAndLogic, b.vecArithAndLogic) && sameBytes(a.memRead, b.memRead);
}
}  // namespace

// Deep comparison with the same coverage as the reference's
// isSimDesignInfoIdentical (Serializer.cpp:400-443), returning false instead
// of asserting.
bool isSimDesignInfoIdentical(const SimDesignInfo &a, const SimDesignInfo &b) {
  if (a.regPoolSize != b.regPoolSize || a.memPoolSize != b.memPoolSize ||
      a.exchangePoolSize != b.exchangePoolSize || a.shouldStop != b.shouldStop)
    return false;
  if (!sameBytes(a.lut, b.lut) || !sameBytes(a.regPool, b.regPool) || !sameBytes(a.memPool, b.memPool) ||
      a.printMsgs != b.printMsgs || a.parts.size() != b.parts.size())
    return false;
  for (size_t i = 0; i < a.parts.size(); ++i) {
    const auto &p = a.parts[i], &q = b.parts[i];
    if (!sameBytes(p.valuePool, q.valuePool) || p.valuePoolSize != q.valuePoolSize ||
        !sameBytes(p.constVecPool, q.constVecPool) || !sameBytes(p.ops_l0_regRead, q.ops_l0_regRead) ||
        !sameBytes(p.ops_l0_exchangeRead, q.ops_l0_exchangeRead) || p.exec_mParts.size() != q.exec_mParts.size())
      return false;
    for (size_t j = 0; j < p.exec_mParts.size(); ++j) {
      if (p.exec_mParts[j].size() != q.exec_mParts[j].size()) return false;
      for (size_t k = 0; k < p.exec_mParts[j].size(); ++k)
        if (!sameMPart(p.exec_mParts[j][k], q.exec_mParts[j][k])) return false;
    }
    if (!samePod(p.op_last_regWrite, q.op_last_regWrite) || !sameBytes(p.ops_last_memWrite, q.ops_last_memWrite) ||
        !sameBytes(p.ops_last_print, q.ops_last_print) || !sameBytes(p.ops_last_stop, q.ops_last_stop) ||
        !samePod(p.op_last_exchangeWrite, q.op_last_exchangeWrite))
      return false;
  }
  if (a.regionPartitionIds.size() != b.regionPartitionIds.size()) return false;
  for (size_t i = 0; i < a.regionPartitionIds.size(); ++i)
    if (!sameBytes(a.regionPartitionIds[i], b.regionPartitionIds[i])) return false;
  return true;
}

}  // namespace toucanGPUSim
