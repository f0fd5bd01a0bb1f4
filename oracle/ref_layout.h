// The reference's device netlist layout, restated field by field.
//
// TEST INFRASTRUCTURE ONLY.  copy_netlist_to_gpu / copyMicroPartToNetlist
// (src/SimEval.cu:69-148,1114-1343) flatten a SimDesignInfo into device
// buffers and __device__ globals that the reference kernels read.
// refgpu_harness.cpp lays a design out this way on the GPU to drive the
// reference's own cubin; layout_dump.cpp lays it out in host memory and
// prints the canonical form (layout_canon.h) that ref_layout_main.cpp prints
// for the reference's own host code, so the restatement is checked against
// the original on the CPU.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <vector>

#include "ToucanGPUGenDataTypes.h"

namespace reflayout {

using namespace toucanGPUSim;

// Device structs of the reference (src/SimEval.cu:152-187), pointer fields as
// 64-bit device addresses.
struct RefPartPtrs {
  uint64_t valuePool;
  uint16_t valuePoolSize;
  uint64_t constVecPool;
  uint64_t netlist;
  uint64_t lastLevelNetlistPtr;
  uint32_t numOpsL0RegRead;
  uint32_t numOpsL0ExgRead;
  uint32_t numExecLevels;
  uint64_t execMPartLevelInfo;
  uint32_t numOpsLastExgWrite;
  uint32_t numOpsLastRegWrite;
  uint32_t numOpsLastMemWrite;
  uint32_t numOpsLastPrint;
  uint32_t numOpsLastStop;
};
static_assert(sizeof(RefPartPtrs) == 88 && offsetof(RefPartPtrs, netlist) == 24 &&
                  offsetof(RefPartPtrs, execMPartLevelInfo) == 56 && offsetof(RefPartPtrs, numOpsLastStop) == 80,
              "SimPartitionPtrs layout");
struct RefLevelInfo {
  uint32_t numMParts;
  uint64_t mPartInfo;
};
static_assert(sizeof(RefLevelInfo) == 16, "SimMPartLevelInfo layout");
struct RefMPartPtr {
  uint32_t netlistOffset, netlistSize;
};

constexpr uint32_t kMagicLut = 0xfb709394u, kMagicVecRead = 0xfb809917u, kMagicMemRead = 0xccccccccu,
                   kMagicVecOp = 0xbeef1234u;
constexpr size_t kMaxLevels = 160, kLutSize = 4642;

template <typename T>
inline void appendRaw(std::vector<char> &b, const std::vector<T> &v) {
  const char *d = reinterpret_cast<const char *>(v.data());
  b.insert(b.end(), d, d + v.size() * sizeof(T));
}
inline void appendU32(std::vector<char> &b, uint32_t v) {
  const char *d = reinterpret_cast<const char *>(&v);
  b.insert(b.end(), d, d + 4);
}
// chunk padded to 16 bytes (appendToNetlistVec, SimEval.cu:1148-1154)
inline void appendPadded(std::vector<char> &net, const char *d, size_t n) {
  net.insert(net.end(), d, d + n);
  for (size_t i = 0; i < (16 - n % 16) % 16; ++i) net.push_back(0);
}

// copyMicroPartToNetlist (SimEval.cu:69-148)
inline std::vector<char> mpartBytes(const CGMicroPartInfo &m) {
  std::vector<char> b;
  if (m.isLUTPart) {
    appendU32(b, kMagicLut);
    appendU32(b, uint32_t(m.middleLevels.size()));
    std::vector<char> sizes(kMaxLevels, 0);
    sizes[0] = char(m.topLevel.size());
    for (size_t i = 0; i < m.middleLevels.size(); ++i) sizes[1 + i] = char(m.middleLevels[i].size());
    sizes[1 + m.middleLevels.size()] = char(m.lastLevel.size());
    b.insert(b.end(), sizes.begin(), sizes.end());
    appendRaw(b, m.topLevel);
    for (auto &l : m.middleLevels) appendRaw(b, l);
    appendRaw(b, m.lastLevel);
  } else if (!m.vecRead.empty()) {
    appendU32(b, kMagicVecRead);
    appendU32(b, uint32_t(m.vecRead.size()));
    appendRaw(b, m.vecRead);
  } else if (!m.vecArithAndLogic.empty()) {
    appendU32(b, kMagicVecOp);
    appendU32(b, uint32_t(m.vecArithAndLogic.size()));
    appendRaw(b, m.vecArithAndLogic);
  } else {
    appendU32(b, kMagicMemRead);
    appendU32(b, uint32_t(m.memRead.size()));
    appendRaw(b, m.memRead);
  }
  return b;
}

// Where the layout goes: device buffers and named __device__ globals.
struct Sink {
  virtual ~Sink() = default;
  virtual uint64_t upload(const void *d, size_t n) = 0;  // a buffer holding the n bytes; its address
  virtual void setGlobal(const char *name, const void *d, size_t n) = 0;
};

// What the caller needs afterwards: the state pools and the launch inputs.
struct Layout {
  uint64_t reg = 0, mem = 0, exg = 0;
  size_t maxVp = 0;
  uint32_t n0 = 0, n1 = 0;
};

// copy_netlist_to_gpu (SimEval.cu:1114-1343) for an initialised design.
inline Layout build(const SimDesignInfo &d, Sink &s) {
  Layout L;
  if (d.lut.size() != kLutSize) throw std::runtime_error("lut size");
  const uint32_t zero32 = 0;
  s.setGlobal("shouldStop", &zero32, 4);
  s.setGlobal("realCycles", &zero32, 4);
  s.setGlobal("lutContent", d.lut.data(), kLutSize);
  L.reg = s.upload(d.regPool.data(), d.regPoolSize);
  L.mem = s.upload(d.memPool.data(), d.memPoolSize);
  std::vector<uint8_t> zeros(d.exchangePoolSize, 0);
  L.exg = s.upload(zeros.data(), zeros.size());
  s.setGlobal("regPool", &L.reg, 8);
  s.setGlobal("memPool", &L.mem, 8);
  s.setGlobal("exchangePool", &L.exg, 8);

  std::vector<RefPartPtrs> parts;
  for (const auto &p : d.parts) {
    RefPartPtrs pp;
    std::memset(&pp, 0, sizeof pp);
    std::vector<char> net;
    pp.valuePool = s.upload(p.valuePool.data(), p.valuePoolSize);
    pp.valuePoolSize = uint16_t(p.valuePoolSize);
    L.maxVp = std::max<size_t>(L.maxVp, p.valuePoolSize);
    pp.constVecPool = p.constVecPool.empty() ? 0 : s.upload(p.constVecPool.data(), p.constVecPool.size());
    pp.numOpsL0RegRead = uint32_t(p.ops_l0_regRead.size());
    if (pp.numOpsL0RegRead)
      appendPadded(net, reinterpret_cast<const char *>(p.ops_l0_regRead.data()), p.ops_l0_regRead.size() * 8);
    pp.numOpsL0ExgRead = uint32_t(p.ops_l0_exchangeRead.size());
    if (pp.numOpsL0ExgRead)
      appendPadded(net, reinterpret_cast<const char *>(p.ops_l0_exchangeRead.data()), p.ops_l0_exchangeRead.size() * 8);
    std::vector<RefLevelInfo> levels;
    for (const auto &lvl : p.exec_mParts) {
      std::vector<RefMPartPtr> ptrs;
      for (const auto &m : lvl) {
        auto b = mpartBytes(m);
        ptrs.push_back({uint32_t(net.size()), uint32_t(b.size())});
        appendPadded(net, b.data(), b.size());
      }
      RefLevelInfo li;
      std::memset(&li, 0, sizeof li);
      li.numMParts = uint32_t(ptrs.size());
      li.mPartInfo = ptrs.empty() ? 0 : s.upload(ptrs.data(), ptrs.size() * sizeof(RefMPartPtr));
      levels.push_back(li);
    }
    pp.numExecLevels = uint32_t(levels.size());
    pp.execMPartLevelInfo = levels.empty() ? 0 : s.upload(levels.data(), levels.size() * sizeof(RefLevelInfo));
    pp.numOpsLastRegWrite = p.op_last_regWrite.count != 0;
    pp.numOpsLastExgWrite = p.op_last_exchangeWrite.count != 0;
    pp.numOpsLastMemWrite = uint32_t(p.ops_last_memWrite.size());
    pp.numOpsLastPrint = uint32_t(p.ops_last_print.size());
    pp.numOpsLastStop = uint32_t(p.ops_last_stop.size());
    size_t lastOff = net.size();
    if (pp.numOpsLastRegWrite) appendPadded(net, reinterpret_cast<const char *>(&p.op_last_regWrite), 8);
    if (pp.numOpsLastExgWrite) appendPadded(net, reinterpret_cast<const char *>(&p.op_last_exchangeWrite), 8);
    if (pp.numOpsLastMemWrite)
      appendPadded(net, reinterpret_cast<const char *>(p.ops_last_memWrite.data()), p.ops_last_memWrite.size() * 24);
    if (pp.numOpsLastPrint)
      appendPadded(net, reinterpret_cast<const char *>(p.ops_last_print.data()), p.ops_last_print.size() * 4);
    if (pp.numOpsLastStop)
      appendPadded(net, reinterpret_cast<const char *>(p.ops_last_stop.data()), p.ops_last_stop.size() * 2);
    pp.netlist = s.upload(net.data(), net.size());
    pp.lastLevelNetlistPtr = pp.netlist + lastOff;
    parts.push_back(pp);
  }
  const uint64_t partsDev = s.upload(parts.data(), parts.size() * sizeof(RefPartPtrs));
  s.setGlobal("partitions", &partsDev, 8);
  if (d.regionPartitionIds.size() != 2) throw std::runtime_error("exactly two regions required");
  L.n0 = uint32_t(d.regionPartitionIds[0].size());
  L.n1 = uint32_t(d.regionPartitionIds[1].size());
  const uint32_t nt = uint32_t(d.parts.size());
  s.setGlobal("numParts_Region0", &L.n0, 4);
  s.setGlobal("numParts_Region1", &L.n1, 4);
  s.setGlobal("numTotalParts", &nt, 4);
  std::vector<uint64_t> msgPtrs;
  for (auto &m : d.printMsgs) msgPtrs.push_back(s.upload(m.c_str(), m.size() + 1));
  const uint64_t msgsDev = s.upload(msgPtrs.data(), msgPtrs.size() * 8);
  s.setGlobal("printMsgs", &msgsDev, 8);
  return L;
}

}  // namespace reflayout
