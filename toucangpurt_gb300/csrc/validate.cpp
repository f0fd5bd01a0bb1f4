// Static design checks.
//
// The reference evaluator trusts its external compiler: it runs the
// micro-partitions of an exec level concurrently with no ordering
// (src/SimEval.cu:824-842), partitions of a region concurrently
// (SimEval.cu:898-918), leaves shared memory uninitialised between
// partitions (SimEval.cu:775-782) and copies registers in whole 32-bit words
// (SimEval.cu:658-665).  A design that reads a slot nobody wrote, or lets two
// micro-partitions of one level touch the same slot, therefore gives
// schedule-dependent results on the reference itself.  These checks accept
// exactly the designs whose values do not depend on the schedule (plus the
// reference runtime's own asserts, SimEval.cu:92-97,1122,1160,1183,1292-1310),
// which is what lets a different schedule stay bit exact.
#include <algorithm>
#include <cstring>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "tgs_internal.h"

namespace tgs {
namespace {

using namespace toucanGPUSim;

[[noreturn]] void fail(uint32_t part, const std::string &what) {
  throw DesignError("partition " + std::to_string(part) + ": " + what);
}

// Reads/writes of one micro-partition, used for the same-level conflict check.
struct Access {
  std::vector<uint32_t> reads, writes;
};

}  // namespace

ValidateInfo validateDesign(const SimDesignInfo &d, const SimDebugInfo *sym) {
  ValidateInfo vi;
  if (d.lut.size() != kLutSize) throw DesignError("lut table must hold exactly 4642 entries (SimEval.cu:1122)");
  for (uint8_t v : d.lut)
    if (v > 15) throw DesignError("lut table entry above 15: values must be nibbles");
  if (d.regionPartitionIds.size() != 2) throw DesignError("exactly two regions are required (SimEval.cu:1292-1295)");
  {
    uint32_t expect = 0;
    for (auto &r : d.regionPartitionIds)
      for (uint32_t id : r)
        if (id != expect++) throw DesignError("region partition ids must be 0..N-1 in order (SimEval.cu:1298-1302)");
    if (expect != d.parts.size()) throw DesignError("regions must cover every partition exactly once");
  }
  if (!d.regPool.empty() && d.regPool.size() != d.regPoolSize) throw DesignError("regPool size mismatch");
  for (uint8_t v : d.regPool)
    if (v > 15) throw DesignError("initial register value above 15");
  for (uint8_t v : d.memPool)
    if (v > 15) throw DesignError("initial memory value above 15");

  const uint64_t regWords = (uint64_t(d.regPoolSize) + 3) / 4, exgWords = (uint64_t(d.exchangePoolSize) + 3) / 4;

  // cross-partition bookkeeping per region
  for (size_t region = 0; region < 2; ++region) {
    std::vector<int32_t> regWriter(regWords, -1), exgWriter(exgWords, -1);
    std::unordered_map<uint64_t, int32_t> memReader, memWriter;
    for (uint32_t pid : d.regionPartitionIds[region]) {
      const SimPartitionInfo &p = d.parts[pid];
      auto claim = [&](std::vector<int32_t> &owner, uint64_t start, uint32_t count, const char *what) {
        if (!count) return;
        uint64_t w0 = start >> 2, w1 = w0 + (count + 3) / 4;
        if (w1 > owner.size()) fail(pid, std::string(what) + " block copy beyond the pool");
        for (uint64_t w = w0; w < w1; ++w) {
          if (owner[w] >= 0 && owner[w] != int32_t(pid))
            fail(pid, std::string(what) + " words also written by partition " + std::to_string(owner[w]) + " in the same region");
          owner[w] = int32_t(pid);
        }
      };
      bool exg = p.op_last_exchangeWrite.count != 0;
      if (exg) {
        const auto op = lastLevelExchangeOp(p);
        claim(exgWriter, op.exchange, op.count, "exchange");
      } else {
        claim(regWriter, p.op_last_regWrite.reg, p.op_last_regWrite.count, "register");
        for (auto &w : p.ops_last_memWrite) {
          auto it = memReader.find(w.memBase);
          if (it != memReader.end() && it->second != int32_t(pid))
            fail(pid, "memory written while partition " + std::to_string(it->second) + " of the same region reads it");
          memWriter[w.memBase] = int32_t(pid);
        }
      }
      for (auto &lvl : p.exec_mParts)
        for (auto &m : lvl)
          for (auto &r : m.memRead) {
            auto it = memWriter.find(r.memBase);
            if (it != memWriter.end() && it->second != int32_t(pid))
              fail(pid, "memory read while partition " + std::to_string(it->second) + " of the same region writes it");
            memReader[r.memBase] = int32_t(pid);
          }
    }
    for (uint32_t pid : d.regionPartitionIds[region]) {
      const SimPartitionInfo &p = d.parts[pid];
      for (auto &r : p.ops_l0_regRead) {
        if (r.reg >= d.regPoolSize) fail(pid, "register read beyond regPool");
        int32_t w = regWriter[r.reg >> 2];
        if (w >= 0 && w != int32_t(pid)) fail(pid, "reads a register written by partition " + std::to_string(w) + " in the same region");
      }
      for (auto &r : p.ops_l0_exchangeRead) {
        if (r.exchange >= d.exchangePoolSize) fail(pid, "exchange read beyond exchangePool");
        int32_t w = exgWriter[r.exchange >> 2];
        if (w >= 0 && w != int32_t(pid)) fail(pid, "reads exchange written by partition " + std::to_string(w) + " in the same region");
      }
    }
  }

  for (uint32_t pid = 0; pid < d.parts.size(); ++pid) {
    const SimPartitionInfo &p = d.parts[pid];
    const uint32_t V = p.valuePoolSize;
    if (V > 65534) fail(pid, "valuePoolSize above 65,534 (ToucanSim.cu:160)");
    vi.maxValuePool = std::max(vi.maxValuePool, V);
    if ((p.ops_l0_regRead.empty()) == (p.ops_l0_exchangeRead.empty()))
      fail(pid, "must read either registers or exchange at level 0 (SimEval.cu:1183)");
    // defStamp[s] = 1 + exec level (0 = L0) at which slot s was last defined; 0 = never
    std::vector<uint32_t> def(V, 0);
    auto slotOk = [&](uint32_t s, const char *what) {
      if (s >= V) fail(pid, std::string(what) + " slot " + std::to_string(s) + " beyond valuePoolSize");
    };
    auto needDef = [&](uint32_t s, uint32_t level, const char *what) {
      slotOk(s, what);
      if (def[s] == 0 || def[s] > level) fail(pid, std::string(what) + " reads slot " + std::to_string(s) + " before it is written");
    };
    for (auto &r : p.ops_l0_regRead) { slotOk(r.result, "L0"); def[r.result] = 1; }
    for (auto &r : p.ops_l0_exchangeRead) {
      if (r.exchange >= d.exchangePoolSize) fail(pid, "exchange read beyond exchangePool");
      slotOk(r.result, "L0");
      def[r.result] = 1;
    }
    vi.l0Ops += p.ops_l0_regRead.size() + p.ops_l0_exchangeRead.size();

    std::vector<uint32_t> writerOf(V, UINT32_MAX);
    for (uint32_t lv = 0; lv < p.exec_mParts.size(); ++lv) {
      const uint32_t here = lv + 2;  // definitions of this level get stamp lv + 2
      std::vector<Access> acc(p.exec_mParts[lv].size());
      for (uint32_t mi = 0; mi < p.exec_mParts[lv].size(); ++mi) {
        const CGMicroPartInfo &m = p.exec_mParts[lv][mi];
        Access &a = acc[mi];
        auto rd = [&](uint32_t s, const char *what) { needDef(s, here - 1, what); a.reads.push_back(s); };
        if (m.isLUTPart) {
          if (m.topLevel.size() > 32 || m.lastLevel.size() > 32) fail(pid, "more than 32 lanes in a level");
          if (m.middleLevels.size() > kMaxMidLevels) fail(pid, "more than 158 middle levels (SimEval.cu:92)");
          for (auto &lvlOps : m.middleLevels)
            if (lvlOps.size() > 32) fail(pid, "more than 32 lanes in a level");
          for (auto &op : m.topLevel) {
            uint32_t mx[3];
            const uint16_t o[3] = {op.op0, op.op1, op.op2};
            for (int k = 0; k < 3; ++k) {
              if (o[k] < 16) {
                mx[k] = o[k];
              } else {
                rd(o[k], "top-level operand");
                mx[k] = 15;
              }
            }
            if (op.lutIndex == 0) {
              ++vi.nopOps;
            } else {
              ++vi.lutOps;
              if (uint32_t(op.lutIndex) + ((mx[0] << 8) | (mx[1] << 4) | mx[2]) >= kLutSize)
                fail(pid, "top-level lut window beyond the 4642-entry table");
            }
          }
          for (auto &lvlOps : m.middleLevels)
            for (auto &op : lvlOps) {
              uint32_t mx[3];
              const uint32_t o[3] = {op.op0(), op.op1(), op.op2()};
              for (int k = 0; k < 3; ++k) {
                if (o[k] < 32) {
                  if (o[k] > 15) fail(pid, "middle-level immediate above 15");
                  mx[k] = o[k];
                } else {
                  mx[k] = 15;
                }
              }
              if (op.lutIndex() == 0) {
                ++vi.nopOps;
              } else {
                ++vi.lutOps;
                if (uint32_t(op.lutIndex()) + ((mx[0] << 8) | (mx[1] << 4) | mx[2]) >= kLutSize)
                  fail(pid, "middle-level lut window beyond the 4642-entry table");
              }
            }
          for (auto &wb : m.lastLevel) {
            if (wb.shuffleId < 32 && wb.shuffleId > 15) fail(pid, "write-back immediate above 15");
            slotOk(wb.result, "write-back");
            a.writes.push_back(wb.result);
          }
        } else {
          if (m.vecRead.size() > 32 || m.vecArithAndLogic.size() > 32 || m.memRead.size() > 32)
            fail(pid, "more than 32 lanes in a special micro-partition");
          if (!m.vecRead.empty()) {
            for (auto &op : m.vecRead) {
              const uint16_t idx[4] = {op.index0, op.index1, op.index2, op.index3};
              for (uint16_t s : idx)
                if (s >= 16) rd(s, "vector-read index");
              if (op.outRangeValue >= 16) rd(op.outRangeValue, "vector-read default");
              if (op.isConstVec) {
                if (uint32_t(op.vecBase) + op.vecLength > p.constVecPool.size()) fail(pid, "const vector beyond constVecPool");
              } else {
                for (uint32_t i = 0; i < op.vecLength; ++i) rd(uint32_t(op.vecBase) + i, "vector-read element");
              }
              slotOk(op.result, "vector-read result");
              a.writes.push_back(op.result);
              ++vi.vecReadOps;
            }
          } else if (!m.vecArithAndLogic.empty()) {
            for (auto &op : m.vecArithAndLogic) {
              if (op.vecLength == 0 || op.vecLength > 31) fail(pid, "vector length outside 1..31 (SimEval.cu:222-228 shifts by 128 at 32)");
              for (int k = 0; k < 2; ++k) {
                bool isConst = (op.isV1V2Const >> (1 - k)) & 1;
                uint32_t base = k ? op.vec2Base : op.vec1Base;
                if (isConst) {
                  if (base + op.vecLength > p.constVecPool.size()) fail(pid, "const vector beyond constVecPool");
                } else {
                  for (uint32_t i = 0; i < op.vecLength; ++i) rd(base + i, "vector operand");
                }
              }
              uint32_t n = op.opName <= VEC_ARITH_MUL ? op.vecLength : 1;
              for (uint32_t i = 0; i < n; ++i) {
                uint32_t s = uint16_t(op.result + i);
                slotOk(s, "vector result");
                a.writes.push_back(s);
              }
              ++vi.vecOps;
            }
          } else {
            for (auto &op : m.memRead) {
              ++vi.memReadOps;
              if (op.en == 0) continue;  // immediate 0: never reads, never writes
              if (op.en >= 16) rd(op.en, "memory-read enable");
              for (uint32_t j = 0; j < 8; ++j) rd(uint32_t(op.addrVec) + j, "memory-read address");
              slotOk(op.result, "memory-read result");
              // a disabled read keeps the slot: it must already hold a value of this cycle
              if (op.en >= 16) needDef(op.result, here - 1, "memory-read result (conditional)");
              a.writes.push_back(op.result);
            }
          }
        }
        // one lane of a micro-partition may not read what another lane writes
        std::sort(a.writes.begin(), a.writes.end());
        if (std::adjacent_find(a.writes.begin(), a.writes.end()) != a.writes.end())
          fail(pid, "two lanes of one micro-partition write the same slot");
        if (!m.isLUTPart)
          for (uint32_t s : a.reads)
            if (std::binary_search(a.writes.begin(), a.writes.end(), s))
              fail(pid, "a special micro-partition reads a slot it writes");
      }
      // same-level conflicts between micro-partitions
      for (uint32_t mi = 0; mi < acc.size(); ++mi)
        for (uint32_t s : acc[mi].writes) {
          if (writerOf[s] != UINT32_MAX && writerOf[s] >> 16 == lv && (writerOf[s] & 0xFFFF) != mi)
            fail(pid, "slot " + std::to_string(s) + " written by two micro-partitions of exec level " + std::to_string(lv));
          writerOf[s] = (lv << 16) | mi;
        }
      for (uint32_t mi = 0; mi < acc.size(); ++mi)
        for (uint32_t s : acc[mi].reads)
          if (writerOf[s] != UINT32_MAX && writerOf[s] >> 16 == lv && (writerOf[s] & 0xFFFF) != mi)
            fail(pid, "slot " + std::to_string(s) + " read and written by different micro-partitions of exec level " + std::to_string(lv));
      for (auto &a : acc)
        for (uint32_t s : a.writes) def[s] = here;
    }

    const uint32_t endLevel = uint32_t(p.exec_mParts.size()) + 1;
    auto copyOk = [&](uint32_t dat, uint32_t count, const char *what) {
      uint32_t from = dat & ~3u, n = (count + 3) / 4 * 4;
      for (uint32_t i = 0; i < n; ++i) needDef(from + i, endLevel, what);
    };
    if (p.op_last_exchangeWrite.count != 0) {
      const auto op = lastLevelExchangeOp(p);
      copyOk(op.dat, op.count, "exchange copy");
    } else {
      if (p.op_last_regWrite.count) copyOk(p.op_last_regWrite.dat, p.op_last_regWrite.count, "register copy");
      for (auto &w : p.ops_last_memWrite) {
        if (w.en >= 16) needDef(w.en, endLevel, "memory-write enable");
        if (w.dat >= 16) needDef(w.dat, endLevel, "memory-write data");
        for (uint32_t j = 0; j < 8; ++j) needDef(uint32_t(w.addrVec) + j, endLevel, "memory-write address");
        ++vi.memWriteOps;
      }
      for (auto &pr : p.ops_last_print) {
        if (pr.en >= 16) needDef(pr.en, endLevel, "print enable");
        if (pr.msg >= d.printMsgs.size()) fail(pid, "print message index beyond printMsgs");
      }
      for (auto &st : p.ops_last_stop)
        if (st.en >= 16) needDef(st.en, endLevel, "stop enable");
    }
  }

  if (sym) {
    for (auto &kv : sym->regDebugInfo)
      for (auto &t : kv.second)
        if (std::get<0>(t) >= d.regPoolSize) throw DesignError("register symbol " + kv.first + " beyond regPool");
    for (auto &kv : sym->memDebugInfo)
      for (auto &t : kv.second)
        if (uint64_t(std::get<0>(t)) + std::get<2>(t) > d.memPoolSize)
          throw DesignError("memory symbol " + kv.first + " beyond memPool");
  }
  return vi;
}

}  // namespace tgs
