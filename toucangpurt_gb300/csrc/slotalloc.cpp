// Value-pool slot allocation: renumbers the value-pool slots of a partition
// so that slots whose live ranges do not overlap share storage.
//
// The value pool is the per-partition scratch array of SimEval.cu:775-782
// (shared memory, `valuePoolSize` nibbles).  The design file numbers its
// slots once per value; on the GB300 the pool sits in shared memory with one
// 32-bit word per slot and group, so its size bounds how many blocks an SM
// holds.  Renumbering is a pure relabelling: every reader of a value still
// reads the value its writer produced, so results are unchanged.  Rules:
//   * a slot's live range runs from its first access to its last access
//     (times: L0 reads = 0, exec level lv = lv + 1, last level = levels + 1);
//     a renumbered slot is reused only by a slot whose range starts at a
//     strictly later time (the schedule's barrier analysis then orders the
//     reuse across warps);
//   * slots that an op addresses as a run (register / exchange block copy,
//     memory address vectors, vector operands and results) keep their
//     relative order and their position modulo 4 (block copies move whole
//     words from `dat & ~3`);
//   * operand fields below 16 are immediates and stay as they are; every
//     renumbered slot is 16 or above.
#include <algorithm>
#include <numeric>
#include <queue>
#include <set>
#include <vector>

#include "slotalloc.h"
#include "tgs_internal.h"

namespace tgs {

using namespace toucanGPUSim;

namespace {

struct Uses {
  std::vector<int32_t> first, last;  // -1: never accessed
  std::vector<std::pair<uint32_t, uint32_t>> runs;  // [start, end) slots addressed together
  explicit Uses(uint32_t V) : first(V, -1), last(V, -1) {}
  void at(uint32_t s, int32_t t) {
    if (s >= first.size()) return;
    if (first[s] < 0 || t < first[s]) first[s] = t;
    last[s] = std::max(last[s], t);
  }
  void run(uint32_t s, uint32_t n, int32_t t) {
    for (uint32_t i = 0; i < n; ++i) at(s + i, t);
    if (n > 1) runs.push_back({s, s + n});
  }
};

// The executed last-level block copy: (dat, count), count 0 for none.
std::pair<uint32_t, uint32_t> copyOp(const SimPartitionInfo &p) {
  if (p.op_last_exchangeWrite.count != 0) {
    const auto op = lastLevelExchangeOp(p);
    return {op.dat, op.count};
  }
  return {p.op_last_regWrite.dat, p.op_last_regWrite.count};
}

Uses collect(const SimPartitionInfo &p, uint32_t V) {
  Uses u(V);
  for (auto &r : p.ops_l0_regRead) u.at(r.result, 0);
  for (auto &r : p.ops_l0_exchangeRead) u.at(r.result, 0);
  for (uint32_t lv = 0; lv < p.exec_mParts.size(); ++lv) {
    const int32_t t = int32_t(lv) + 1;
    for (const auto &m : p.exec_mParts[lv]) {
      if (m.isLUTPart) {
        for (auto &o : m.topLevel)
          for (uint16_t s : {o.op0, o.op1, o.op2})
            if (s >= 16) u.at(s, t);
        for (auto &w : m.lastLevel) u.at(w.result, t);
      } else if (!m.vecRead.empty()) {
        for (auto &o : m.vecRead) {
          for (uint16_t s : {o.index0, o.index1, o.index2, o.index3, o.outRangeValue})
            if (s >= 16) u.at(s, t);
          if (!o.isConstVec) u.run(o.vecBase, o.vecLength, t);
          u.at(o.result, t);
        }
      } else if (!m.vecArithAndLogic.empty()) {
        for (auto &o : m.vecArithAndLogic) {
          if (!(o.isV1V2Const & 2)) u.run(o.vec1Base, o.vecLength, t);
          if (!(o.isV1V2Const & 1)) u.run(o.vec2Base, o.vecLength, t);
          u.run(o.result, o.opName <= VEC_ARITH_MUL ? o.vecLength : 1, t);
        }
      } else {
        for (auto &o : m.memRead) {
          if (o.en == 0) continue;  // never reads, never writes
          if (o.en >= 16) u.at(o.en, t);
          u.run(o.addrVec, 8, t);
          u.at(o.result, t);
        }
      }
    }
  }
  const int32_t T = int32_t(p.exec_mParts.size()) + 1;
  const auto cp = copyOp(p);
  if (cp.second) u.run(cp.first & ~3u, (cp.second + 3) / 4 * 4, T);
  if (p.op_last_exchangeWrite.count == 0) {
    for (auto &w : p.ops_last_memWrite) {
      for (uint16_t s : {w.en, w.dat})
        if (s >= 16) u.at(s, T);
      u.run(w.addrVec, 8, T);
    }
    for (auto &pr : p.ops_last_print)
      if (pr.en >= 16) u.at(pr.en, T);
    for (auto &st : p.ops_last_stop)
      if (st.en >= 16) u.at(st.en, T);
  }
  return u;
}

}  // namespace

uint32_t planSlots(const SimPartitionInfo &p, std::vector<uint32_t> &newOf, const std::vector<uint32_t> *keep) {
  const uint32_t V = std::max<uint32_t>(p.valuePoolSize, 16);
  Uses u = collect(p, V);
  if (keep)
    for (uint32_t s : *keep) u.at(s, int32_t(p.exec_mParts.size()) + 1);
  // blocks: maximal runs of slots joined by run constraints
  std::vector<uint32_t> joinNext(V + 1, 0);  // slot s and s + 1 in one block
  for (auto &r : u.runs)
    for (uint32_t s = r.first; s + 1 < std::min(r.second, V); ++s) joinNext[s] = 1;
  struct Block {
    uint32_t base, size;
    int32_t start, end;
    bool run;
  };
  std::vector<Block> blocks;
  for (uint32_t s = 0; s < V;) {
    uint32_t e = s;
    while (e + 1 < V && joinNext[e]) ++e;
    Block b{s, e - s + 1, -1, -1, e > s};
    for (uint32_t i = s; i <= e; ++i) {
      if (u.first[i] < 0) continue;
      b.start = b.start < 0 ? u.first[i] : std::min(b.start, u.first[i]);
      b.end = std::max(b.end, u.last[i]);
    }
    if (b.start >= 0) blocks.push_back(b);
    s = e + 1;
  }
  std::vector<uint32_t> order(blocks.size());
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) {
    if (blocks[a].start != blocks[b].start) return blocks[a].start < blocks[b].start;
    return blocks[a].size > blocks[b].size;
  });
  // allocation: first fit over new slots 16.., singles from a free set
  std::vector<uint8_t> used;
  std::set<uint32_t> freeSingles;  // free positions below the high-water mark
  uint32_t hwm = 16;
  auto occupy = [&](uint32_t pos, uint32_t n) {
    if (used.size() < pos + n) used.resize(pos + n, 0);
    for (uint32_t i = pos; i < pos + n; ++i) {
      used[i] = 1;
      freeSingles.erase(i);
    }
    for (uint32_t i = hwm; i < pos; ++i)
      if (!used[i]) freeSingles.insert(i);
    hwm = std::max(hwm, pos + n);
  };
  using E = std::pair<int32_t, uint32_t>;  // (end, block)
  std::priority_queue<E, std::vector<E>, std::greater<E>> live;
  std::vector<uint32_t> at(blocks.size(), 0);
  for (uint32_t bi : order) {
    const Block &b = blocks[bi];
    while (!live.empty() && live.top().first < b.start) {
      const uint32_t x = live.top().second;
      live.pop();
      for (uint32_t i = at[x]; i < at[x] + blocks[x].size; ++i) {
        used[i] = 0;
        freeSingles.insert(i);
      }
    }
    uint32_t pos;
    if (!b.run) {
      pos = freeSingles.empty() ? hwm : *freeSingles.begin();
    } else {
      pos = 16 + ((b.base - 16) & 3u);  // same position modulo 4
      for (;; pos += 4) {
        bool ok = true;
        for (uint32_t i = pos; i < pos + b.size && ok; ++i) ok = i >= used.size() || !used[i];
        if (ok) break;
      }
    }
    occupy(pos, b.size);
    at[bi] = pos;
    live.push({b.end, bi});
  }
  newOf.assign(V, kNoSlot);
  uint32_t top = 16;
  for (uint32_t bi = 0; bi < blocks.size(); ++bi) {
    for (uint32_t i = 0; i < blocks[bi].size; ++i) newOf[blocks[bi].base + i] = at[bi] + i;
    top = std::max(top, at[bi] + blocks[bi].size);
  }
  return top;
}

void renameSlots(SimPartitionInfo &p, const std::vector<uint32_t> &newOf, uint32_t newSize) {
  // slot fields (any value) and operand fields (values below 16 are immediates)
  auto slot = [&](auto &f) {
    if (f < newOf.size() && newOf[f] != kNoSlot) f = static_cast<std::remove_reference_t<decltype(f)>>(newOf[f]);
  };
  auto operand = [&](auto &f) {
    if (f >= 16) slot(f);
  };
  for (auto &r : p.ops_l0_regRead) slot(r.result);
  for (auto &r : p.ops_l0_exchangeRead) slot(r.result);
  for (auto &lvl : p.exec_mParts)
    for (auto &m : lvl) {
      for (auto &o : m.topLevel) {
        operand(o.op0);
        operand(o.op1);
        operand(o.op2);
      }
      for (auto &w : m.lastLevel) slot(w.result);
      for (auto &o : m.vecRead) {
        operand(o.index0);
        operand(o.index1);
        operand(o.index2);
        operand(o.index3);
        operand(o.outRangeValue);
        if (!o.isConstVec) slot(o.vecBase);
        slot(o.result);
      }
      for (auto &o : m.vecArithAndLogic) {
        if (!(o.isV1V2Const & 2)) slot(o.vec1Base);
        if (!(o.isV1V2Const & 1)) slot(o.vec2Base);
        slot(o.result);
      }
      for (auto &o : m.memRead) {
        if (o.en == 0) continue;
        operand(o.en);
        slot(o.addrVec);
        slot(o.result);
      }
    }
  // block copies: the run starts at dat & ~3 and keeps its position modulo 4
  auto copyDat = [&](uint16_t &dat) {
    const uint32_t from = dat & ~3u;
    if (from < newOf.size() && newOf[from] != kNoSlot) dat = uint16_t(newOf[from] + (dat & 3u));
  };
  copyDat(p.op_last_regWrite.dat);
  copyDat(p.op_last_exchangeWrite.dat);
  for (auto &w : p.ops_last_memWrite) {
    operand(w.en);
    operand(w.dat);
    slot(w.addrVec);
  }
  for (auto &pr : p.ops_last_print) operand(pr.en);
  for (auto &st : p.ops_last_stop) operand(st.en);
  p.valuePoolSize = newSize;
  p.valuePool.assign(newSize, 0);
}

}  // namespace tgs
