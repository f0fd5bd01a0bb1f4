// CPU oracle for the Toucan per-cycle netlist evaluation.
//
// TEST INFRASTRUCTURE ONLY (see toucan_oracle.h): the checker for the GPU
// path and the timed CPU baseline, never part of the product.
//
// Parity status: the design-file parser and Init/Randomize are pinned against
// the reference's own Serializer.cpp / SimInit.cpp compiled from source
// (oracle/ref_tool.cpp); the evaluator is pinned against the reference's own
// GPU kernel (src/SimEval.cu compiled to a cubin and driven by
// oracle/refgpu_harness.cpp) through the committed fixtures in tests/golden.
//
// Every function names the reference lines it restates.
#include "toucan_oracle.h"

#include <array>
#include <atomic>
#include <barrier>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <iterator>
#include <mutex>
#include <algorithm>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <tuple>
#include <vector>

namespace {

struct Err : std::runtime_error {
  using std::runtime_error::runtime_error;
};

// ---------------------------------------------------------------- parsing --
// Field offsets follow the struct layouts of include/ToucanGPUGenDataTypes.h
// (reference lines 18-211); each record is decoded from its raw bytes.
struct Cursor {
  const uint8_t *p;
  size_t n, off = 0;
  const uint8_t *take(size_t k) {
    if (k > n - off) throw Err("truncated file");
    const uint8_t *r = p + off;
    off += k;
    return r;
  }
  template <typename T>
  T get() {
    T v;
    std::memcpy(&v, take(sizeof(T)), sizeof(T));
    return v;
  }
  uint64_t cnt(size_t elem) {
    uint64_t c = get<uint64_t>();
    if (elem && c > (n - off) / elem) throw Err("count beyond file end");
    return c;
  }
};

template <typename T>
T rd(const uint8_t *p, size_t o) {
  T v;
  std::memcpy(&v, p + o, sizeof(T));
  return v;
}

struct Top { uint16_t lut, a, b, c; };
struct WB { uint8_t src; uint16_t res; };
struct VRead { uint16_t base, len, off; bool isConst; uint16_t idx[4]; uint16_t outRange, res; };
struct VOp { uint16_t v1, v2, len; uint8_t op, cflags; uint16_t res; };
struct MRead { bool multi; uint64_t base; uint16_t en, addr, res; };
struct MWrite { bool multi; uint64_t base; uint16_t addr, dat, en; };
struct Copy { uint32_t dst; uint16_t dat, count; };

struct MPart {
  bool isLUT = false;
  std::vector<Top> top;
  std::vector<std::vector<uint32_t>> mid;
  std::vector<WB> wb;
  std::vector<VRead> vr;
  std::vector<VOp> vo;
  std::vector<MRead> mr;
};

struct Part {
  uint32_t vpSize = 0;
  std::vector<uint8_t> constVec;
  std::vector<std::pair<uint32_t, uint16_t>> regRead, exgRead;
  std::vector<std::vector<MPart>> levels;
  Copy regWrite{}, exgWrite{};
  std::vector<MWrite> memW;
  std::vector<std::pair<uint16_t, uint16_t>> print;
  std::vector<uint16_t> stop;
};

}  // namespace

struct orc_design {
  uint32_t regSize = 0, memSize = 0, exgSize = 0;
  std::vector<uint8_t> lut, regInit, memInit;
  std::vector<Part> parts;
  std::vector<std::vector<uint32_t>> regions;
  std::vector<std::string> msgs;
  uint64_t lutOps = 0;
};

namespace {

template <typename F>
void forVec(Cursor &c, size_t elem, F f) {
  uint64_t k = c.cnt(elem);
  for (uint64_t i = 0; i < k; ++i) f(c.take(elem));
}

MPart parseMPart(Cursor &c) {
  MPart m;
  m.isLUT = c.get<uint8_t>() != 0;
  if (m.isLUT) {
    forVec(c, 8, [&](const uint8_t *p) { m.top.push_back({rd<uint16_t>(p, 0), rd<uint16_t>(p, 2), rd<uint16_t>(p, 4), rd<uint16_t>(p, 6)}); });
    uint64_t nMid = c.cnt(8);
    for (uint64_t l = 0; l < nMid; ++l) {
      std::vector<uint32_t> lvl;
      forVec(c, 4, [&](const uint8_t *p) { lvl.push_back(rd<uint32_t>(p, 0)); });
      m.mid.push_back(std::move(lvl));
    }
    forVec(c, 4, [&](const uint8_t *p) { m.wb.push_back({p[0], rd<uint16_t>(p, 2)}); });
  } else {
    forVec(c, 20, [&](const uint8_t *p) {
      VRead v;
      v.base = rd<uint16_t>(p, 0); v.len = rd<uint16_t>(p, 2); v.off = rd<uint16_t>(p, 4);
      v.isConst = p[6] != 0;
      for (int k = 0; k < 4; ++k) v.idx[k] = rd<uint16_t>(p, 8 + 2 * k);
      v.outRange = rd<uint16_t>(p, 16); v.res = rd<uint16_t>(p, 18);
      m.vr.push_back(v);
    });
    forVec(c, 10, [&](const uint8_t *p) {
      m.vo.push_back({rd<uint16_t>(p, 0), rd<uint16_t>(p, 2), rd<uint16_t>(p, 4), p[6], p[7], rd<uint16_t>(p, 8)});
    });
    forVec(c, 24, [&](const uint8_t *p) {
      m.mr.push_back({p[0] != 0, rd<uint64_t>(p, 8), rd<uint16_t>(p, 16), rd<uint16_t>(p, 18), rd<uint16_t>(p, 20)});
    });
  }
  return m;
}

Part parsePart(Cursor &c) {
  Part p;
  forVec(c, 1, [](const uint8_t *) {});  // valuePool contents are never read by the kernel (SimEval.cu:778-782)
  p.vpSize = c.get<uint32_t>();
  forVec(c, 1, [&](const uint8_t *q) { p.constVec.push_back(q[0]); });
  forVec(c, 8, [&](const uint8_t *q) { p.regRead.push_back({rd<uint32_t>(q, 0), rd<uint16_t>(q, 4)}); });
  forVec(c, 8, [&](const uint8_t *q) { p.exgRead.push_back({rd<uint32_t>(q, 0), rd<uint16_t>(q, 4)}); });
  uint64_t nLevels = c.cnt(8);
  for (uint64_t l = 0; l < nLevels; ++l) {
    uint64_t k = c.cnt(1);
    std::vector<MPart> lvl;
    for (uint64_t i = 0; i < k; ++i) lvl.push_back(parseMPart(c));
    p.levels.push_back(std::move(lvl));
  }
  const uint8_t *q = c.take(8);
  p.regWrite = {rd<uint32_t>(q, 0), rd<uint16_t>(q, 4), rd<uint16_t>(q, 6)};
  forVec(c, 24, [&](const uint8_t *r) {
    p.memW.push_back({r[0] != 0, rd<uint64_t>(r, 8), rd<uint16_t>(r, 16), rd<uint16_t>(r, 18), rd<uint16_t>(r, 20)});
  });
  forVec(c, 4, [&](const uint8_t *r) { p.print.push_back({rd<uint16_t>(r, 0), rd<uint16_t>(r, 2)}); });
  forVec(c, 2, [&](const uint8_t *r) { p.stop.push_back(rd<uint16_t>(r, 0)); });
  q = c.take(8);
  p.exgWrite = {rd<uint32_t>(q, 0), rd<uint16_t>(q, 4), rd<uint16_t>(q, 6)};
  return p;
}

std::vector<uint8_t> readFile(const char *path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Err(std::string("cannot open ") + path);
  return std::vector<uint8_t>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

// Init() + Randomize(seed 0) restated from SimInit.cpp:16-64 and the symbol
// file grammar of Serializer.cpp:264-300.
void initState(orc_design &d, const std::vector<uint8_t> &regVec, const std::vector<uint8_t> &memVec,
               const std::vector<uint8_t> &sym, bool randomize) {
  d.regInit = regVec;
  d.regInit.resize(d.regSize, 0);
  d.memInit = memVec;
  d.memInit.resize(d.memSize, 0);
  if (!randomize) return;
  std::mt19937 gen(0);
  std::uniform_int_distribution<uint8_t> dist(0, 15);
  std::array<uint8_t, 1024> tbl;
  for (auto &t : tbl) t = dist(gen);
  Cursor c{sym.data(), sym.size()};
  for (int map = 0; map < 3; ++map) {
    uint64_t n = c.cnt(16);
    for (uint64_t i = 0; i < n; ++i) {
      uint64_t sl = c.cnt(1);
      c.take(sl);
      int arity = map == 0 ? 2 : 3;
      uint64_t k = c.cnt(4 * arity);
      for (uint64_t j = 0; j < k; ++j) {
        uint32_t f0 = c.get<uint32_t>(), f1 = c.get<uint32_t>(), f2 = arity == 3 ? c.get<uint32_t>() : 0;
        int mask = (1 << f1) - 1;
        if (map == 0) {
          if (f0 >= d.regSize) throw Err("register symbol beyond regPool");
          d.regInit[f0] = uint8_t(tbl[f0 % 1024] & mask);
        } else if (map == 2) {
          if (uint64_t(f0) + f2 > d.memSize) throw Err("memory symbol beyond memPool");
          for (uint64_t e = 0; e < f2; ++e) d.memInit[f0 + e] = uint8_t(tbl[(f0 + e) % 1024] & mask);
        }
      }
    }
  }
}

// ------------------------------------------------------------- evaluation --
inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

uint64_t digestPool(const uint8_t *p, size_t n) {
  uint64_t s = 0;
  for (size_t i = 0; i < n; ++i) s += mix64((uint64_t(i) << 8) | p[i]);
  return s;
}

struct StreamState {
  std::vector<uint8_t> regs, mems, exg;
  bool stop = false;
};

struct EvalCtx {
  const orc_design *d;
  std::vector<uint8_t> vp;  // stale between partitions, like a block's shared memory
  std::string *err;
  // signal probes: per partition (slot, probe index); values after the exec levels
  const std::vector<std::vector<std::pair<uint32_t, uint32_t>>> *probes = nullptr;
  std::vector<uint8_t> *probeValues = nullptr;
};

// Signed 128-bit sign extension at bit `pos` (SimEval.cu:222-228).
inline __int128 signExtend(__int128 v, unsigned pos) {
  if (!((v >> pos) & 1)) return v;
  __int128 mask = (__int128(1) << (pos + 1)) - 1;
  return v | ~mask;
}

inline uint8_t lutAt(const orc_design &d, uint32_t pos) {
  if (pos >= d.lut.size()) throw Err("lut index beyond table");
  return d.lut[pos];
}

// evalSingleMicroPart, SimEval.cu:304-580.  Lanes of one level run in lock
// step: every lane reads before any lane of the mPart writes.
void evalMPart(EvalCtx &cx, const Part &p, const MPart &m, StreamState &st) {
  const orc_design &d = *cx.d;
  uint8_t *vp = cx.vp.data();
  if (m.isLUT) {
    uint8_t lane[32] = {0};
    // top level (SimEval.cu:337-362): operands < 16 are immediates
    for (size_t l = 0; l < m.top.size() && l < 32; ++l) {
      const Top &o = m.top[l];
      uint32_t a = o.a < 16 ? o.a : vp[o.a], b = o.b < 16 ? o.b : vp[o.b], c = o.c < 16 ? o.c : vp[o.c];
      lane[l] = o.lut == 0 ? uint8_t(c) : lutAt(d, uint16_t(o.lut + ((a << 8) | (b << 4) | c)));
    }
    // middle levels (SimEval.cu:365-420): operands < 32 immediate, else lane op & 31
    for (const auto &lvl : m.mid) {
      uint8_t next[32];
      for (uint32_t l = 0; l < 32; ++l) {
        uint32_t w = l < lvl.size() ? lvl[l] : 0u;
        uint32_t c = w & 63, b = (w >> 6) & 63, a = (w >> 12) & 63, lut = w >> 18;
        uint32_t av = a < 32 ? a : lane[a & 31], bv = b < 32 ? b : lane[b & 31], cv = c < 32 ? c : lane[c & 31];
        next[l] = lut == 0 ? uint8_t(cv) : lutAt(d, uint16_t(lut + ((av << 8) | (bv << 4) | cv)));
      }
      std::memcpy(lane, next, 32);
    }
    // write-back (SimEval.cu:423-447): shuffleId < 32 is an immediate
    uint8_t val[32];
    for (size_t l = 0; l < m.wb.size() && l < 32; ++l) {
      uint32_t s = m.wb[l].src;
      val[l] = s < 32 ? uint8_t(s) : lane[s & 31];
    }
    for (size_t l = 0; l < m.wb.size() && l < 32; ++l) vp[m.wb[l].res] = val[l];
    return;
  }
  if (!m.vr.empty()) {  // VecRead, SimEval.cu:449-480
    std::vector<std::pair<uint16_t, uint8_t>> out;
    for (size_t l = 0; l < m.vr.size() && l < 32; ++l) {
      const VRead &o = m.vr[l];
      uint32_t iv[4];
      for (int k = 0; k < 4; ++k) iv[k] = o.idx[k] < 16 ? o.idx[k] : vp[o.idx[k]];
      uint32_t off = ((iv[0] << 12) | (iv[1] << 8) | (iv[2] << 4) | iv[3]) + o.off;
      uint8_t r;
      if (off < o.len) {
        uint32_t at = uint32_t(o.base) + off;
        if (o.isConst) {
          if (at >= p.constVec.size()) throw Err("constVecPool read out of range");
          r = p.constVec[at];
        } else {
          r = vp[at];
        }
      } else {
        r = o.outRange < 16 ? uint8_t(o.outRange) : vp[o.outRange];
      }
      out.push_back({o.res, r});
    }
    for (auto &w : out) vp[w.first] = w.second;
    return;
  }
  if (!m.vo.empty()) {  // VecArithOrLogic, SimEval.cu:482-548
    struct W { uint16_t res; uint16_t len; bool vec; unsigned __int128 v; uint8_t bit; };
    std::vector<W> out;
    for (size_t l = 0; l < m.vo.size() && l < 32; ++l) {
      const VOp &o = m.vo[l];
      bool c1 = (o.cflags & 2) != 0, c2 = (o.cflags & 1) != 0;
      unsigned __int128 u1 = 0, u2 = 0;
      for (uint32_t i = 0; i < o.len; ++i) {
        uint32_t i1 = uint32_t(o.v1) + i, i2 = uint32_t(o.v2) + i;
        if ((c1 && i1 >= p.constVec.size()) || (c2 && i2 >= p.constVec.size())) throw Err("constVecPool read out of range");
        unsigned __int128 s1 = c1 ? p.constVec[i1] : vp[i1];
        unsigned __int128 s2 = c2 ? p.constVec[i2] : vp[i2];
        u1 |= s1 << (4 * i);
        u2 |= s2 << (4 * i);
      }
      if (o.len == 0 || o.len > 31) throw Err("vecLength outside 1..31");
      __int128 a = signExtend(__int128(u1), 4u * o.len - 1), b = signExtend(__int128(u2), 4u * o.len - 1);
      W w{o.res, o.len, false, 0, 0};
      switch (o.op) {
        case 0: w.vec = true; w.v = (unsigned __int128)a + (unsigned __int128)b; break;
        case 1: w.vec = true; w.v = (unsigned __int128)a - (unsigned __int128)b; break;
        case 2: w.vec = true; w.v = (unsigned __int128)a * (unsigned __int128)b; break;
        case 3: w.bit = a == b; break;
        case 4: w.bit = a < b; break;
        case 5: w.bit = a <= b; break;
        default: w.bit = 0; break;
      }
      out.push_back(w);
    }
    for (auto &w : out) {
      if (w.vec) {
        unsigned __int128 v = w.v;
        for (uint32_t i = 0; i < w.len; ++i, v >>= 4) vp[uint16_t(w.res + i)] = uint8_t(v & 0xF);
      } else {
        vp[w.res] = w.bit;
      }
    }
    return;
  }
  // MemRead, SimEval.cu:550-575: en == 0 leaves the slot untouched
  std::vector<std::pair<uint16_t, uint8_t>> out;
  for (size_t l = 0; l < m.mr.size() && l < 32; ++l) {
    const MRead &o = m.mr[l];
    uint32_t en = o.en < 16 ? o.en : vp[o.en];
    if (!en) continue;
    uint32_t addr = 0;
    for (uint32_t j = 0; j < 8; ++j) addr |= uint32_t(vp[o.addr + j]) << (4 * j);
    if (o.multi) addr <<= 2;
    uint64_t at = o.base + addr;
    if (at >= st.mems.size()) throw Err("memory read address beyond memPool");
    out.push_back({o.res, st.mems[at]});
  }
  for (auto &w : out) vp[w.first] = w.second;
}

// Word copy of (count+3)/4 32-bit words from slot (dat & ~3) to (dst & ~3)
// (SimEval.cu:658-665, 751-758).
void wordCopy(const uint8_t *vp, uint32_t dat, uint32_t count, std::vector<uint8_t> &pool, uint32_t dst) {
  uint32_t words = (count + 3) / 4;
  size_t from = size_t(dat >> 2) * 4, to = size_t(dst >> 2) * 4, bytes = size_t(words) * 4;
  if (to + bytes > ((pool.size() + 3) & ~size_t(3))) throw Err("block copy beyond pool");
  for (size_t i = 0; i < bytes; ++i)
    if (to + i < pool.size()) pool[to + i] = vp[from + i];
}

// evalEachPartition, SimEval.cu:765-864.
void evalPartition(EvalCtx &cx, uint32_t pid, StreamState &st, uint32_t cycle, uint32_t *stopCycle,
                   std::vector<std::string> *printed, bool enablePrint) {
  const orc_design &d = *cx.d;
  const Part &p = d.parts[pid];
  uint8_t *vp = cx.vp.data();
  for (auto &r : p.regRead) {  // evalPartL0RegRead, :582-601
    if (r.first >= st.regs.size()) throw Err("register read beyond regPool");
    vp[r.second] = st.regs[r.first];
  }
  for (auto &r : p.exgRead) {  // evalPartL0ExgRead, :603-622
    if (r.first >= st.exg.size()) throw Err("exchange read beyond exchangePool");
    vp[r.second] = st.exg[r.first];
  }
  for (auto &lvl : p.levels)
    for (auto &m : lvl) evalMPart(cx, p, m, st);
  if (cx.probes && pid < cx.probes->size())  // value-pool slots the symbol file names as signals
    for (auto &pr : (*cx.probes)[pid]) (*cx.probeValues)[pr.second] = vp[pr.first];

  if (p.exgWrite.count != 0) {
    // evalLastLevelExgWrite, :732-761.  The op is read from the start of the
    // last-level block, which holds the reg-write op first when one exists
    // (copy_netlist_to_gpu, :1249-1257).
    const Copy &op = p.regWrite.count != 0 ? p.regWrite : p.exgWrite;
    wordCopy(vp, op.dat, op.count, st.exg, op.dst);
    return;
  }
  // evalLastLevel, :625-729
  if (p.regWrite.count != 0) wordCopy(vp, p.regWrite.dat, p.regWrite.count, st.regs, p.regWrite.dst);
  for (auto &o : p.memW) {
    uint32_t en = o.en < 16 ? o.en : vp[o.en];
    if (!en) continue;
    uint8_t dat = o.dat < 16 ? uint8_t(o.dat) : vp[o.dat];
    uint32_t addr = 0;
    for (uint32_t j = 0; j < 8; ++j) addr |= uint32_t(vp[o.addr + j]) << (4 * j);
    if (o.multi) addr <<= 2;
    uint64_t at = o.base + addr;
    if (at >= st.mems.size()) throw Err("memory write address beyond memPool");
    st.mems[at] = dat;
  }
  if (enablePrint && printed) {
    for (auto &o : p.print) {
      uint32_t en = o.first < 16 ? o.first : vp[o.first];
      if (en && o.second < d.msgs.size()) printed->push_back(d.msgs[o.second]);
    }
  }
  for (auto &o : p.stop) {
    uint32_t en = o < 16 ? o : vp[o];
    if (en) {
      if (!st.stop && stopCycle) *stopCycle = cycle;
      st.stop = true;
    }
  }
}

// One cycle: region 0 then region 1 (evalFreeRunningNCycles, :889-995).
void evalCycle(EvalCtx &cx, StreamState &st, uint32_t cycle, uint32_t *stopCycle) {
  for (auto &region : cx.d->regions)
    for (uint32_t pid : region) evalPartition(cx, pid, st, cycle, stopCycle, nullptr, false);
}

void applyStimulus(const orc_stimulus *stim, uint64_t streamSeed, uint32_t cycle, StreamState &st) {
  if (!stim) return;
  for (uint32_t i = 0; i < stim->n_inputs; ++i) {
    uint64_t h = mix64(streamSeed ^ mix64((uint64_t(cycle) << 32) | i));
    uint8_t mask = uint8_t((1u << stim->bits[i]) - 1);
    uint32_t id = stim->reg[i];
    if (id >= st.regs.size()) throw Err("stimulus register beyond regPool");
    uint16_t t = stim->toggle ? stim->toggle[i] : 0;
    if (t == 0)
      st.regs[id] = uint8_t(h & mask);
    else if ((h >> 48) < t)
      st.regs[id] ^= mask;
  }
}

void setErr(char *err, size_t len, const std::string &m) {
  if (err && len) std::snprintf(err, len, "%s", m.c_str());
}

}  // namespace

struct orc_state {
  const orc_design *d;
  StreamState st;
  EvalCtx cx;
  std::vector<std::vector<std::pair<uint32_t, uint32_t>>> probes;
  std::vector<uint8_t> probeValues;
};

extern "C" {

uint64_t orc_mix64(uint64_t x) { return mix64(x); }
uint64_t orc_digest(const uint8_t *pool, size_t n) { return digestPool(pool, n); }

orc_design *orc_load(const char *design_path, const char *symbol_path, int randomize, char *err, size_t errlen) {
  try {
    auto buf = readFile(design_path);
    auto sym = symbol_path ? readFile(symbol_path) : std::vector<uint8_t>(24, 0);
    auto *d = new orc_design();
    try {
      Cursor c{buf.data(), buf.size()};
      d->regSize = c.get<uint32_t>();
      d->memSize = c.get<uint32_t>();
      d->exgSize = c.get<uint32_t>();
      c.get<uint8_t>();
      std::vector<uint8_t> regVec, memVec;
      forVec(c, 1, [&](const uint8_t *q) { d->lut.push_back(q[0]); });
      forVec(c, 1, [&](const uint8_t *q) { regVec.push_back(q[0]); });
      forVec(c, 1, [&](const uint8_t *q) { memVec.push_back(q[0]); });
      uint64_t np = c.cnt(8);
      for (uint64_t i = 0; i < np; ++i) d->parts.push_back(parsePart(c));
      uint64_t nr = c.cnt(8);
      for (uint64_t i = 0; i < nr; ++i) {
        std::vector<uint32_t> ids;
        forVec(c, 4, [&](const uint8_t *q) { ids.push_back(rd<uint32_t>(q, 0)); });
        for (uint32_t id : ids)
          if (id >= d->parts.size()) throw Err("region names an unknown partition");
        d->regions.push_back(std::move(ids));
      }
      uint64_t nm = c.cnt(8);
      for (uint64_t i = 0; i < nm; ++i) {
        uint64_t k = c.cnt(1);
        const uint8_t *q = c.take(k);
        d->msgs.emplace_back(reinterpret_cast<const char *>(q), k);
      }
      initState(*d, regVec, memVec, sym, randomize != 0);
      for (auto &p : d->parts)
        for (auto &lvl : p.levels)
          for (auto &m : lvl) {
            for (auto &t : m.top) d->lutOps += t.lut != 0;
            for (auto &l : m.mid)
              for (uint32_t w : l) d->lutOps += (w >> 18) != 0;
          }
    } catch (...) {
      delete d;
      throw;
    }
    return d;
  } catch (const std::exception &e) {
    setErr(err, errlen, e.what());
    return nullptr;
  }
}

void orc_free(orc_design *d) { delete d; }
uint32_t orc_reg_pool_size(const orc_design *d) { return d->regSize; }
uint32_t orc_mem_pool_size(const orc_design *d) { return d->memSize; }
uint32_t orc_num_parts(const orc_design *d) { return uint32_t(d->parts.size()); }
uint64_t orc_num_lut_ops(const orc_design *d) { return d->lutOps; }
const uint8_t *orc_initial_regs(const orc_design *d) { return d->regInit.data(); }
const uint8_t *orc_initial_mems(const orc_design *d) { return d->memInit.data(); }

int orc_run(const orc_design *d, uint32_t n_streams, const uint32_t *cycles, const orc_stimulus *stim,
            orc_result *res, int threads, char *err, size_t errlen) {
  if (threads <= 0) threads = int(std::max(1u, std::thread::hardware_concurrency()));
  std::atomic<uint32_t> next{0};
  std::atomic<bool> failed{false};
  std::string firstErr;
  std::mutex errMu;
  auto worker = [&]() {
    EvalCtx cx{d, std::vector<uint8_t>(65536 + 64, 0), nullptr};
    StreamState st;
    for (;;) {
      uint32_t s = next.fetch_add(1);
      if (s >= n_streams || failed.load()) return;
      try {
        st.regs = d->regInit;
        st.mems = d->memInit;
        st.exg.assign(d->exgSize, 0);
        st.stop = false;
        uint64_t seed = mix64((stim ? stim->base_seed : 0) ^ s);
        uint64_t roll = 0;
        uint32_t stopC = 0xFFFFFFFFu;
        for (uint32_t c = 0; c < cycles[s]; ++c) {
          applyStimulus(stim, seed, c, st);
          if (res && (res->rolling_digest || res->cycle_digest)) {
            uint64_t dg = digestPool(st.regs.data(), st.regs.size());
            roll = mix64(roll + dg);
            if (res->cycle_digest && c < res->cycle_stride) res->cycle_digest[size_t(s) * res->cycle_stride + c] = dg;
          }
          evalCycle(cx, st, c, &stopC);
        }
        if (res) {
          if (res->final_reg_digest) res->final_reg_digest[s] = digestPool(st.regs.data(), st.regs.size());
          if (res->final_mem_digest) res->final_mem_digest[s] = digestPool(st.mems.data(), st.mems.size());
          if (res->rolling_digest) res->rolling_digest[s] = roll;
          if (res->stop_cycle) res->stop_cycle[s] = stopC;
          if (res->final_regs) std::memcpy(res->final_regs + size_t(s) * d->regSize, st.regs.data(), d->regSize);
          if (res->final_mems) std::memcpy(res->final_mems + size_t(s) * d->memSize, st.mems.data(), d->memSize);
        }
      } catch (const std::exception &e) {
        std::lock_guard<std::mutex> g(errMu);
        if (!failed.exchange(true)) firstErr = e.what();
        return;
      }
    }
  };
  int nt = std::min<int>(threads, int(std::max<uint32_t>(1, n_streams)));
  if (nt == 1 && n_streams == 1 && threads > 1 && d->parts.size() > 1) {
    // one stream, many partitions: partitions of a region in parallel, a
    // barrier between regions (the CPU analogue of the grid barrier)
    StreamState st;
    st.regs = d->regInit;
    st.mems = d->memInit;
    st.exg.assign(d->exgSize, 0);
    uint64_t seed = mix64((stim ? stim->base_seed : 0) ^ 0);
    uint64_t roll = 0;
    uint32_t stopC = 0xFFFFFFFFu;
    std::vector<uint32_t> stopPer(threads, 0xFFFFFFFFu);
    std::atomic<uint32_t> cursor{0};
    std::barrier bar(threads);
    std::vector<std::thread> pool;
    int T = threads;
    for (int t = 0; t < T; ++t) {
      pool.emplace_back([&, t]() {
        EvalCtx cx{d, std::vector<uint8_t>(65536 + 64, 0), nullptr};
        for (uint32_t c = 0; c < cycles[0]; ++c) {
          if (t == 0) {
            try {
              applyStimulus(stim, seed, c, st);
              if (res && (res->rolling_digest || res->cycle_digest)) {
                uint64_t dg = digestPool(st.regs.data(), st.regs.size());
                roll = mix64(roll + dg);
                if (res->cycle_digest && c < res->cycle_stride) res->cycle_digest[c] = dg;
              }
            } catch (const std::exception &e) {
              std::lock_guard<std::mutex> g(errMu);
              if (!failed.exchange(true)) firstErr = e.what();
            }
          }
          for (auto &region : d->regions) {
            if (t == 0) cursor.store(0);
            bar.arrive_and_wait();
            for (;;) {
              uint32_t k = cursor.fetch_add(1);
              if (k >= region.size() || failed.load()) break;
              try {
                evalPartition(cx, region[k], st, c, &stopPer[t], nullptr, false);
              } catch (const std::exception &e) {
                std::lock_guard<std::mutex> g(errMu);
                if (!failed.exchange(true)) firstErr = e.what();
              }
            }
            bar.arrive_and_wait();
          }
        }
      });
    }
    for (auto &th : pool) th.join();
    for (uint32_t s : stopPer) stopC = std::min(stopC, s);
    if (!failed && res) {
      if (res->final_reg_digest) res->final_reg_digest[0] = digestPool(st.regs.data(), st.regs.size());
      if (res->final_mem_digest) res->final_mem_digest[0] = digestPool(st.mems.data(), st.mems.size());
      if (res->rolling_digest) res->rolling_digest[0] = roll;
      if (res->stop_cycle) res->stop_cycle[0] = stopC;
      if (res->final_regs) std::memcpy(res->final_regs, st.regs.data(), d->regSize);
      if (res->final_mems) std::memcpy(res->final_mems, st.mems.data(), d->memSize);
    }
  } else {
    std::vector<std::thread> pool;
    for (int t = 0; t < nt; ++t) pool.emplace_back(worker);
    for (auto &th : pool) th.join();
  }
  if (failed) {
    setErr(err, errlen, firstErr);
    return -1;
  }
  return 0;
}

orc_state *orc_state_new(const orc_design *d) {
  auto *s = new orc_state{d, {}, {d, std::vector<uint8_t>(65536 + 64, 0), nullptr}, {}, {}};
  s->st.regs = d->regInit;
  s->st.mems = d->memInit;
  s->st.exg.assign(d->exgSize, 0);
  return s;
}
void orc_state_free(orc_state *s) { delete s; }

// Probes: value-pool slot `slots[i]` of partition `parts[i]` is recorded after
// that partition's exec levels in every evaluated cycle (the value a signal of
// the symbol file names); orc_state_probe_values returns the last cycle's.
int orc_state_set_probes(orc_state *s, const uint32_t *parts, const uint32_t *slots, uint32_t n) {
  s->probes.assign(s->d->parts.size(), {});
  for (uint32_t i = 0; i < n; ++i) {
    if (parts[i] >= s->d->parts.size() || slots[i] >= 65536) return -1;
    s->probes[parts[i]].push_back({slots[i], i});
  }
  s->probeValues.assign(n, 0);
  s->cx.probes = &s->probes;
  s->cx.probeValues = &s->probeValues;
  return 0;
}
const uint8_t *orc_state_probe_values(const orc_state *s) { return s->probeValues.data(); }
uint8_t *orc_state_regs(orc_state *s) { return s->st.regs.data(); }
uint8_t *orc_state_mems(orc_state *s) { return s->st.mems.data(); }

int orc_state_eval(orc_state *s, uint32_t cycles, int *stop, char *err, size_t errlen) {
  try {
    for (uint32_t c = 0; c < cycles; ++c) evalCycle(s->cx, s->st, c, nullptr);
    if (stop) *stop = s->st.stop ? 1 : 0;
    return 0;
  } catch (const std::exception &e) {
    setErr(err, errlen, e.what());
    return -1;
  }
}

}  // extern "C"
