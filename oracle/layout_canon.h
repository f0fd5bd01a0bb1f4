// Canonical text form of a reference device netlist layout.
//
// TEST INFRASTRUCTURE ONLY.  The layout is read the way the reference
// kernels read it (src/SimEval.cu:152-215: the __device__ globals, the
// SimPartitionPtrs array, each partition's level table and micro-partition
// pointer tables, the print messages) and printed with buffer sizes, 64-bit
// digests of their bytes and every scalar field, but no addresses, so two
// layouts of one design built by different host code compare as text.
#pragma once

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

namespace reflayout {

// The buffer holding a device address: its bytes and the address's offset.
struct Found {
  const uint8_t *p = nullptr;
  size_t n = 0, off = 0;
};
using Resolve = std::function<bool(uint64_t addr, Found &f)>;
using Global = std::function<bool(const char *name, std::vector<uint8_t> &bytes)>;

inline uint64_t canonMix(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
inline uint64_t canonDigest(const uint8_t *p, size_t n) {
  uint64_t s = 0;
  for (size_t i = 0; i < n; ++i) s += canonMix((uint64_t(i) << 8) | p[i]);
  return s;
}

template <typename T>
inline T canonRead(const uint8_t *p, size_t off) {
  T v;
  std::memcpy(&v, p + off, sizeof v);
  return v;
}

inline std::string canonical(const Resolve &resolve, const Global &global) {
  std::string out;
  char line[256];
  auto put = [&](const char *fmt, auto... a) {
    std::snprintf(line, sizeof line, fmt, a...);
    out += line;
  };
  // n bytes at addr (n = 0: to the end of its buffer); "empty" for a null
  // address or no bytes, "bad" for an address outside every buffer
  auto buffer = [&](uint64_t addr, size_t n, std::vector<uint8_t> *copy) -> std::string {
    if (addr == 0) return "empty";
    Found f;
    if (!resolve(addr, f) || f.off > f.n) return "bad";
    const size_t avail = f.n - f.off;
    if (n == 0) n = avail;
    if (n > avail) return "short";
    if (copy) copy->assign(f.p + f.off, f.p + f.off + n);
    if (n == 0) return "empty";
    char b[64];
    std::snprintf(b, sizeof b, "%zu:%016llx", n, (unsigned long long)canonDigest(f.p + f.off, n));
    return b;
  };
  auto u32global = [&](const char *name) -> uint32_t {
    std::vector<uint8_t> g;
    if (!global(name, g) || g.size() < 4) return 0xFFFFFFFFu;
    return canonRead<uint32_t>(g.data(), 0);
  };
  auto ptrGlobal = [&](const char *name) -> uint64_t {
    std::vector<uint8_t> g;
    if (!global(name, g) || g.size() < 8) return 0;
    return canonRead<uint64_t>(g.data(), 0);
  };

  {
    std::vector<uint8_t> lut;
    if (global("lutContent", lut))
      put("lutContent %zu:%016llx\n", lut.size(), (unsigned long long)canonDigest(lut.data(), lut.size()));
    else
      out += "lutContent missing\n";
  }
  for (const char *g : {"regPool", "memPool", "exchangePool"}) out += std::string(g) + " " + buffer(ptrGlobal(g), 0, nullptr) + "\n";
  const uint32_t n0 = u32global("numParts_Region0"), n1 = u32global("numParts_Region1"), nt = u32global("numTotalParts");
  put("numParts %u %u %u\n", n0, n1, nt);
  put("shouldStop %u realCycles %u\n", u32global("shouldStop"), u32global("realCycles"));

  std::vector<uint8_t> parts;
  const std::string pb = buffer(ptrGlobal("partitions"), size_t(nt) * 88, &parts);
  out += "partitions " + std::string(parts.size() == size_t(nt) * 88 ? "ok" : pb) + "\n";
  for (uint32_t i = 0; parts.size() == size_t(nt) * 88 && i < nt; ++i) {
    const uint8_t *q = parts.data() + size_t(i) * 88;
    const uint16_t vpSize = canonRead<uint16_t>(q, 8);
    const uint64_t net = canonRead<uint64_t>(q, 24), last = canonRead<uint64_t>(q, 32);
    const uint32_t nLv = canonRead<uint32_t>(q, 48);
    put("part %u vp %s size %u\n", i, buffer(canonRead<uint64_t>(q, 0), vpSize, nullptr).c_str(), unsigned(vpSize));
    out += "  constVec " + buffer(canonRead<uint64_t>(q, 16), 0, nullptr) + "\n";
    out += "  netlist " + buffer(net, 0, nullptr) + "\n";
    put("  last %lld\n", (long long)(last - net));
    put("  l0 %u %u levels %u last-ops %u %u %u %u %u\n", canonRead<uint32_t>(q, 40), canonRead<uint32_t>(q, 44), nLv,
        canonRead<uint32_t>(q, 64), canonRead<uint32_t>(q, 68), canonRead<uint32_t>(q, 72), canonRead<uint32_t>(q, 76),
        canonRead<uint32_t>(q, 80));
    std::vector<uint8_t> lv;
    const std::string lb = buffer(canonRead<uint64_t>(q, 56), size_t(nLv) * 16, &lv);
    if (nLv && lv.size() != size_t(nLv) * 16) {
      out += "  levels " + lb + "\n";
      continue;
    }
    for (uint32_t j = 0; j < nLv; ++j) {
      const uint32_t nm = canonRead<uint32_t>(lv.data(), size_t(j) * 16);
      put("  level %u mparts %u %s\n", j, nm,
          buffer(canonRead<uint64_t>(lv.data(), size_t(j) * 16 + 8), size_t(nm) * 8, nullptr).c_str());
    }
  }
  std::vector<uint8_t> msgs;
  const uint64_t msgAddr = ptrGlobal("printMsgs");
  buffer(msgAddr, 0, &msgs);
  put("printMsgs %zu\n", msgs.size() / 8);
  for (size_t k = 0; k + 8 <= msgs.size(); k += 8) {
    Found f;
    const uint64_t a = canonRead<uint64_t>(msgs.data(), k);
    if (!resolve(a, f)) {
      out += "  msg bad\n";
      continue;
    }
    std::string s;
    for (size_t i = f.off; i < f.n && f.p[i]; ++i) s += char(f.p[i]);
    out += "  msg " + s + "\n";
  }
  return out;
}

}  // namespace reflayout
