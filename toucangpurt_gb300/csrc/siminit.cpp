// Design state initialisation (reference src/SimInit.cpp:16-64).
//
// Init() sizes the register / memory pools (zero filled, existing contents
// kept) and the per-partition value pools.  Randomize(seed) draws a table of
// 1,024 nibbles from std::mt19937(seed) through
// std::uniform_int_distribution<uint8_t>(0, 15) and assigns nibble id i the
// table entry i % 1024 masked to the nibble's bit width, for every register
// and every memory word named in the symbol table.  Using the same standard
// library engine and distribution keeps the initial state identical to the
// reference build on the same toolchain.
#include <array>
#include <random>

#include "ToucanGPUGenDataTypes.h"

namespace toucanGPUSim {

void SimDesignInfo::Init() {
  shouldStop = false;
  regPool.resize(regPoolSize, 0);
  memPool.resize(memPoolSize, 0);
  for (auto &p : parts) p.valuePool.resize(p.valuePoolSize);
}

void SimDesignInfo::Randomize(uint32_t seed, SimDebugInfo &symbols) {
  constexpr size_t kTable = 1024;
  std::mt19937 gen(seed);
  std::uniform_int_distribution<uint8_t> nibble(0, 0xF);
  std::array<uint8_t, kTable> table;
  for (auto &t : table) t = nibble(gen);

  for (const auto &entry : symbols.regDebugInfo) {
    for (const auto &loc : entry.second) {
      uint32_t id = std::get<0>(loc);
      int mask = (1 << std::get<1>(loc)) - 1;
      regPool[id] = uint8_t(table[id % kTable] & mask);
    }
  }
  for (const auto &entry : symbols.memDebugInfo) {
    for (const auto &loc : entry.second) {
      uint32_t start = std::get<0>(loc);
      int mask = (1 << std::get<1>(loc)) - 1;
      uint32_t depth = std::get<2>(loc);
      for (size_t i = 0; i < depth; ++i) {
        size_t idx = size_t(start) + i;
        memPool[idx] = uint8_t(table[idx % kTable] & mask);
      }
    }
  }
}

}  // namespace toucanGPUSim
