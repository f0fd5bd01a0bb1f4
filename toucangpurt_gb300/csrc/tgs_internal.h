// Internal declarations shared by the host-side translation units.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "ToucanGPUGenDataTypes.h"
#include "toucan_gb300.h"

namespace tgs {

// Errors carry the C-ABI status they map to.
struct Error : std::runtime_error {
  int code;
  Error(int c, const std::string &m) : std::runtime_error(m), code(c) {}
};
struct FormatError : Error {
  explicit FormatError(const std::string &m) : Error(TGS_ERR_FORMAT, "design format: " + m) {}
};
struct DesignError : Error {
  explicit DesignError(const std::string &m) : Error(TGS_ERR_INVALID_DESIGN, "invalid design: " + m) {}
};

void parseDesign(const uint8_t *data, size_t n, toucanGPUSim::SimDesignInfo &d);
void parseSymbols(const uint8_t *data, size_t n, toucanGPUSim::SimDebugInfo &s);
std::vector<uint8_t> readFileBytes(const std::string &path);

// Reference evaluator constants (src/SimEval.cu:33-35).
constexpr uint32_t kLutSize = 4642;
constexpr uint32_t kMaxMidLevels = 158;

// Static design checks that make a design's behaviour schedule-independent
// (the reference leaves all of these to its external compiler).  Throws
// DesignError with the first violation.
struct ValidateInfo {
  uint64_t lutOps = 0;     // LUT ops with lutIndex != 0
  uint64_t nopOps = 0;     // moves (lutIndex == 0)
  uint64_t memReadOps = 0, memWriteOps = 0, vecOps = 0, vecReadOps = 0;
  uint64_t l0Ops = 0;
  uint32_t maxValuePool = 0;
};
ValidateInfo validateDesign(const toucanGPUSim::SimDesignInfo &d, const toucanGPUSim::SimDebugInfo *sym);

// The op an exchange-writing partition executes: the reference reads it from
// the start of the partition's last-level block, which holds the register
// write op first when one exists (src/SimEval.cu:741-749, 1249-1257).
inline toucanGPUSim::CGExchangeWriteMetaInfo lastLevelExchangeOp(const toucanGPUSim::SimPartitionInfo &p) {
  if (p.op_last_regWrite.count) return {p.op_last_regWrite.reg, p.op_last_regWrite.dat, p.op_last_regWrite.count};
  return p.op_last_exchangeWrite;
}

void generateDesign(const tgs_gen_config &cfg, toucanGPUSim::SimDesignInfo &d, toucanGPUSim::SimDebugInfo &s,
                    tgs_gen_info *info);

inline uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

void setLastError(const std::string &m);

}  // namespace tgs
