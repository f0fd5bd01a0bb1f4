// Design-file data model of the Toucan GPU RTL simulator.
//
// These PODs ARE the on-disk format: the design file stores each op vector as
// raw struct bytes (padding included), so every struct below keeps the field
// order, types and therefore the exact size/offsets of the reference
// definitions in include/ToucanGPUGenDataTypes.h:18-282 (ucsc-vama/toucanGPURT).
// The static_asserts at the end pin the x86-64 / aarch64 layouts.
#pragma once

#include <cassert>
#include <cstddef>
#include <cstdint>
#include <fstream>
#include <string>
#include <tuple>
#include <unordered_map>
#include <vector>

#ifdef __CUDACC__
#define TGS_HD __host__ __device__
#else
#define TGS_HD
#endif

namespace toucanGPUSim {

// ---- level 0 (partition inputs) -------------------------------------------
struct CGRegReadMetaInfo {       // regPool[reg] -> valuePool[result]
  uint32_t reg;
  uint16_t result;
};
struct CGExchangeReadMetaInfo {  // exchangePool[exchange] -> valuePool[result]
  uint32_t exchange;
  uint16_t result;
};
struct CGExchangeWriteMetaInfo { // word copy valuePool[dat..] -> exchangePool[exchange..]
  uint32_t exchange;
  uint16_t dat;
  uint16_t count;
};

// ---- last level (partition outputs) ---------------------------------------
struct CGPrintMetaInfo {
  uint16_t en;
  uint16_t msg;
};
struct CGStopMetaInfo {
  uint16_t en;
};
struct CGRegWriteMetaInfo {      // word copy valuePool[dat..] -> regPool[reg..]
  uint32_t reg;
  uint16_t dat;
  uint16_t count;
};
struct CGMemWriteMetaInfo {
  bool hasMultipleWriter;        // index = memBase + (addr << 2) when set
  uint64_t memBase;
  uint16_t addrVec;              // 8 consecutive slots, least significant nibble first
  uint16_t dat;
  uint16_t en;
};

// ---- micro-partition (one warp) ops ---------------------------------------
struct CGMicroPartLUTTopLevelOp {
  uint16_t lutIndex;             // 0 = move op2
  uint16_t op0;                  // < 16: immediate nibble, else valuePool slot
  uint16_t op1;
  uint16_t op2;
};

// Middle-level op packed into one 32-bit word:
//   bits 31..18 lutIndex (14 b) | 17..12 op0 | 11..6 op1 | 5..0 op2
// operand < 32 is an immediate, 32..63 selects lane (operand - 32) of the
// previous level.
#pragma pack(push, 1)
struct CGMicroPartLUTMiddleLevelOp {
 private:
  uint32_t packed_data;

 public:
  TGS_HD CGMicroPartLUTMiddleLevelOp() : packed_data(0) {}
  TGS_HD explicit CGMicroPartLUTMiddleLevelOp(uint16_t lut, uint8_t a, uint8_t b, uint8_t c)
      : packed_data((uint32_t(lut & 0x3FFFu) << 18) | (uint32_t(a & 0x3Fu) << 12) |
                    (uint32_t(b & 0x3Fu) << 6) | uint32_t(c & 0x3Fu)) {}

  TGS_HD uint16_t lutIndex() const { return uint16_t(packed_data >> 18); }
  TGS_HD uint8_t op0() const { return uint8_t((packed_data >> 12) & 0x3Fu); }
  TGS_HD uint8_t op1() const { return uint8_t((packed_data >> 6) & 0x3Fu); }
  TGS_HD uint8_t op2() const { return uint8_t(packed_data & 0x3Fu); }

  TGS_HD void setLutIndex(uint16_t v) { packed_data = (packed_data & 0x0003FFFFu) | (uint32_t(v & 0x3FFFu) << 18); }
  TGS_HD void setOp0(uint8_t v) { packed_data = (packed_data & ~(0x3Fu << 12)) | (uint32_t(v & 0x3Fu) << 12); }
  TGS_HD void setOp1(uint8_t v) { packed_data = (packed_data & ~(0x3Fu << 6)) | (uint32_t(v & 0x3Fu) << 6); }
  TGS_HD void setOp2(uint8_t v) { packed_data = (packed_data & ~0x3Fu) | uint32_t(v & 0x3Fu); }

  TGS_HD uint32_t getPacked() const { return packed_data; }
  TGS_HD void setPacked(uint32_t v) { packed_data = v; }
};
#pragma pack(pop)

struct CGMicroPartLUTLastLevelWriteBack {
  uint8_t shuffleId;             // < 32: immediate, else lane (shuffleId mod 32)
  uint16_t result;
};

struct CGMicroPartVecRead {
  uint16_t vecBase;
  uint16_t vecLength;
  uint16_t offset;
  bool isConstVec;
  uint16_t index0;               // index nibbles, most significant first
  uint16_t index1;
  uint16_t index2;
  uint16_t index3;
  uint16_t outRangeValue;
  uint16_t result;
};

#define VEC_ARITH_ADD 0
#define VEC_ARITH_SUB 1
#define VEC_ARITH_MUL 2
#define VEC_LOGIC_EQ 3
#define VEC_LOGIC_LT 4
#define VEC_LOGIC_LE 5

struct CGMicroPartVecArithOrLogic {
  uint16_t vec1Base;
  uint16_t vec2Base;
  uint16_t vecLength;            // nibbles, least significant at the base slot
  uint8_t opName;
  uint8_t isV1V2Const;           // bit1: vec1 from constVecPool, bit0: vec2
  uint16_t result;
};

struct CGMicroPartMemRead {
  bool hasMultipleWriter;
  uint64_t memBase;
  uint16_t en;
  uint16_t addrVec;
  uint16_t result;
};

struct CGMicroPartInfo {
  bool isLUTPart;
  std::vector<CGMicroPartLUTTopLevelOp> topLevel;
  std::vector<std::vector<CGMicroPartLUTMiddleLevelOp>> middleLevels;
  std::vector<CGMicroPartLUTLastLevelWriteBack> lastLevel;
  std::vector<CGMicroPartVecRead> vecRead;
  std::vector<CGMicroPartVecArithOrLogic> vecArithAndLogic;
  std::vector<CGMicroPartMemRead> memRead;
};

struct SimDebugInfo {
  // register name -> (regPool nibble id, bit width) per nibble, most significant first
  std::unordered_map<std::string, std::vector<std::tuple<uint32_t, uint32_t>>> regDebugInfo;
  // signal name -> (partition, valuePool slot, bit width) per nibble
  std::unordered_map<std::string, std::vector<std::tuple<uint32_t, uint32_t, uint32_t>>> signalDebugInfo;
  // memory name -> (memPool start, bit width, depth) per nibble memory
  std::unordered_map<std::string, std::vector<std::tuple<uint32_t, uint32_t, uint32_t>>> memDebugInfo;
};

struct SimPartitionInfo {
  std::vector<uint8_t> valuePool;
  uint32_t valuePoolSize;
  std::vector<uint8_t> constVecPool;
  std::vector<CGRegReadMetaInfo> ops_l0_regRead;
  std::vector<CGExchangeReadMetaInfo> ops_l0_exchangeRead;
  std::vector<std::vector<CGMicroPartInfo>> exec_mParts;
  CGRegWriteMetaInfo op_last_regWrite;
  std::vector<CGMemWriteMetaInfo> ops_last_memWrite;
  std::vector<CGPrintMetaInfo> ops_last_print;
  std::vector<CGStopMetaInfo> ops_last_stop;
  CGExchangeWriteMetaInfo op_last_exchangeWrite;
};

struct SimDesignInfo {
  std::vector<uint8_t> lut;
  std::vector<uint8_t> regPool;
  std::vector<uint8_t> memPool;
  uint32_t regPoolSize;
  uint32_t memPoolSize;
  uint32_t exchangePoolSize;
  std::vector<SimPartitionInfo> parts;
  std::vector<std::vector<uint32_t>> regionPartitionIds;
  bool shouldStop;
  std::vector<std::string> printMsgs;

  void Init();
  void Randomize(uint32_t seed, SimDebugInfo &symbols);
};

void serializeSimDesignInfo(std::ostream &out, const SimDesignInfo &info);
void deserializeSimDesignInfo(std::istream &in, SimDesignInfo &info);
void serializeSimDebugInfo(std::ostream &out, const SimDebugInfo &info);
void deserializeSimDebugInfo(std::istream &in, SimDebugInfo &info);
bool isSimDesignInfoIdentical(const SimDesignInfo &a, const SimDesignInfo &b);

// ---- layout pins (the file format depends on them) -------------------------
static_assert(sizeof(CGRegReadMetaInfo) == 8, "format");
static_assert(sizeof(CGExchangeReadMetaInfo) == 8, "format");
static_assert(sizeof(CGExchangeWriteMetaInfo) == 8, "format");
static_assert(sizeof(CGPrintMetaInfo) == 4, "format");
static_assert(sizeof(CGStopMetaInfo) == 2, "format");
static_assert(sizeof(CGRegWriteMetaInfo) == 8, "format");
static_assert(sizeof(CGMemWriteMetaInfo) == 24 && offsetof(CGMemWriteMetaInfo, memBase) == 8 &&
                  offsetof(CGMemWriteMetaInfo, addrVec) == 16 && offsetof(CGMemWriteMetaInfo, dat) == 18 &&
                  offsetof(CGMemWriteMetaInfo, en) == 20,
              "format");
static_assert(sizeof(CGMicroPartLUTTopLevelOp) == 8, "format");
static_assert(sizeof(CGMicroPartLUTMiddleLevelOp) == 4, "format");
static_assert(sizeof(CGMicroPartLUTLastLevelWriteBack) == 4 &&
                  offsetof(CGMicroPartLUTLastLevelWriteBack, result) == 2,
              "format");
static_assert(sizeof(CGMicroPartVecRead) == 20 && offsetof(CGMicroPartVecRead, isConstVec) == 6 &&
                  offsetof(CGMicroPartVecRead, index0) == 8 && offsetof(CGMicroPartVecRead, outRangeValue) == 16 &&
                  offsetof(CGMicroPartVecRead, result) == 18,
              "format");
static_assert(sizeof(CGMicroPartVecArithOrLogic) == 10 && offsetof(CGMicroPartVecArithOrLogic, opName) == 6 &&
                  offsetof(CGMicroPartVecArithOrLogic, isV1V2Const) == 7 &&
                  offsetof(CGMicroPartVecArithOrLogic, result) == 8,
              "format");
static_assert(sizeof(CGMicroPartMemRead) == 24 && offsetof(CGMicroPartMemRead, memBase) == 8 &&
                  offsetof(CGMicroPartMemRead, en) == 16 && offsetof(CGMicroPartMemRead, addrVec) == 18 &&
                  offsetof(CGMicroPartMemRead, result) == 20,
              "format");

}  // namespace toucanGPUSim
