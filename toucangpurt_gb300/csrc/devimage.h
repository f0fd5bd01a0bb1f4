// Device image of a design: the GB300 layout the cycle kernel executes.
//
// It replaces the reference's per-partition pointer tables
// (SimPartitionPtrs / SimMPartLevelInfo / SimMicroPartNetlistHeader,
// src/SimEval.cu:61-65,152-187) with one 16-byte aligned word array per
// design, offsets instead of pointers, lane-major op words (lane l of a warp
// loads word l of every level, one 128-byte transaction per warp), and a
// static warp schedule per exec level in place of the shared-memory atomic
// work queue (SimEval.cu:818-843).
//
// Values: every value-pool slot, register and exchange entry is one 32-bit
// word holding the nibbles of 8 streams (stream k of a group in bits
// 4k..4k+3).  The reference stores one stream, one nibble per byte.
#pragma once
#include <vector_types.h>

#include <cstdint>

namespace tgs {

// Micro-partition kinds (first header word, bits 0..1).
enum : uint32_t { kMPLut = 0, kMPVecRead = 1, kMPVecOp = 2, kMPMemRead = 3 };

// Header word: kind | lanes(6) << 2 | nMid(8) << 8 | nWB(6) << 16 | nTop(6) << 24
// | direct write-back << 30 (LUT: write-back entry l takes lane l's result,
// shuffleId == 32 + l for every entry, so no lane exchange is needed)
// | fast top level << 31 (every top-level op has a word-wide form: its lut
// field holds the fast code of emit.h, not a table offset) | some fast op is
// a multiplexer << 23 | compact lanes << 22 (see below).
// LUT micro-partition words after the 4-word header (all lane-major):
//   top:  2 * W words, lane l: [lutIndex | op0 << 16, op1 | op2 << 16] (zero for idle lanes)
//   mid:  nMid * W words, the reference's packed middle-level op (zero = move of immediate 0)
//   wb :  W words, lane l: shuffleId | result << 16
// A compact record (no middle levels, write-back entry l = lane l for every
// lane, all slots below 4096) holds one word pair per lane and no wb block:
//   lane l: [op0 | op1 << 12 | (op2 & 255) << 24, op2 >> 8 | result << 4 | lut field << 16]
// Special micro-partitions: header, then per lane fixed-size records:
//   VecRead (5 words): vecBase | vecLength << 16, offset | isConst << 16,
//                      idx0 | idx1 << 16, idx2 | idx3 << 16, outRange | result << 16
//   VecOp   (3 words): vec1 | vec2 << 16, vecLength | opName << 16 | isV1V2Const << 24, result
//   MemRead (4 words): memBase lo, memBase hi | multiWriter << 31, en | addrVec << 16, result
constexpr uint32_t kMPHeaderWords = 4;
constexpr uint32_t kMPDirectWB = 1u << 30;
constexpr uint32_t kMPFastTop = 1u << 31, kMPFastSel = 1u << 23, kMPCompact = 1u << 22;
// Top-level words of a word-wide ("fast") op, in a record with kMPFastTop:
//   lut field: lutIndex | kind << kFastKindShift | kFastOp
//   kind 0: out = g(b, c) bit by bit (bit (x << 1 | y) of g = g(b bit x,
//           c bit y)); op0 field = op0 (an immediate) | g << 4
//   kind 1: out = a ? b : c, kind 2: out = a ? c : b, for select nibbles 0
//           and 1 (a word with another select value reads the table)
// so the table form (lutIndex, op0 & 15 for kind 0) stays available: single
// streams (one stream per word) evaluate every op by lookup.  A move is kind
// 0 with g = kGPassC; idle lanes have zero words (g = 0, out = 0).
constexpr uint32_t kFastOp = 0x8000u, kFastKindShift = 13;
constexpr uint32_t kGPassC = 0xAu, kGPassB = 0xCu;  // g of "c" and of "b"
constexpr uint32_t kVecReadWords = 5, kVecOpWords = 3, kMemReadWords = 4;
// schedule unit word: record offset (words from the level block) | first
// group << 24 | (groups - 1) << 27
constexpr uint32_t kUnitOffsetMask = (1u << 24) - 1u;

struct PartDesc {
  uint32_t vpSlots;      // value-pool slots (multiple of 4)
  uint32_t l0Count;      // L0 reads
  uint32_t l0Off;        // word offset: src[l0Count], then dst packed two per word
  uint32_t l0Exchange;   // 1: L0 reads the exchange pool, 0: registers
  uint32_t nLevels;      // exec levels
  uint32_t schedOff;     // word offset of the warp schedule (see below)
  uint32_t copyKind;     // 0 none, 1 register pool, 2 exchange pool
  uint32_t copySrc;      // first source slot (dat & ~3)
  uint32_t copyDst;      // first destination entry (reg/exchange & ~3)
  uint32_t copySlots;    // 4 * ((count + 3) / 4)
  uint32_t memWCount, memWOff;   // 4 words per op: memBase lo, hi | multi << 31, addrVec | dat << 16, en
  uint32_t printCount, printOff; // 1 word per op: en | msg << 16
  uint32_t stopCount, stopOff;   // 1 word per op: en
  uint32_t constOff, constLen;   // byte offset / length in the const-vector byte array
  uint32_t region;
  uint32_t probeCount, probeOff;  // signal probes: 2 words per probe (slot, probe index)
  uint32_t pad[3];
};
static_assert(sizeof(PartDesc) == 96, "PartDesc size");

// Exec levels (KParams::sched), for NW warps: one 16-byte aligned block per
// partition level, [flags (bit0: block barrier)][NW + 1 prefix offsets into
// the unit list][unit list: unit words (kUnitOffsetMask), each a record
// offset relative to the block and a range of stream groups][micro-partition
// records, once each, in warp order].  KParams::levelDesc
// holds (block offset, block words) per level; PartDesc::schedOff indexes
// the partition's first level there.  A block is staged into shared memory
// with one bulk async copy while the previous level computes, or, when the
// levels of every partition a block evaluates fit in its shared memory, they
// are copied there once per launch and stay resident (a partition's level
// blocks are contiguous in KParams::sched).

// Kernel parameters (passed by value).
struct KParams {
  const uint32_t *net;        // design words
  const uint32_t *sched;      // exec-level blocks
  const uint2 *levelDesc;     // (block offset, words) per partition level
  uint32_t stageWords;        // capacity of each shared-memory stage buffer (0 = no staging)
  uint32_t constSlots;        // 1: value-pool slots 0..15 are free (renumbered pools) and hold the immediates
  uint32_t resWords;          // words of a block's resident exec levels (0: staged or read from global memory)
  const uint32_t *itemRes;    // per item: word offset of its partition's levels in the block's resident area
  const uint32_t *resCopy;    // (schedule word, words, resident word) per copy: a partition's levels, contiguous
  const uint32_t *resCopyBegin;  // [2][nBlocks + 1] prefix offsets into resCopy (triples) per region and block
  const PartDesc *parts;
  const uint8_t *constVec;
  const uint8_t *lutTable;    // 4642 entries, padded to 4656
  const uint32_t *items;      // per region: list of (part | groupBlock << 20)
  const uint32_t *itemBegin;  // [2][nBlocks + 1] prefix offsets into items per block
  uint32_t *regs;             // [regSlots][gpad] words
  uint32_t *exg;              // [exgSlots][gpad] words
  uint8_t *mems;              // [nStreams][memStride]
  const uint8_t *initRegs;    // [regSlots] initial nibbles
  const uint8_t *initMems;    // [memPoolSize]
  uint32_t *stop;             // [nStreams] sticky stop flags
  uint32_t *stopCycle;        // [nStreams] first stop cycle
  uint32_t *err;              // device error word (kErr*)
  uint32_t *errInfo;          // [4] detail of the first error
  uint32_t *barrier;          // [2]: grid-barrier arrival counter (zeroed per launch), unused word
  uint32_t *realCycles;
  unsigned long long *digAcc; // [nStreams] per-cycle digest accumulators
  unsigned long long *roll;   // [nStreams] rolling digests
  unsigned long long *cycDig; // [nStreams][cycStride] or null
  long long *profUseful;      // [nParts] or null
  long long *profTotal;       // [nParts] or null
  // stimulus
  const uint32_t *stimReg;
  const uint8_t *stimBits;
  const uint16_t *stimToggle;
  const unsigned long long *streamSeed;  // [nStreams]
  uint32_t nStim;
  uint32_t regSlots, exgSlots, memPoolSize;
  unsigned long long memStride;
  uint32_t nStreams, gpad;    // streams, padded 8-stream groups
  uint32_t groupsPerItem;
  uint32_t maxVpSlots;
  uint32_t nBlocks;
  uint32_t nParts;
  uint32_t cycStride;
  uint32_t cycBase;           // cycle of index 0 in cycDig rows (direct runs)
  uint32_t enablePrint;
  uint32_t flags;             // kFlag*
  uint32_t printDiag;         // reference-style first-stop diagnostics (single stream)
  unsigned long long timeoutNs;
  const char *const *printMsgs;
  uint32_t nPrintMsgs;
  uint32_t stimTableC0;       // first cycle the stimulus table covers
  const uint8_t *stimTable;   // [cycle][input][stream] nibbles, or null (hash stimulus)
  // admission (kFlagSlots): queued job streams run on the resident slots
  uint32_t *slotStream;       // [slots] job stream, kNoStream when idle
  uint32_t *slotStart;        // [slots] global cycle of the stream's cycle 0
  uint32_t *slotRetire;       // [slots] global cycle at which it retires (start + length)
  const uint32_t *jobLen;     // [jobs]
  const unsigned long long *jobSeed;  // [jobs]
  const uint32_t *queueOrder; // [jobs] admission order (longest first)
  uint32_t *queueHead;        // next position in queueOrder
  uint32_t *queueSnap;        // queueHead when the current cycle's retirements were listed
  uint32_t *retList;          // [slots] slots retiring in the current cycle, in slot order
  uint32_t *retCount;         // their number (written every cycle)
  uint32_t *nDone;            // job streams retired so far
  uint32_t *eventHint;        // [4] when to scan for retirements (per cycle parity: next length retirement, stop cycle + 1)
  uint32_t *retireMask;       // [gpad] nibble masks of the current cycle's retiring slots
  unsigned long long *memAcc; // [slots] final memory digests
  unsigned long long *outReg, *outMem, *outRoll;  // [jobs]
  uint32_t *outStop;          // [jobs]
  uint32_t nJobs;
  // per-micro-partition clock64 profile (kFlagProfileMP), indexed by the id in header word 1
  unsigned long long *mpCycles;
  uint32_t *mpCount;
  // graph form: {cycle counter, unused, end cycle, first cycle, exit} on the
  // device, so one captured chunk serves every call
  uint32_t *graphState;
  uint32_t *nStopped;         // kFlagStopExit: streams stopped so far
  uint32_t *probeBuf;         // signal capture: [probe][gpad] value-pool words after the exec levels (null = off)
};

constexpr uint32_t kNoStream = 0xFFFFFFFFu;
constexpr uint32_t kMaxSlotWords = 128;  // admission: at most 4,096 slots (one bit each in shared memory)

enum : uint32_t {
  kFlagStimulus = 1u,   // apply the stimulus before every cycle
  kFlagDigest = 2u,     // per-cycle register digests (rolling / per-cycle array)
  kFlagProfile = 4u,    // per-partition clock64 profile (free-running)
  kFlagCountCycles = 8u, // advance realCycles (free-running launches only, SimEval.cu:985-989)
  kFlagSlots = 16u,      // job streams queued onto resident slots, retired and admitted in place
  kFlagProfileMP = 32u,  // clock64 cycles of every micro-partition evaluation (cost-model samples)
  kFlagStopExit = 64u    // a stream freezes after its stop cycle; the launch ends once every stream stopped
};

enum : uint32_t {
  kErrNone = 0,
  kErrTimeout = 1,      // grid barrier wait ran out of budget
  kErrMemRange = 2,     // memory read/write beyond the pool
  kErrBadOp = 3,        // unknown micro-partition kind
};

constexpr uint32_t kLutTablePadded = 4656;  // 4642 rounded up to 16 bytes

}  // namespace tgs
