// Host-side device image and schedule (see emit.cpp).
#pragma once
#include <cstdint>
#include <vector>

#include "devimage.h"
#include "tgs_internal.h"

namespace tgs {

// Structural features of one micro-partition: the inputs of the learned cost
// model and of the gate-count fallback.
struct MPartFeat {
  uint32_t kind = 0;        // kMPLut / kMPVecRead / kMPVecOp / kMPMemRead
  uint32_t lanes = 0;       // widest level
  uint32_t depth = 0;       // levels (top + middle)
  uint32_t ops = 0;         // op slots (LUT + moves, or special lanes)
  uint32_t nops = 0;        // moves
  uint32_t threeOp = 0;     // ops with a non-immediate op0
  uint32_t vpReads = 0;     // value-pool operand reads
  uint32_t writes = 0;      // slots written
  uint32_t memPorts = 0;
  uint32_t vecNibbles = 0;
  uint32_t fanIn = 0;       // distinct slots read
  uint32_t fanOut = 0;      // later readers of its outputs
  uint32_t partLevels = 0;  // exec levels of its partition
  uint32_t fastOps = 0;     // LUT ops evaluated with word-wide logic (no table read)
  uint32_t fastTop = 0;     // 1: the top level is word-wide (kMPFastTop)
};

struct MPartRef {
  uint32_t off = 0;    // word offset in DeviceImage::net
  uint32_t words = 0;  // record size, multiple of 4
  uint32_t id = 0;     // design-wide micro-partition index
  MPartFeat feat;
  std::vector<uint32_t> reads, writes;
};

struct DeviceImage {
  std::vector<uint32_t> net;
  std::vector<PartDesc> parts;
  std::vector<uint8_t> constVec;
  std::vector<uint32_t> partRegion;
  std::vector<std::vector<std::vector<MPartRef>>> mp;  // [part][level][i]
  uint32_t maxVpSlots = 0;
  uint32_t nMParts = 0;
  bool renumbered = false;  // every partition's slots renumbered (slots 0..15 unused)
};

struct Schedule {
  uint32_t NW = 0;
  // exec-level blocks: per partition and level, [flags][NW + 1 prefix
  // offsets][unit offsets][micro-partition records in warp order], 16-byte
  // aligned so a level is one bulk copy; levelDesc = (block offset, words)
  // per level, PartDesc::schedOff indexes the partition's first level
  std::vector<uint32_t> words;
  std::vector<uint32_t> levelDesc;
  uint32_t maxLevelWords = 0;
  std::vector<uint32_t> items;      // (part | groupBlock << 20) per region and block
  std::vector<uint32_t> itemBegin;  // [2][nBlocks + 1]
  std::vector<double> partCost;
  double makespan[2] = {0, 0};
  uint64_t barriers = 0, levels = 0;
  uint64_t fusedLevels = 0;  // exec levels merged into the block before them (levels per barrier > 1)
  // per level block, summed: the most loaded warp's cost, all units' cost,
  // max(cost / warps, largest unit) (no schedule does better) and
  // cost / warps + largest unit (a list schedule of single units does no worse)
  double planMakespan = 0, planWork = 0, planLower = 0, planUpper = 0;
};

// Schedule knobs (tgs_options.mpart_lanes / levels_per_barrier).
struct SchedOpts {
  uint32_t unitLanes = 32;       // LUTs a warp takes per unit of its level plan: 32, 64 or 128
  uint32_t levelsPerBarrier = 1;  // exec levels one block may merge: 1, 2 or 4
};

// Word-wide evaluation of palette LUT ops.  A LUT op reads table entry
// lutIndex + (a << 8 | b << 4 | c) per stream (src/SimEval.cu:350-356).
// When a is an immediate and the 256 entries of that row are a bitwise
// function g of (b, c) -- every output bit i equal to g(b_i, c_i): AND, OR,
// XOR, NAND, a move ... -- the kernel computes the 8 streams of a word with
// three bitwise instructions instead of eight table reads.  When a is a slot
// and rows a = 0 and a = 1 pass c and b (a multiplexer) or b and c, the word
// is c ^ (mask(a) & (b ^ c)) whenever every stream's a is 0 or 1; a word with
// another select value reads the table.  Every entry of a row is compared
// with the function at load time, so results equal the table lookups.
//
// The device image's encoding of fast ops: kFastOp and friends (devimage.h).

class FastLuts {
 public:
  explicit FastLuts(const std::vector<uint8_t> &lut);
  // the op's fast lut field, or 0 when it needs table lookups
  uint16_t code(const toucanGPUSim::CGMicroPartLUTTopLevelOp &o);
  int rowCode(uint32_t row);
  int muxCode(uint32_t base);

 private:
  const std::vector<uint8_t> &lut_;
  std::vector<int> rowCode_, muxCode_;  // -2: not computed yet
};

// One exec level with its single-level LUT micro-partitions (top level and
// write-back only) regrouped op by op: ops with a fast form first, then ops
// that need table lookups, each group packed into micro-partitions of up to
// 32 lanes and 32 write-back entries, so that a warp evaluates ops of one
// kind.  Ops of such micro-partitions are independent (each reads slots no
// op of the level writes), which is checked; a level that breaks it is
// returned unchanged.  fast == nullptr: repacked in op order.
std::vector<toucanGPUSim::CGMicroPartInfo> regroupLevel(const std::vector<toucanGPUSim::CGMicroPartInfo> &in,
                                                       FastLuts *fast);

// compactSlots: renumber value-pool slots by live range (slotalloc.h).
// probes (optional): per partition, (value-pool slot, probe index) pairs
// whose values the kernel records after the exec levels (signal capture).
using ProbeList = std::vector<std::vector<std::pair<uint32_t, uint32_t>>>;
// One exec level with its LUT micro-partitions of up to 16 lanes laid side by
// side into 32-lane ones (same values; emit.cpp).
std::vector<toucanGPUSim::CGMicroPartInfo> packLevel(const std::vector<toucanGPUSim::CGMicroPartInfo> &in);

// packLanes: packLevel applied to every exec level; fastLuts: palette ops
// evaluated word-wide, single-level micro-partitions regrouped by kind
// (after packing).
void buildImage(const toucanGPUSim::SimDesignInfo &d, DeviceImage &img, bool compactSlots,
                const ProbeList *probes = nullptr, bool packLanes = false, bool fastLuts = false);
// cost: optional [part][level][mpart] predicted cost; null = gate count.
// G: stream groups per item (special micro-partitions are split by group).
// so: micro-partition size (LUT units bundled per warp) and levels per
// barrier (consecutive exec levels merged into one block where every
// dependency inside stays on one warp and the merged block is no slower).
void buildSchedule(const toucanGPUSim::SimDesignInfo &d, DeviceImage &img, uint32_t NW, uint32_t G,
                   const std::vector<std::vector<std::vector<float>>> *cost, uint32_t nBlocks, uint32_t nGroupBlocks,
                   Schedule &out, const SchedOpts &so = SchedOpts());
float gateCost(const MPartFeat &f);

}  // namespace tgs
