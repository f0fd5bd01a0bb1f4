// Host runtime and C ABI (include/toucan_gb300.h).
//
// Replaces the reference host path: ToucanSimulator::init / setupGPU /
// eval / eval_free_running (src/ToucanSim.cu:16-267), copy_netlist_to_gpu and
// the register I/O (src/SimEval.cu:1058-1343).  Differences by design: a
// handle instead of process-global device state, every allocation freed by
// tgs_destroy, status codes instead of exit(), and many streams per handle.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <fstream>
#include <iterator>
#include <map>
#include <memory>
#include <numeric>
#include <queue>
#include <tuple>
#include <string>
#include <vector>

#include "emit.h"
#include "slotalloc.h"
#include "kernels.h"
#include "learned.h"
#include "tgs_internal.h"

using namespace toucanGPUSim;

namespace tgs {

namespace {
thread_local std::string gLastError;
}

void setLastError(const std::string &m) { gLastError = m; }

std::vector<uint8_t> readFileBytes(const std::string &path) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error(TGS_ERR_IO, "cannot open " + path);
  return std::vector<uint8_t>(std::istreambuf_iterator<char>(f), std::istreambuf_iterator<char>());
}

#define TGS_CUDA(call)                                                                                     \
  do {                                                                                                     \
    cudaError_t e_ = (call);                                                                               \
    if (e_ != cudaSuccess) throw ::tgs::Error(TGS_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// Device buffer owned by a handle.
template <typename T>
struct DBuf {
  T *p = nullptr;
  size_t n = 0;
  void alloc(size_t count) {
    free();
    if (count == 0) count = 1;
    TGS_CUDA(cudaMalloc(&p, count * sizeof(T)));
    n = count;
  }
  void upload(const T *src, size_t count, cudaStream_t s) {
    if (count > n) alloc(count);
    if (count) TGS_CUDA(cudaMemcpyAsync(p, src, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void upload(const std::vector<T> &v, cudaStream_t s) { upload(v.data(), v.size(), s); }
  void free() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  ~DBuf() { free(); }
};

}  // namespace tgs

struct tgs_sim {
  tgs_options opt{};
  SimDesignInfo design;
  SimDebugInfo symbols;
  tgs::ValidateInfo vinfo;
  tgs::DeviceImage img;
  tgs::Schedule sched;
  bool loaded = false;
  int device = -1;
  cudaDeviceProp props{};
  cudaStream_t stream = nullptr;
  bool enablePrint = false;
  uint64_t cycleCnt = 0;
  uint64_t streamCycles = 0;  // batch bookkeeping

  // launch configuration
  tgs::LaunchCfg lc;
  uint32_t spw = 1, groups = 1, gpad = 1, nStreams = 1, regSlots = 4, exgSlots = 4, stageWords = 0;
  uint32_t resWords = 0;  // words of a block's resident exec levels (0: staged or global)
  unsigned long long memStride = 16;

  // device memory
  tgs::DBuf<uint32_t> itemRes, resCopy, resCopyBegin;  // resident exec levels (see configure)
  tgs::DBuf<uint32_t> net, schedW, levelDesc, items, itemBegin, regs, exg, stop, stopCycle, err, errInfo, barrier, realCycles, stimReg;
  tgs::DBuf<tgs::PartDesc> parts;
  tgs::DBuf<uint8_t> constVec, lutTable, mems, initRegs, initMems, stimBits;
  tgs::DBuf<uint16_t> stimToggle;
  tgs::DBuf<unsigned long long> digAcc, roll, cycDig, seeds, outA, outB;
  tgs::DBuf<long long> profU, profT;
  tgs::DBuf<char *> msgPtrs;
  std::vector<tgs::DBuf<char>> msgs;
  tgs::DBuf<uint32_t> ioIds;
  tgs::DBuf<uint32_t> slotStream, slotStart, slotRetire, jobLen, queueOrder, retList, retireMask, outStop;
  tgs::DBuf<uint32_t> admW;  // admission words: queue head, queue snapshot, retire count, done count, scan hints [4]
  tgs::DBuf<unsigned long long> jobSeed, memAcc, outReg, outMem, outRoll;
  tgs::DBuf<uint8_t> stimTable;
  tgs::DBuf<unsigned long long> mpCycles;
  tgs::DBuf<uint32_t> graphState;  // graph form: cycle counter, unused, end, first cycle, exit
  tgs::DBuf<uint32_t> nStopped;    // stop exit: streams stopped
  // signal capture (symbol file signalDebugInfo): probe = one (partition,
  // slot) section; a signal = its sections' probes and widths, most
  // significant first
  bool captureSignals = false;
  tgs::ProbeList probes;
  uint32_t nProbes = 0;
  std::map<std::string, std::vector<std::pair<uint32_t, uint32_t>>> signalProbes;  // name -> (probe, width)
  tgs::DBuf<uint32_t> probeBuf;    // [probe][gpad]
  // VCD dump (ToucanSimulator::enableVCDDump)
  std::unique_ptr<std::ofstream> vcd;
  std::vector<std::string> vcdNames, vcdIds;
  std::vector<uint32_t> vcdWidths;
  std::vector<std::string> vcdLast;
  bool vcdFirst = true;
  // instantiated graph chunks, keyed by the launch parameters they captured
  struct GraphEntry {
    std::vector<uint8_t> key;
    cudaGraphExec_t exec = nullptr;
  };
  std::vector<GraphEntry> graphs;
  uint64_t graphLaunches = 0;
  uint32_t lastLaunches = 0;  // kernel launches of the last cycle run
  tgs::DBuf<uint32_t> mpCount;
  uint64_t batchCycle = 0;  // cycles run by TGS_BATCH_CONTINUE batches since the last reset
  tgs::DBuf<uint8_t> ioBytes;
  tgs::KParams kp{};
  // learned cost model (optional)
  std::unique_ptr<tgs::CostModel> model;

  ~tgs_sim() {
    if (device >= 0) cudaSetDevice(device);
    for (auto &g : graphs) cudaGraphExecDestroy(g.exec);
    for (auto &m : msgs) m.free();
    if (stream) cudaStreamDestroy(stream);
  }
};

namespace tgs {
namespace {

float runTimed(tgs_sim *h, uint32_t c0, uint32_t n, uint32_t flags);

void checkDeviceError(tgs_sim *h) {
  uint32_t info[4] = {0, 0, 0, 0};
  TGS_CUDA(cudaMemcpy(info, h->errInfo.p, sizeof(info), cudaMemcpyDeviceToHost));
  uint32_t code = 0;
  TGS_CUDA(cudaMemcpy(&code, h->err.p, sizeof(code), cudaMemcpyDeviceToHost));
  if (code == kErrNone) return;
  uint32_t zero[4] = {0, 0, 0, 0};
  TGS_CUDA(cudaMemcpy(h->err.p, zero, sizeof(uint32_t), cudaMemcpyHostToDevice));
  TGS_CUDA(cudaMemcpy(h->errInfo.p, zero, sizeof(zero), cudaMemcpyHostToDevice));
  char buf[256];
  if (code == kErrTimeout) {
    std::snprintf(buf, sizeof buf, "device barrier wait ran out of its budget (block %u, generation %u)", info[1], info[2]);
    throw Error(TGS_ERR_TIMEOUT, buf);
  }
  if (code == kErrMemRange) {
    unsigned long long idx = (unsigned long long)info[1] | ((unsigned long long)info[2] << 32);
    std::snprintf(buf, sizeof buf, "memory access at index %llu beyond memPool (stream %u)", idx, info[3]);
    throw Error(TGS_ERR_DEVICE_FAULT, buf);
  }
  std::snprintf(buf, sizeof buf, "device check failed (code %u)", code);
  throw Error(TGS_ERR_DEVICE_FAULT, buf);
}

void fillParams(tgs_sim *h) {
  KParams &p = h->kp;
  std::memset(&p, 0, sizeof(p));
  p.net = h->net.p;
  p.sched = h->schedW.p;
  p.levelDesc = reinterpret_cast<const uint2 *>(h->levelDesc.p);
  p.stageWords = h->stageWords;
  p.resWords = h->resWords;
  p.itemRes = h->itemRes.p;
  p.resCopy = h->resCopy.p;
  p.resCopyBegin = h->resCopyBegin.p;
  p.constSlots = h->img.renumbered ? 1u : 0u;
  p.parts = h->parts.p;
  p.constVec = h->constVec.p;
  p.lutTable = h->lutTable.p;
  p.items = h->items.p;
  p.itemBegin = h->itemBegin.p;
  p.regs = h->regs.p;
  p.exg = h->exg.p;
  p.mems = h->mems.p;
  p.initRegs = h->initRegs.p;
  p.initMems = h->initMems.p;
  p.stop = h->stop.p;
  p.stopCycle = h->stopCycle.p;
  p.err = h->err.p;
  p.errInfo = h->errInfo.p;
  p.barrier = h->barrier.p;
  p.realCycles = h->realCycles.p;
  p.nStopped = h->nStopped.p;
  p.probeBuf = h->probeBuf.p;
  p.digAcc = h->digAcc.p;
  p.roll = h->roll.p;
  p.cycDig = nullptr;
  p.profUseful = h->profU.p;
  p.profTotal = h->profT.p;
  p.streamSeed = h->seeds.p;
  p.regSlots = h->regSlots;
  p.exgSlots = h->exgSlots;
  p.memPoolSize = h->design.memPoolSize;
  p.memStride = h->memStride;
  p.nStreams = h->nStreams;
  p.gpad = h->gpad;
  p.groupsPerItem = uint32_t(h->lc.G);
  p.maxVpSlots = h->img.maxVpSlots;
  p.nBlocks = h->lc.blocks;
  p.nParts = uint32_t(h->design.parts.size());
  p.enablePrint = h->enablePrint ? 1 : 0;
  p.printDiag = h->nStreams == 1 ? 1 : 0;
  p.timeoutNs = (unsigned long long)std::max<uint32_t>(1, h->opt.barrier_timeout_ms) * 1000000ull;
  p.printMsgs = h->msgPtrs.p;
  p.nPrintMsgs = uint32_t(h->msgs.size());
}

// Launch shape, schedule and per-stream state for the current options.
// Default warps per block: the most common amount of work in an exec level,
// counted in units (a LUT micro-partition is one unit, a special one G units;
// with 8 streams per word a word-wide LUT micro-partition counts a quarter:
// three bitwise instructions per word instead of eight table reads), within
// 6..16, so that a typical level keeps every warp of the block busy (below 6
// the wider levels of a design wait on too few warps: on the mixed 4M-LUT
// design 4 warps ran 236K and 6 warps 247K stimulus-cycles/s).
uint32_t autoWarps(const DeviceImage &img, uint32_t G, uint32_t spw) {
  std::vector<uint64_t> count(33, 0);
  for (const auto &part : img.mp)
    for (const auto &lv : part) {
      uint32_t quarters = 0;
      for (const auto &m : lv) quarters += m.feat.kind != kMPLut ? 4u * G : (spw == 8 && m.feat.fastTop) ? 1u : 4u;
      const uint32_t u = (quarters + 3) / 4;
      if (u) count[std::min<uint32_t>(u, 32)]++;
    }
  uint32_t best = 8;
  uint64_t bestN = 0;
  for (uint32_t u = 1; u <= 32; ++u)
    if (count[u] > bestN) {
      bestN = count[u];
      best = u;
    }
  return std::clamp<uint32_t>(best, 6, 16);
}

void configure(tgs_sim *h) {
  const tgs_options &o = h->opt;
  h->nStreams = std::max<uint32_t>(1, o.n_streams);
  h->spw = h->nStreams == 1 ? 1 : 8;
  h->groups = (h->nStreams + h->spw - 1) / h->spw;
  int G = 1;
  if (h->spw == 8) {
    if (o.groups_per_item) {
      G = int(o.groups_per_item);
      if (G != 1 && G != 2 && G != 4 && G != 8) throw Error(TGS_ERR_ARG, "groups_per_item must be 1, 2, 4 or 8");
    } else {
      // default: 4 groups per item (independent work per warp) while a
      // region still has two items per SM; fewer for few, narrow partitions
      size_t parts = 1;
      for (auto &r : h->design.regionPartitionIds) parts = std::max(parts, r.size());
      const size_t want = 2 * size_t(std::max(1, h->props.multiProcessorCount));
      G = 4;
      while (G > 1 && parts * ((h->groups + G - 1) / G) < want) G >>= 1;
    }
    while (G > 1 && uint32_t(G) > h->groups) G >>= 1;
  }
  h->gpad = (h->groups + G - 1) / G * G;
  SchedOpts so;
  so.unitLanes = o.mpart_lanes ? o.mpart_lanes : 32u;
  so.levelsPerBarrier = o.levels_per_barrier ? o.levels_per_barrier : 1u;
  if (so.unitLanes != 32 && so.unitLanes != 64 && so.unitLanes != 128)
    throw Error(TGS_ERR_ARG, "mpart_lanes must be 32, 64 or 128");
  if (so.levelsPerBarrier != 1 && so.levelsPerBarrier != 2 && so.levelsPerBarrier != 4)
    throw Error(TGS_ERR_ARG, "levels_per_barrier must be 1, 2 or 4");
  uint32_t NW = o.warps_per_block ? o.warps_per_block : autoWarps(h->img, uint32_t(G), h->spw);
  if (NW < 1 || NW > 32) throw Error(TGS_ERR_ARG, "warps_per_block must be 1 to 32");
  h->lc.spw = int(h->spw);
  h->lc.G = G;
  h->lc.threads = NW * 32;
  h->lc.stream = h->stream;
  h->lc.res = false;
  void *fn = cycleKernelFor(int(h->spw), G, false);
  void *fnRegion = regionKernelFor(int(h->spw), G, false);
  const size_t vpBytes = size_t(h->img.maxVpSlots) * size_t(G) * 4;
  const uint32_t nGB = h->gpad / uint32_t(G);
  size_t maxItems = 1;
  for (auto &r : h->design.regionPartitionIds) maxItems = std::max(maxItems, r.size() * nGB);

  // schedule (greedy gate count or learned cost); exec-level blocks are
  // staged through shared memory when two of the largest fit next to the
  // value pool (option resident_netlist = 2 disables staging)
  std::vector<std::vector<std::vector<float>>> cost;
  const std::vector<std::vector<std::vector<float>>> *costPtr = nullptr;
  if (o.schedule == TGS_SCHED_LEARNED && h->model && h->model->trained()) {
    h->model->predictAll(h->img, cost);
    costPtr = &cost;
  }
  // the kernels' static shared memory (barrier words, retirement bitmask)
  // comes out of the same per-block limit
  cudaFuncAttributes fa{}, fr{};
  TGS_CUDA(cudaFuncGetAttributes(&fa, fn));
  TGS_CUDA(cudaFuncGetAttributes(&fr, fnRegion));
  const size_t optin = size_t(h->props.sharedMemPerBlockOptin) - std::max(fa.sharedSizeBytes, fr.sharedSizeBytes);
  auto shape = [&](uint32_t stage) {
    h->lc.smem = kLutTablePadded + 2 * size_t(stage) * 4 + vpBytes;
    if (h->lc.smem > optin) return 0;
    TGS_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(h->lc.smem)));
    TGS_CUDA(cudaFuncSetAttribute(fnRegion, cudaFuncAttributeMaxDynamicSharedMemorySize, int(h->lc.smem)));
    int perSM = 0;
    TGS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM, fn, int(h->lc.threads), h->lc.smem));
    if (o.blocks_per_sm) perSM = std::min<int>(perSM, int(o.blocks_per_sm));
    return perSM;
  };
  if (kLutTablePadded + vpBytes > optin)
    throw Error(TGS_ERR_RESOURCES, "value pool of " + std::to_string(h->img.maxVpSlots) + " slots x " + std::to_string(G) +
                                       " groups needs " + std::to_string(kLutTablePadded + vpBytes) +
                                       " B of shared memory; lower groups_per_item");
  // first pass to learn the largest level block (independent of the block count)
  buildSchedule(h->design, h->img, NW, uint32_t(G), costPtr, 1, nGB, h->sched, so);
  // Stage buffer size: the largest level, or a smaller size that still
  // stages nearly every level when it puts more blocks on an SM (levels
  // larger than the buffers are read from global memory; mixed 4M-LUT
  // design: 4 -> 5 blocks per SM, 256K -> 310K stimulus-cycles/s)
  uint32_t stage = o.resident_netlist == 2 ? 0u : std::min<uint32_t>(h->sched.maxLevelWords, 4096u);
  if (o.stage_words) stage = std::min<uint32_t>(stage, (o.stage_words + 3u) & ~3u);
  int perSM = shape(stage);
  if (stage) {
    std::vector<uint32_t> sizes;
    for (size_t i = 1; i < h->sched.levelDesc.size(); i += 2) sizes.push_back(h->sched.levelDesc[i]);
    std::sort(sizes.begin(), sizes.end());
    // items in flight: blocks on the GPU at once, up to the items of a region
    auto inFlight = [&](int n) { return std::min(maxItems, size_t(std::max(n, 0)) * size_t(h->props.multiProcessorCount)); };
    for (double q : {0.99, 0.98, 0.95}) {
      const uint32_t cand = (sizes[size_t(q * double(sizes.size() - 1))] + 3u) & ~3u;
      if (cand >= stage || cand == 0) continue;
      const int n = shape(cand);
      if (inFlight(n) > inFlight(perSM)) {
        stage = cand;
        perSM = n;
      }
    }
  }
  const int perSMNoStage = shape(0);
  if (stage && perSM < std::max(1, perSMNoStage / 2)) {  // keep at least half the occupancy
    stage = std::min<uint32_t>(stage, 1024u);
    perSM = shape(stage);
    if (perSM <= 0) {
      stage = 0;
      perSM = shape(0);
    }
  } else if (stage && perSM <= 0) {
    stage = 0;
    perSM = shape(0);
  }
  perSM = shape(stage);  // leaves the kernel attribute at the chosen size
  if (perSM <= 0) throw Error(TGS_ERR_RESOURCES, "no block of the cycle kernel fits on an SM with this configuration");
  // More items than blocks in flight: 4-warp blocks when they put at least
  // a quarter more items in flight (blocks on the GPU at once, up to the
  // items of a region), so more items are evaluated side by side (a single
  // stream of the 16M-LUT design, 1,024 items per region: 1,024 blocks of 4
  // warps instead of 760 of 6, 5.6K -> 7.6K cycles/s)
  if (!o.warps_per_block && NW > 4) {
    int perSM4 = 0;
    TGS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSM4, fn, 128, h->lc.smem));
    if (o.blocks_per_sm) perSM4 = std::min<int>(perSM4, int(o.blocks_per_sm));
    const size_t sms = size_t(h->props.multiProcessorCount);
    const size_t inFlight = std::min(maxItems, size_t(perSM) * sms), inFlight4 = std::min(maxItems, size_t(perSM4) * sms);
    if (4 * inFlight4 >= 5 * inFlight) {
      NW = 4;
      h->lc.threads = 128;
      perSM = perSM4;
    }
  }
  h->stageWords = stage;
  h->lc.blocks = uint32_t(std::max<size_t>(1, std::min<size_t>(size_t(perSM) * h->props.multiProcessorCount, maxItems)));
  buildSchedule(h->design, h->img, NW, uint32_t(G), costPtr, h->lc.blocks, nGB, h->sched, so);

  // Resident exec levels: the levels of every partition a block evaluates
  // (both regions, one contiguous range of the schedule per partition) are
  // copied into the block's shared memory once per launch, replacing one
  // bulk copy per level whose latency a short level cannot hide.  Chosen
  // when every block of the grid still fits on the GPU at once.
  h->resWords = 0;
  {
    const uint32_t B = h->lc.blocks;
    std::vector<uint32_t> itemRes(h->sched.items.size(), 0), resCopy, resBegin(2 * (B + 1), 0), at(B, 0);
    std::vector<uint32_t> placedAt(h->design.parts.size(), UINT32_MAX);
    for (uint32_t r = 0; r < 2; ++r)
      for (uint32_t b = 0; b <= B; ++b) {
        resBegin[r * (B + 1) + b] = uint32_t(resCopy.size() / 3);
        if (b == B) break;
        const uint32_t i0 = h->sched.itemBegin[r * (B + 1) + b], i1 = h->sched.itemBegin[r * (B + 1) + b + 1];
        std::vector<uint32_t> placed;
        for (uint32_t i = i0; i < i1; ++i) {
          const uint32_t pid = h->sched.items[i] & 0xFFFFFu;
          const PartDesc &pd = h->img.parts[pid];
          if (placedAt[pid] == UINT32_MAX && pd.nLevels) {
            const uint32_t first = h->sched.levelDesc[2 * pd.schedOff];
            const uint32_t last = pd.schedOff + pd.nLevels - 1;
            const uint32_t end = (h->sched.levelDesc[2 * last] + h->sched.levelDesc[2 * last + 1] + 3u) & ~3u;
            placedAt[pid] = at[b];
            resCopy.insert(resCopy.end(), {first, end - first, at[b]});
            at[b] += end - first;
            placed.push_back(pid);
          }
          itemRes[i] = placedAt[pid] == UINT32_MAX ? 0u : placedAt[pid];
        }
        for (uint32_t pid : placed) placedAt[pid] = UINT32_MAX;
      }
    const uint32_t words = B ? *std::max_element(at.begin(), at.end()) : 0u;
    const uint32_t want = o.resident_netlist;  // 0 auto, 1 resident, 2 global, 3 staged
    if ((want == 0 || want == 1) && words) {
      const size_t smemRes = kLutTablePadded + vpBytes + size_t(words) * 4;
      int perSMRes = 0;
      void *fnRes = cycleKernelFor(int(h->spw), G, true), *fnRegionRes = regionKernelFor(int(h->spw), G, true);
      cudaFuncAttributes ra{}, rr{};
      TGS_CUDA(cudaFuncGetAttributes(&ra, fnRes));
      TGS_CUDA(cudaFuncGetAttributes(&rr, fnRegionRes));
      const size_t optinRes = size_t(h->props.sharedMemPerBlockOptin) - std::max(ra.sharedSizeBytes, rr.sharedSizeBytes);
      if (smemRes <= optinRes) {
        TGS_CUDA(cudaFuncSetAttribute(fnRes, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smemRes)));
        TGS_CUDA(cudaFuncSetAttribute(fnRegionRes, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smemRes)));
        TGS_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&perSMRes, fnRes, int(h->lc.threads), smemRes));
        if (o.blocks_per_sm) perSMRes = std::min<int>(perSMRes, int(o.blocks_per_sm));
      }
      if (perSMRes > 0 && size_t(perSMRes) * h->props.multiProcessorCount >= B) {
        h->resWords = words;
        h->stageWords = 0;
        h->lc.smem = smemRes;
        h->lc.res = true;
        h->itemRes.upload(itemRes, h->stream);
        h->resCopy.upload(resCopy, h->stream);
        h->resCopyBegin.upload(resBegin, h->stream);
      } else {
        if (want == 1)
          throw Error(TGS_ERR_RESOURCES, "resident exec levels need " + std::to_string(smemRes) +
                                             " B of shared memory per block for " + std::to_string(B) + " blocks");
        shape(stage);  // back to the staged (or global) size
      }
    } else if (want == 1) {
      throw Error(TGS_ERR_RESOURCES, "resident exec levels: the blocks have no levels to keep");
    }
  }
  h->parts.upload(h->img.parts, h->stream);
  h->schedW.upload(h->sched.words, h->stream);
  h->levelDesc.upload(h->sched.levelDesc, h->stream);
  h->items.upload(h->sched.items, h->stream);
  h->itemBegin.upload(h->sched.itemBegin, h->stream);

  // per-stream state
  h->regSlots = std::max<uint32_t>(4, (h->design.regPoolSize + 3) & ~3u);
  h->exgSlots = std::max<uint32_t>(4, (h->design.exchangePoolSize + 3) & ~3u);
  h->memStride = std::max<unsigned long long>(16, (h->design.memPoolSize + 15ull) & ~15ull);
  h->regs.alloc(size_t(h->regSlots) * h->gpad);
  h->exg.alloc(size_t(h->exgSlots) * h->gpad);
  h->mems.alloc(size_t(h->memStride) * h->nStreams);
  h->stop.alloc(h->nStreams);
  h->stopCycle.alloc(h->nStreams);
  h->digAcc.alloc(h->nStreams);
  h->roll.alloc(h->nStreams);
  h->seeds.alloc(h->nStreams);
  h->outA.alloc(h->nStreams);
  h->outB.alloc(h->nStreams);
  if (h->captureSignals && h->nProbes) {
    h->probeBuf.alloc(size_t(h->nProbes) * h->gpad);
    TGS_CUDA(cudaMemsetAsync(h->probeBuf.p, 0, size_t(h->nProbes) * h->gpad * 4, h->stream));
  } else {
    h->probeBuf.free();
  }
  fillParams(h);
}

void resetState(tgs_sim *h) {
  TGS_CUDA(launchInitState(int(h->spw), h->kp, h->stream));
  for (uint32_t s = 0; s < h->nStreams; ++s)
    TGS_CUDA(cudaMemcpyAsync(h->mems.p + size_t(s) * h->memStride, h->initMems.p, h->design.memPoolSize,
                             cudaMemcpyDeviceToDevice, h->stream));
  TGS_CUDA(cudaMemsetAsync(h->stop.p, 0, h->nStreams * sizeof(uint32_t), h->stream));
  TGS_CUDA(cudaMemsetAsync(h->stopCycle.p, 0xFF, h->nStreams * sizeof(uint32_t), h->stream));
  TGS_CUDA(cudaMemsetAsync(h->realCycles.p, 0, sizeof(uint32_t), h->stream));
  TGS_CUDA(cudaStreamSynchronize(h->stream));
}

void setupDevice(tgs_sim *h, int gpu) {
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) throw Error(TGS_ERR_NO_DEVICE, "no CUDA device available");
  if (gpu < 0 || gpu >= n) throw Error(TGS_ERR_NO_DEVICE, "gpu id " + std::to_string(gpu) + " out of range");
  TGS_CUDA(cudaSetDevice(gpu));
  TGS_CUDA(cudaGetDeviceProperties(&h->props, gpu));
  // sm_103a code only (the reference requires cc >= 7.0, ToucanSim.cu:34-43)
  if (h->props.major != 10) throw Error(TGS_ERR_NO_DEVICE, std::string("the library is compiled for sm_103a; found ") + h->props.name);
  if (!h->props.cooperativeLaunch) throw Error(TGS_ERR_NO_DEVICE, "GPU does not support cooperative launch");
  h->device = gpu;
  if (!h->stream) TGS_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
}

// Probes of every signal in the symbol file (option capture_signals).
void buildProbes(tgs_sim *h) {
  h->captureSignals = h->opt.capture_signals != 0;
  h->probes.assign(h->design.parts.size(), {});
  h->signalProbes.clear();
  h->nProbes = 0;
  if (!h->captureSignals) return;
  std::map<std::pair<uint32_t, uint32_t>, uint32_t> index;
  std::vector<std::string> names;
  for (auto &kv : h->symbols.signalDebugInfo) names.push_back(kv.first);
  std::sort(names.begin(), names.end());
  for (auto &name : names) {
    auto &secs = h->symbols.signalDebugInfo.at(name);
    std::vector<std::pair<uint32_t, uint32_t>> sp;
    for (auto &t : secs) {
      const uint32_t part = std::get<0>(t), slot = std::get<1>(t), width = std::get<2>(t);
      if (part >= h->design.parts.size() || slot >= std::max<uint32_t>(h->design.parts[part].valuePoolSize, 16))
        throw Error(TGS_ERR_INVALID_DESIGN, "signal " + name + " names a slot beyond its partition's value pool");
      if (width > 4) throw Error(TGS_ERR_INVALID_DESIGN, "signal " + name + " has a section wider than a nibble");
      auto it = index.find({part, slot});
      if (it == index.end()) {
        it = index.emplace(std::make_pair(part, slot), h->nProbes++).first;
        h->probes[part].push_back({slot, it->second});
      }
      sp.push_back({it->second, width});
    }
    h->signalProbes[name] = std::move(sp);
  }
}

void upload(tgs_sim *h) {
  cudaStream_t s = h->stream;
  buildProbes(h);
  buildImage(h->design, h->img, h->opt.value_pool == 0, h->captureSignals ? &h->probes : nullptr,
             h->opt.lane_packing == 0, h->opt.fast_luts == 0 && h->opt.n_streams > 1);
  h->net.upload(h->img.net, s);
  h->constVec.upload(h->img.constVec, s);
  std::vector<uint8_t> lut(kLutTablePadded, 0);
  std::memcpy(lut.data(), h->design.lut.data(), std::min<size_t>(h->design.lut.size(), kLutSize));
  h->lutTable.upload(lut, s);
  std::vector<uint8_t> ir(std::max<uint32_t>(4, (h->design.regPoolSize + 3) & ~3u), 0);
  std::memcpy(ir.data(), h->design.regPool.data(), h->design.regPool.size());
  h->initRegs.upload(ir, s);
  // rounded up to 16 bytes: the in-kernel memory reset copies 16-byte vectors
  h->initMems.alloc(std::max<size_t>(16, (h->design.memPool.size() + 15) & ~size_t(15)));
  TGS_CUDA(cudaMemsetAsync(h->initMems.p, 0, h->initMems.n, s));
  if (!h->design.memPool.empty())
    TGS_CUDA(cudaMemcpyAsync(h->initMems.p, h->design.memPool.data(), h->design.memPool.size(), cudaMemcpyHostToDevice, s));
  h->err.alloc(1);
  h->errInfo.alloc(4);
  h->graphState.alloc(5);
  h->nStopped.alloc(1);
  h->barrier.alloc(2);
  h->realCycles.alloc(1);
  TGS_CUDA(cudaMemsetAsync(h->err.p, 0, sizeof(uint32_t), s));
  TGS_CUDA(cudaMemsetAsync(h->errInfo.p, 0, 4 * sizeof(uint32_t), s));
  h->profU.alloc(h->design.parts.size());
  h->profT.alloc(h->design.parts.size());
  // print messages (copy_netlist_to_gpu, SimEval.cu:1313-1326)
  for (auto &m : h->msgs) m.free();
  h->msgs.clear();
  h->msgs.resize(h->design.printMsgs.size());
  std::vector<char *> ptrs;
  for (size_t i = 0; i < h->design.printMsgs.size(); ++i) {
    const std::string &str = h->design.printMsgs[i];
    h->msgs[i].upload(str.c_str(), str.size() + 1, s);
    ptrs.push_back(h->msgs[i].p);
  }
  if (ptrs.empty()) ptrs.push_back(nullptr);
  h->msgPtrs.upload(ptrs, s);
  TGS_CUDA(cudaStreamSynchronize(s));
}

void initCommon(tgs_sim *h, int gpu, const uint8_t *design, size_t dn, const uint8_t *sym, size_t sn, bool randomize,
                bool print) {
  h->loaded = false;
  h->design = SimDesignInfo();
  h->symbols = SimDebugInfo();
  parseDesign(design, dn, h->design);
  if (sym) parseSymbols(sym, sn, h->symbols);
  h->design.Init();
  if (randomize) h->design.Randomize(0, h->symbols);
  h->vinfo = ValidateInfo();
  if (h->opt.validate) h->vinfo = validateDesign(h->design, &h->symbols);
  setupDevice(h, gpu);
  h->enablePrint = print;
  upload(h);
  configure(h);
  resetState(h);
  h->cycleCnt = 0;
  h->loaded = true;
}

void requireLoaded(tgs_sim *h) {
  if (!h) throw Error(TGS_ERR_ARG, "null handle");
  if (!h->loaded) throw Error(TGS_ERR_STATE, "simulator not initialised");
  TGS_CUDA(cudaSetDevice(h->device));
}

// Graph form: chunks of up to 32 cycles (two region launches and an admit
// launch per cycle) captured once and replayed.  The kernels read the cycle,
// the event cursor and the end cycle from device words, so a chunk captured
// for one call serves every later call with the same launch parameters.
cudaGraphExec_t graphChunk(tgs_sim *h, const KParams &p, uint32_t k, bool admit) {
  std::vector<uint8_t> key(sizeof(KParams) + 7 * sizeof(uint32_t));
  std::memcpy(key.data(), &p, sizeof(KParams));
  const uint32_t tail[7] = {k, admit ? 1u : 0u, uint32_t(h->lc.spw), uint32_t(h->lc.G), h->lc.blocks, h->lc.threads,
                            uint32_t(h->lc.smem)};
  std::memcpy(key.data() + sizeof(KParams), tail, sizeof(tail));
  for (auto &g : h->graphs)
    if (g.key == key) return g.exec;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  TGS_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
  const cudaError_t e = enqueueGraphChunk(h->lc, p, k, admit);
  const cudaError_t e2 = cudaStreamEndCapture(h->stream, &graph);
  if (e != cudaSuccess || e2 != cudaSuccess) {
    if (graph) cudaGraphDestroy(graph);
    TGS_CUDA(e != cudaSuccess ? e : e2);
  }
  const cudaError_t e3 = cudaGraphInstantiate(&exec, graph, 0);
  cudaGraphDestroy(graph);
  TGS_CUDA(e3);
  if (h->graphs.size() >= 4) {
    cudaGraphExecDestroy(h->graphs.front().exec);
    h->graphs.erase(h->graphs.begin());
  }
  h->graphs.push_back({std::move(key), exec});
  return exec;
}

void runGraph(tgs_sim *h, uint32_t c0, uint32_t n, uint32_t flags, uint32_t stopped0) {
  KParams p = h->kp;
  p.graphState = h->graphState.p;
  const uint32_t exit0 = (flags & kFlagStopExit) && stopped0 >= h->nStreams ? 1u : 0u;
  const uint32_t state[5] = {c0, 0, c0 + n, c0, exit0};
  TGS_CUDA(cudaMemcpyAsync(h->graphState.p, state, sizeof(state), cudaMemcpyHostToDevice, h->stream));
  if ((flags & kFlagStimulus) && !exit0) TGS_CUDA(launchStimulus(int(h->spw), p, c0, h->stream));
  const uint32_t k = std::min<uint32_t>(n, 32);
  const bool admit = (flags & (kFlagSlots | kFlagCountCycles | kFlagStopExit)) != 0;
  cudaGraphExec_t exec = graphChunk(h, p, k, admit);
  const uint32_t chunks = (n + k - 1) / k;
  for (uint32_t i = 0; i < chunks; ++i) TGS_CUDA(cudaGraphLaunch(exec, h->stream));
  h->graphLaunches += chunks;
  const uint32_t perCycle = 2u + (admit ? 1u : 0u) + ((flags & kFlagStopExit) && (flags & kFlagStimulus) ? 1u : 0u);
  h->lastLaunches = chunks * (k * perCycle + 1u) + ((flags & kFlagStimulus) ? 1u : 0u);
}

void runCycles(tgs_sim *h, uint32_t c0, uint32_t n, uint32_t flags) {
  if (n == 0) return;
  uint32_t stopped0 = 0;
  if (flags & kFlagStopExit) {
    // streams that stopped before this launch count towards the exit
    std::vector<uint32_t> st(h->nStreams);
    TGS_CUDA(cudaMemcpyAsync(st.data(), h->stop.p, h->nStreams * 4ull, cudaMemcpyDeviceToHost, h->stream));
    TGS_CUDA(cudaStreamSynchronize(h->stream));
    for (uint32_t v : st) stopped0 += v != 0;
    h->lastLaunches = 0;
    if (stopped0 >= h->nStreams) return;  // every stream already stopped
    TGS_CUDA(cudaMemcpyAsync(h->nStopped.p, &stopped0, 4, cudaMemcpyHostToDevice, h->stream));
    TGS_CUDA(cudaStreamSynchronize(h->stream));
  }
  // the graph form records no per-partition profile (persistent form only)
  if (h->opt.mode == TGS_MODE_GRAPH && !(flags & kFlagProfileMP)) flags &= ~kFlagProfile;
  h->kp.flags = flags;
  if (h->opt.mode == TGS_MODE_GRAPH && !(flags & kFlagProfileMP)) {
    runGraph(h, c0, n, flags, stopped0);
    return;
  }
  TGS_CUDA(cudaMemsetAsync(h->barrier.p, 0, 2 * sizeof(uint32_t), h->stream));
  TGS_CUDA(launchCycles(h->lc, h->kp, c0, n));
  h->lastLaunches = 1;
}

int stopFlag(tgs_sim *h) {
  std::vector<uint32_t> st(h->nStreams);
  TGS_CUDA(cudaMemcpy(st.data(), h->stop.p, st.size() * sizeof(uint32_t), cudaMemcpyDeviceToHost));
  for (uint32_t v : st)
    if (v) return 1;
  return 0;
}

const std::vector<std::tuple<uint32_t, uint32_t>> &regLocs(tgs_sim *h, const char *name) {
  if (!name) throw Error(TGS_ERR_ARG, "null register name");
  auto it = h->symbols.regDebugInfo.find(name);
  if (it == h->symbols.regDebugInfo.end()) throw Error(TGS_ERR_NOT_FOUND, std::string("unknown register ") + name);
  if (it->second.size() > 16) throw Error(TGS_ERR_RANGE, std::string("register wider than 64 bits: ") + name);
  return it->second;
}

void streamPos(tgs_sim *h, uint32_t s, uint32_t &g, uint32_t &k) {
  if (s >= h->nStreams) throw Error(TGS_ERR_ARG, "stream index out of range");
  g = s / h->spw;
  k = s % h->spw;
}

// write_reg_to_gpu (SimEval.cu:1072-1081): least significant nibble to the
// last listed id; all nibbles written in one kernel.
void setRegister(tgs_sim *h, uint32_t s, const char *name, uint64_t value) {
  const auto &locs = regLocs(h, name);
  std::vector<uint32_t> ids;
  std::vector<uint8_t> vals;
  uint64_t v = value;
  for (auto it = locs.rbegin(); it != locs.rend(); ++it) {
    ids.push_back(std::get<0>(*it));
    vals.push_back(uint8_t(v & 0xF));
    v >>= 4;
  }
  if (v != 0) throw Error(TGS_ERR_RANGE, std::string("value wider than register ") + name);
  for (uint32_t id : ids)
    if (id >= h->design.regPoolSize) throw Error(TGS_ERR_RANGE, "register id beyond regPool");
  uint32_t g, k;
  streamPos(h, s, g, k);
  h->ioIds.upload(ids, h->stream);
  h->ioBytes.upload(vals, h->stream);
  TGS_CUDA(launchPokeRegs(h->regs.p, h->gpad, g, k, h->ioIds.p, h->ioBytes.p, uint32_t(ids.size()), h->stream));
  TGS_CUDA(cudaStreamSynchronize(h->stream));
}

// read_reg_from_gpu (SimEval.cu:1058-1069): most significant nibble first.
// Probe nibbles of one stream (the values of the last evaluated cycle).
std::vector<uint8_t> probeNibbles(tgs_sim *h, uint32_t s) {
  if (!h->captureSignals) throw Error(TGS_ERR_STATE, "signal capture is off (set options.capture_signals before tgs_init)");
  uint32_t g, k;
  streamPos(h, s, g, k);
  std::vector<uint32_t> words(std::max<uint32_t>(1, h->nProbes));
  if (h->nProbes)
    TGS_CUDA(cudaMemcpy2D(words.data(), 4, h->probeBuf.p + g, size_t(h->gpad) * 4, 4, h->nProbes, cudaMemcpyDeviceToHost));
  std::vector<uint8_t> out(h->nProbes);
  for (uint32_t i = 0; i < h->nProbes; ++i) out[i] = uint8_t((words[i] >> (4 * k)) & 15u);
  return out;
}

// A signal's value: its sections' low `width` bits, most significant first
// (the reference's VCD writer order, unsupport/SimVCD.cpp:226-236).
uint64_t readSignal(tgs_sim *h, uint32_t s, const char *name) {
  if (!h->symbols.signalDebugInfo.count(name)) throw Error(TGS_ERR_NOT_FOUND, std::string("unknown signal ") + name);
  const std::vector<uint8_t> nib = probeNibbles(h, s);  // throws when capture is off
  const auto it = h->signalProbes.find(name);
  uint32_t bits = 0;
  uint64_t v = 0;
  for (auto &pw : it->second) {
    bits += pw.second;
    v = (v << pw.second) | (nib[pw.first] & ((1u << pw.second) - 1u));
  }
  if (bits > 64) throw Error(TGS_ERR_RANGE, std::string("signal ") + name + " is wider than 64 bits");
  return v;
}

// VCD identifier of signal i: base-94 over the printable characters.
std::string vcdId(uint32_t i) {
  std::string id;
  do {
    id.push_back(char(33 + i % 94));
    i /= 94;
  } while (i);
  return id;
}

void enableVcd(tgs_sim *h, const char *path) {
  if (!h->captureSignals) {
    // signal capture changes the device image: only before the first cycle
    if (h->cycleCnt != 0) throw Error(TGS_ERR_STATE, "enable the VCD dump before the first cycle");
    h->opt.capture_signals = 1;
    upload(h);
    configure(h);
    resetState(h);
  }
  auto f = std::make_unique<std::ofstream>(path);
  if (!*f) throw Error(TGS_ERR_IO, std::string("cannot write ") + path);
  h->vcdNames.clear();
  h->vcdWidths.clear();
  for (auto &kv : h->signalProbes) {  // sorted by name
    uint32_t w = 0;
    for (auto &pw : kv.second) w += pw.second;
    h->vcdNames.push_back(kv.first);
    h->vcdWidths.push_back(std::max<uint32_t>(w, 1));
  }
  h->vcdIds.clear();
  for (uint32_t i = 0; i < h->vcdNames.size(); ++i) h->vcdIds.push_back(vcdId(i));
  h->vcdLast.assign(h->vcdNames.size(), std::string());
  h->vcdFirst = true;
  std::ofstream &o = *f;
  char date[64];
  const std::time_t now = std::time(nullptr);
  std::strftime(date, sizeof date, "%Y-%m-%d %H:%M:%S UTC", std::gmtime(&now));
  o << "$date\n    " << date << "\n$end\n$version\n    toucan_gb300\n$end\n$timescale\n    1ps\n$end\n";
  // scopes from the dotted names: a.b.c -> module a, module b, wire c
  std::vector<std::string> open;
  for (uint32_t i = 0; i < h->vcdNames.size(); ++i) {
    std::vector<std::string> parts;
    std::string cur;
    for (char ch : h->vcdNames[i]) {
      if (ch == '.') {
        parts.push_back(cur);
        cur.clear();
      } else {
        cur.push_back(ch);
      }
    }
    size_t common = 0;
    while (common < open.size() && common < parts.size() && open[common] == parts[common]) ++common;
    while (open.size() > common) {
      o << "$upscope $end\n";
      open.pop_back();
    }
    for (size_t j = common; j < parts.size(); ++j) {
      o << "$scope module " << parts[j] << " $end\n";
      open.push_back(parts[j]);
    }
    o << "$var wire " << h->vcdWidths[i] << " " << h->vcdIds[i] << " " << cur << " $end\n";
  }
  while (!open.empty()) {
    o << "$upscope $end\n";
    open.pop_back();
  }
  o << "$enddefinitions $end\n$dumpvars\n";
  h->vcd = std::move(f);
}

// One VCD time step (stream 0): the signals whose value changed.
void vcdDump(tgs_sim *h, uint64_t cycle) {
  if (!h->vcd) return;
  const std::vector<uint8_t> nib = probeNibbles(h, 0);
  std::ofstream &o = *h->vcd;
  o << "#" << cycle << "\n";
  size_t i = 0;
  for (auto &kv : h->signalProbes) {
    std::string bits;
    for (auto &pw : kv.second)
      for (int b = int(pw.second) - 1; b >= 0; --b) bits.push_back(char('0' + ((nib[pw.first] >> b) & 1)));
    if (bits.empty()) bits = "0";
    if (h->vcdFirst || bits != h->vcdLast[i]) {
      if (h->vcdWidths[i] == 1)
        o << bits << h->vcdIds[i] << "\n";
      else
        o << "b" << bits << " " << h->vcdIds[i] << "\n";
      h->vcdLast[i] = bits;
    }
    ++i;
  }
  h->vcdFirst = false;
  o.flush();
}

// read_reg_from_gpu (SimEval.cu:1058-1069), most significant nibble first,
// for many registers at once: the nibbles of every listed register are
// gathered by one kernel and read back with one copy (the reference copies
// one byte per nibble, each a blocking cudaMemcpy).
void readRegisters(tgs_sim *h, uint32_t s, const char *const *names, uint32_t n, uint64_t *out) {
  if (n && (!names || !out)) throw Error(TGS_ERR_ARG, "null names or values");
  std::vector<uint32_t> ids, first(n + 1, 0);
  for (uint32_t i = 0; i < n; ++i) {
    first[i] = uint32_t(ids.size());
    for (auto &l : regLocs(h, names[i])) {
      const uint32_t id = std::get<0>(l);
      if (id >= h->design.regPoolSize) throw Error(TGS_ERR_RANGE, "register id beyond regPool");
      ids.push_back(id);
    }
  }
  first[n] = uint32_t(ids.size());
  uint32_t g, k;
  streamPos(h, s, g, k);
  std::vector<uint8_t> nibs(ids.size());
  if (!ids.empty()) {
    h->ioIds.upload(ids, h->stream);
    if (h->ioBytes.n < ids.size()) h->ioBytes.alloc(ids.size());
    TGS_CUDA(launchPeekRegs(h->regs.p, h->gpad, g, k, h->ioIds.p, h->ioBytes.p, uint32_t(ids.size()), h->stream));
    TGS_CUDA(cudaMemcpyAsync(nibs.data(), h->ioBytes.p, nibs.size(), cudaMemcpyDeviceToHost, h->stream));
    TGS_CUDA(cudaStreamSynchronize(h->stream));
  }
  for (uint32_t i = 0; i < n; ++i) {
    uint64_t r = 0;
    for (uint32_t j = first[i]; j < first[i + 1]; ++j) r = (r << 4) | (nibs[j] & 0xFu);
    out[i] = r;
  }
}

uint64_t readRegister(tgs_sim *h, uint32_t s, const char *name) {
  uint64_t r = 0;
  readRegisters(h, s, &name, 1, &r);
  return r;
}

template <typename F>
int guard(F f) {
  try {
    f();
    return TGS_OK;
  } catch (const Error &e) {
    setLastError(e.what());
    return e.code;
  } catch (const std::bad_alloc &) {
    setLastError("host out of memory");
    return TGS_ERR_RESOURCES;
  } catch (const std::exception &e) {
    setLastError(e.what());
    return TGS_ERR_ARG;
  }
}

}  // namespace

// ---- batch runs -------------------------------------------------------------
void batchRun(tgs_sim *h, const tgs_batch *job, tgs_batch_result *res);

}  // namespace tgs

using namespace tgs;

extern "C" {

const char *tgs_last_error(void) { return gLastError.c_str(); }
const char *tgs_version(void) { return "toucan-gb300 0.1 (sm_103a)"; }

int tgs_create(tgs_sim **out) {
  return guard([&] {
    if (!out) throw Error(TGS_ERR_ARG, "null output pointer");
    *out = new tgs_sim();
    tgs_default_options(&(*out)->opt);
  });
}

int tgs_destroy(tgs_sim *h) {
  return guard([&] { delete h; });
}

int tgs_default_options(tgs_options *o) {
  return guard([&] {
    if (!o) throw Error(TGS_ERR_ARG, "null options");
    std::memset(o, 0, sizeof(*o));
    o->n_streams = 1;
    o->warps_per_block = 0;  // the design's typical exec-level width
    o->groups_per_item = 0;  // 4, or fewer when a region would have too few items
    o->blocks_per_sm = 0;
    o->schedule = TGS_SCHED_GREEDY;
    o->mode = TGS_MODE_PERSISTENT;
    o->barrier_timeout_ms = 5000;
    o->validate = 1;
    o->resident_netlist = 0;
  });
}

int tgs_set_options(tgs_sim *h, const tgs_options *o) {
  return guard([&] {
    if (!h || !o) throw Error(TGS_ERR_ARG, "null argument");
    h->opt = *o;
    if (h->loaded) {
      TGS_CUDA(cudaSetDevice(h->device));
      configure(h);
      resetState(h);
    }
  });
}

int tgs_autotune(tgs_sim *h, const tgs_tune_opts *opts, tgs_tune_trial *trials, uint32_t max_trials,
                 uint32_t *n_trials, tgs_tune_trial *best) {
  return guard([&] {
    if (!h) throw Error(TGS_ERR_ARG, "null handle");
    if (!h->loaded) throw Error(TGS_ERR_STATE, "tgs_autotune before tgs_init");
    TGS_CUDA(cudaSetDevice(h->device));
    tgs_tune_opts o{};
    if (opts) o = *opts;
    const uint32_t cycles = o.cycles ? o.cycles : 16, warm = o.warmup ? o.warmup : 2;
    const uint32_t modes = o.modes ? o.modes : 3u;
    const tgs_options base = h->opt;
    std::vector<uint32_t> Gs = {1};
    if (h->nStreams > 1) Gs = {1, 2, 4, 8};
    const uint32_t NWs[] = {4, 6, 8, 12, 16};
    const uint32_t BPS[] = {1, 2, 0};
    std::vector<tgs_tune_trial> all;
    tgs_tune_trial win{};
    win.ms_per_cycle = -1.f;
    for (uint32_t G : Gs)
      for (uint32_t NW : NWs)
        for (uint32_t stagedOpt = 0; stagedOpt < (o.try_unstaged ? 2u : 1u); ++stagedOpt) {
          uint32_t lastBlocks = 0;
          for (uint32_t bps : BPS) {
            tgs_options t = base;
            t.groups_per_item = G;
            t.warps_per_block = NW;
            t.blocks_per_sm = bps;
            t.resident_netlist = stagedOpt ? 2u : 0u;
            h->opt = t;
            tgs_tune_trial tr{G, NW, bps, 0, 0, 0, -1.f, base.mpart_lanes ? base.mpart_lanes : 32u,
                              base.levels_per_barrier ? base.levels_per_barrier : 1u};
            bool fits = true;
            try {
              configure(h);
            } catch (const Error &e) {
              if (e.code != TGS_ERR_RESOURCES && e.code != TGS_ERR_ARG) throw;
              fits = false;
            }
            if (fits && h->lc.G != int(G)) fits = false;  // fewer groups than G: same as a smaller G
            if (fits && h->lc.blocks == lastBlocks) continue;  // same grid as the previous trial
            if (fits) lastBlocks = h->lc.blocks;
            tr.blocks = fits ? h->lc.blocks : 0;
            tr.staged = !fits ? 0u : h->resWords ? 2u : h->stageWords ? 1u : 0u;
            for (uint32_t mode = 0; mode < 2; ++mode) {
              if (!(modes & (1u << mode))) continue;
              tr.mode = mode;
              tr.ms_per_cycle = -1.f;
              if (fits) {
                h->opt.mode = mode;
                resetState(h);
                fillParams(h);
                runTimed(h, 0, warm, 0);
                tr.ms_per_cycle = runTimed(h, warm, cycles, 0) / float(cycles);
                if (win.ms_per_cycle < 0 || tr.ms_per_cycle < win.ms_per_cycle) win = tr;
              }
              all.push_back(tr);
            }
          }
        }
    if (win.ms_per_cycle < 0) {
      h->opt = base;
      configure(h);
      resetState(h);
      throw Error(TGS_ERR_RESOURCES, "no configuration fits");
    }
    h->opt = base;
    h->opt.groups_per_item = win.groups_per_item;
    h->opt.warps_per_block = win.warps_per_block;
    h->opt.blocks_per_sm = win.blocks_per_sm;
    h->opt.mode = win.mode;
    h->opt.resident_netlist = win.staged ? 0u : 2u;  // the default picks resident / staged as in the trial
    // schedule knobs with the fastest launch configuration: micro-partition
    // size x levels per barrier
    {
      const tgs_options launch = h->opt;
      for (uint32_t lanes : {32u, 64u, 128u})
        for (uint32_t lpbv : {1u, 2u, 4u}) {
          if (lanes == win.mpart_lanes && lpbv == win.levels_per_barrier) continue;  // timed already
          tgs_options t = launch;
          t.mpart_lanes = lanes;
          t.levels_per_barrier = lpbv;
          h->opt = t;
          tgs_tune_trial tr = win;
          tr.mpart_lanes = lanes;
          tr.levels_per_barrier = lpbv;
          tr.ms_per_cycle = -1.f;
          bool fits = true;
          try {
            configure(h);
          } catch (const Error &e) {
            if (e.code != TGS_ERR_RESOURCES && e.code != TGS_ERR_ARG) throw;
            fits = false;
          }
          if (fits) {
            tr.blocks = h->lc.blocks;
            tr.staged = h->resWords ? 2u : h->stageWords ? 1u : 0u;
            resetState(h);
            fillParams(h);
            runTimed(h, 0, warm, 0);
            tr.ms_per_cycle = runTimed(h, warm, cycles, 0) / float(cycles);
            if (tr.ms_per_cycle < win.ms_per_cycle) win = tr;
          }
          all.push_back(tr);
        }
      h->opt = launch;
      h->opt.mpart_lanes = win.mpart_lanes;
      h->opt.levels_per_barrier = win.levels_per_barrier;
    }
    configure(h);
    resetState(h);
    h->cycleCnt = 0;
    h->batchCycle = 0;
    if (trials)
      for (uint32_t i = 0; i < std::min<uint32_t>(max_trials, uint32_t(all.size())); ++i) trials[i] = all[i];
    if (n_trials) *n_trials = uint32_t(all.size());
    if (best) *best = win;
  });
}

int tgs_get_options(const tgs_sim *h, tgs_options *o) {
  return guard([&] {
    if (!h || !o) throw Error(TGS_ERR_ARG, "null argument");
    *o = h->opt;
  });
}

int tgs_init(tgs_sim *h, int gpu_id, const char *design_path, const char *symbol_path, int randomize, int enable_print) {
  return guard([&] {
    if (!h || !design_path) throw Error(TGS_ERR_ARG, "null argument");
    auto d = readFileBytes(design_path);
    std::vector<uint8_t> s;
    if (symbol_path) s = readFileBytes(symbol_path);
    initCommon(h, gpu_id, d.data(), d.size(), symbol_path ? s.data() : nullptr, s.size(), randomize != 0, enable_print != 0);
  });
}

int tgs_init_from_memory(tgs_sim *h, int gpu_id, const void *design, size_t dn, const void *symbols, size_t sn,
                         int randomize, int enable_print) {
  return guard([&] {
    if (!h || !design) throw Error(TGS_ERR_ARG, "null argument");
    initCommon(h, gpu_id, static_cast<const uint8_t *>(design), dn, static_cast<const uint8_t *>(symbols), sn,
               randomize != 0, enable_print != 0);
  });
}

int tgs_eval(tgs_sim *h, int *stop) {
  return guard([&] {
    requireLoaded(h);
    runCycles(h, uint32_t(h->cycleCnt), 1, 0);
    TGS_CUDA(cudaStreamSynchronize(h->stream));
    checkDeviceError(h);
    vcdDump(h, h->cycleCnt);  // time step = the cycle just evaluated
    h->cycleCnt += 1;
    if (stop) *stop = stopFlag(h);
  });
}

int tgs_eval_free_running(tgs_sim *h, uint32_t cycles, int *stop) {
  return guard([&] {
    requireLoaded(h);
    TGS_CUDA(cudaMemsetAsync(h->profU.p, 0, h->profU.n * sizeof(long long), h->stream));
    TGS_CUDA(cudaMemsetAsync(h->profT.p, 0, h->profT.n * sizeof(long long), h->stream));
    runCycles(h, uint32_t(h->cycleCnt), cycles, kFlagCountCycles | kFlagProfile);
    TGS_CUDA(cudaStreamSynchronize(h->stream));
    checkDeviceError(h);
    if (cycles) vcdDump(h, h->cycleCnt + cycles - 1);  // signals of the last cycle
    h->cycleCnt += cycles;
    if (stop) *stop = stopFlag(h);
  });
}

int tgs_eval_until_stop(tgs_sim *h, uint32_t max_cycles, int *stop, uint32_t *cycles_run) {
  return guard([&] {
    requireLoaded(h);
    uint32_t r0 = 0, r1 = 0;
    TGS_CUDA(cudaMemcpy(&r0, h->realCycles.p, 4, cudaMemcpyDeviceToHost));
    runCycles(h, uint32_t(h->cycleCnt), max_cycles, kFlagCountCycles | kFlagStopExit);
    TGS_CUDA(cudaStreamSynchronize(h->stream));
    checkDeviceError(h);
    TGS_CUDA(cudaMemcpy(&r1, h->realCycles.p, 4, cudaMemcpyDeviceToHost));
    if (r1 != r0) vcdDump(h, h->cycleCnt + (r1 - r0) - 1);
    h->cycleCnt += r1 - r0;
    if (cycles_run) *cycles_run = r1 - r0;
    if (stop) *stop = stopFlag(h);
  });
}

int tgs_set_register(tgs_sim *h, const char *name, uint64_t value) {
  return guard([&] { requireLoaded(h); setRegister(h, 0, name, value); });
}
int tgs_read_register(tgs_sim *h, const char *name, uint64_t *value) {
  return guard([&] {
    requireLoaded(h);
    if (!value) throw Error(TGS_ERR_ARG, "null output");
    *value = readRegister(h, 0, name);
  });
}
int tgs_set_register_stream(tgs_sim *h, uint32_t s, const char *name, uint64_t value) {
  return guard([&] { requireLoaded(h); setRegister(h, s, name, value); });
}
int tgs_read_register_stream(tgs_sim *h, uint32_t s, const char *name, uint64_t *value) {
  return guard([&] {
    requireLoaded(h);
    if (!value) throw Error(TGS_ERR_ARG, "null output");
    *value = readRegister(h, s, name);
  });
}

int tgs_read_registers(tgs_sim *h, uint32_t stream, const char *const *names, uint32_t n, uint64_t *values) {
  return guard([&] {
    requireLoaded(h);
    readRegisters(h, stream, names, n, values);
  });
}

int tgs_read_signal(tgs_sim *h, const char *name, uint64_t *value) {
  return guard([&] {
    requireLoaded(h);
    if (!name || !value) throw Error(TGS_ERR_ARG, "null argument");
    *value = readSignal(h, 0, name);
  });
}

int tgs_read_signal_stream(tgs_sim *h, uint32_t stream, const char *name, uint64_t *value) {
  return guard([&] {
    requireLoaded(h);
    if (!name || !value) throw Error(TGS_ERR_ARG, "null argument");
    *value = readSignal(h, stream, name);
  });
}

int tgs_enable_vcd(tgs_sim *h, const char *path) {
  return guard([&] {
    requireLoaded(h);
    if (!path) throw Error(TGS_ERR_ARG, "null path");
    enableVcd(h, path);
  });
}

int tgs_get_real_cycles(tgs_sim *h, uint32_t *c) {
  return guard([&] {
    requireLoaded(h);
    if (!c) throw Error(TGS_ERR_ARG, "null output");
    TGS_CUDA(cudaMemcpy(c, h->realCycles.p, sizeof(uint32_t), cudaMemcpyDeviceToHost));
  });
}
int tgs_get_cycle_cnt(tgs_sim *h, uint64_t *c) {
  return guard([&] {
    requireLoaded(h);
    if (!c) throw Error(TGS_ERR_ARG, "null output");
    *c = h->cycleCnt;
  });
}
int tgs_set_enable_print(tgs_sim *h, int en) {
  return guard([&] {
    requireLoaded(h);
    h->enablePrint = en != 0;
    h->kp.enablePrint = en ? 1 : 0;
  });
}
int tgs_get_eval_done(tgs_sim *h, int *stop) {
  return guard([&] {
    requireLoaded(h);
    if (!stop) throw Error(TGS_ERR_ARG, "null output");
    *stop = stopFlag(h);
  });
}

int tgs_copy_profile_data(tgs_sim *h, int64_t *useful, int64_t *total, size_t count) {
  return guard([&] {
    requireLoaded(h);
    if (count > h->design.parts.size()) throw Error(TGS_ERR_RANGE, "count beyond partition count");
    if (useful) TGS_CUDA(cudaMemcpy(useful, h->profU.p, count * sizeof(int64_t), cudaMemcpyDeviceToHost));
    if (total) TGS_CUDA(cudaMemcpy(total, h->profT.p, count * sizeof(int64_t), cudaMemcpyDeviceToHost));
  });
}

int tgs_get_pool_sizes(const tgs_sim *h, uint32_t *r, uint32_t *m, uint32_t *e) {
  return guard([&] {
    if (!h || !h->loaded) throw Error(TGS_ERR_STATE, "simulator not initialised");
    if (r) *r = h->design.regPoolSize;
    if (m) *m = h->design.memPoolSize;
    if (e) *e = h->design.exchangePoolSize;
  });
}

int tgs_read_reg_pool(tgs_sim *h, uint32_t s, uint8_t *out, size_t bytes) {
  return guard([&] {
    requireLoaded(h);
    if (!out || bytes != h->design.regPoolSize) throw Error(TGS_ERR_ARG, "buffer must hold regPoolSize bytes");
    uint32_t g, k;
    streamPos(h, s, g, k);
    h->ioBytes.alloc(std::max<size_t>(h->ioBytes.n, h->regSlots));
    TGS_CUDA(launchGatherRegs(h->regs.p, h->regSlots, h->gpad, g, k, h->ioBytes.p, h->stream));
    TGS_CUDA(cudaMemcpyAsync(out, h->ioBytes.p, bytes, cudaMemcpyDeviceToHost, h->stream));
    TGS_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int tgs_write_reg_pool(tgs_sim *h, uint32_t s, const uint8_t *in, size_t bytes) {
  return guard([&] {
    requireLoaded(h);
    if (!in || bytes != h->design.regPoolSize) throw Error(TGS_ERR_ARG, "buffer must hold regPoolSize bytes");
    uint32_t g, k;
    streamPos(h, s, g, k);
    std::vector<uint8_t> buf(h->regSlots, 0);
    std::memcpy(buf.data(), in, bytes);
    // keep the padding slots as they are: read them first
    std::vector<uint8_t> cur(h->regSlots);
    h->ioBytes.alloc(std::max<size_t>(h->ioBytes.n, h->regSlots));
    TGS_CUDA(launchGatherRegs(h->regs.p, h->regSlots, h->gpad, g, k, h->ioBytes.p, h->stream));
    TGS_CUDA(cudaMemcpyAsync(cur.data(), h->ioBytes.p, h->regSlots, cudaMemcpyDeviceToHost, h->stream));
    TGS_CUDA(cudaStreamSynchronize(h->stream));
    for (size_t i = bytes; i < h->regSlots; ++i) buf[i] = cur[i];
    h->ioBytes.upload(buf, h->stream);
    TGS_CUDA(launchScatterRegs(h->regs.p, h->regSlots, h->gpad, g, k, h->ioBytes.p, h->stream));
    TGS_CUDA(cudaStreamSynchronize(h->stream));
  });
}

int tgs_read_mem_pool(tgs_sim *h, uint32_t s, uint8_t *out, size_t bytes) {
  return guard([&] {
    requireLoaded(h);
    if (!out || bytes != h->design.memPoolSize) throw Error(TGS_ERR_ARG, "buffer must hold memPoolSize bytes");
    if (s >= h->nStreams) throw Error(TGS_ERR_ARG, "stream index out of range");
    TGS_CUDA(cudaMemcpy(out, h->mems.p + size_t(s) * h->memStride, bytes, cudaMemcpyDeviceToHost));
  });
}

int tgs_write_mem_pool(tgs_sim *h, uint32_t s, const uint8_t *in, size_t bytes) {
  return guard([&] {
    requireLoaded(h);
    if (!in || bytes != h->design.memPoolSize) throw Error(TGS_ERR_ARG, "buffer must hold memPoolSize bytes");
    if (s >= h->nStreams) throw Error(TGS_ERR_ARG, "stream index out of range");
    TGS_CUDA(cudaMemcpy(h->mems.p + size_t(s) * h->memStride, in, bytes, cudaMemcpyHostToDevice));
  });
}

namespace {

constexpr char kStateMagic[8] = {'T', 'G', 'S', 'S', 'T', 'A', 'T', 'E'};
constexpr uint32_t kStateVersion = 1;

struct StateHeader {
  char magic[8];
  uint32_t version, nStreams;
  uint64_t fingerprint;
  uint32_t regPoolSize, pad0;
  uint64_t memPoolSize;
  uint64_t cycleCnt, batchCycle;
  uint32_t realCycles, pad1;
};
static_assert(sizeof(StateHeader) == 64, "state header");

// Structure of the design (pool sizes, partitions, ops per level): enough to
// refuse a checkpoint of another design.
uint64_t designFingerprint(const SimDesignInfo &d) {
  uint64_t h = 0x243F6A8885A308D3ull;
  auto add = [&](uint64_t v) { h = mix64(h ^ v); };
  add(d.regPoolSize);
  add(d.memPoolSize);
  add(d.exchangePoolSize);
  add(d.parts.size());
  for (const auto &p : d.parts) {
    add(p.valuePoolSize);
    add(p.ops_l0_regRead.size() | (uint64_t(p.ops_l0_exchangeRead.size()) << 32));
    add(p.exec_mParts.size());
    for (const auto &lv : p.exec_mParts) add(lv.size());
  }
  return h;
}

}  // namespace

int tgs_dump_state(tgs_sim *h, const char *path) {
  return guard([&] {
    requireLoaded(h);
    if (!path) throw Error(TGS_ERR_ARG, "null path");
    std::ofstream o(path, std::ios::binary);
    if (!o) throw Error(TGS_ERR_IO, std::string("cannot write ") + path);
    const uint32_t n = h->nStreams;
    StateHeader hd{};
    std::memcpy(hd.magic, kStateMagic, 8);
    hd.version = kStateVersion;
    hd.nStreams = n;
    hd.fingerprint = designFingerprint(h->design);
    hd.regPoolSize = h->design.regPoolSize;
    hd.memPoolSize = h->design.memPoolSize;
    hd.cycleCnt = h->cycleCnt;
    hd.batchCycle = h->batchCycle;
    TGS_CUDA(cudaMemcpy(&hd.realCycles, h->realCycles.p, 4, cudaMemcpyDeviceToHost));
    o.write(reinterpret_cast<const char *>(&hd), sizeof(hd));
    std::vector<uint32_t> stop(n), stopCycle(n);
    std::vector<unsigned long long> roll(n);
    TGS_CUDA(cudaMemcpy(stop.data(), h->stop.p, n * 4ull, cudaMemcpyDeviceToHost));
    TGS_CUDA(cudaMemcpy(stopCycle.data(), h->stopCycle.p, n * 4ull, cudaMemcpyDeviceToHost));
    TGS_CUDA(cudaMemcpy(roll.data(), h->roll.p, n * 8ull, cudaMemcpyDeviceToHost));
    o.write(reinterpret_cast<const char *>(stop.data()), n * 4ull);
    o.write(reinterpret_cast<const char *>(stopCycle.data()), n * 4ull);
    o.write(reinterpret_cast<const char *>(roll.data()), n * 8ull);
    h->ioBytes.alloc(std::max<size_t>(h->ioBytes.n, h->regSlots));
    std::vector<uint8_t> buf(std::max<size_t>(h->regSlots, size_t(1) << 24));
    for (uint32_t st = 0; st < n; ++st) {
      uint32_t g, k;
      streamPos(h, st, g, k);
      TGS_CUDA(launchGatherRegs(h->regs.p, h->regSlots, h->gpad, g, k, h->ioBytes.p, h->stream));
      TGS_CUDA(cudaMemcpyAsync(buf.data(), h->ioBytes.p, hd.regPoolSize, cudaMemcpyDeviceToHost, h->stream));
      TGS_CUDA(cudaStreamSynchronize(h->stream));
      o.write(reinterpret_cast<const char *>(buf.data()), hd.regPoolSize);
    }
    for (uint32_t st = 0; st < n; ++st)
      for (uint64_t off = 0; off < hd.memPoolSize; off += buf.size()) {
        const size_t len = size_t(std::min<uint64_t>(buf.size(), hd.memPoolSize - off));
        TGS_CUDA(cudaMemcpy(buf.data(), h->mems.p + size_t(st) * h->memStride + off, len, cudaMemcpyDeviceToHost));
        o.write(reinterpret_cast<const char *>(buf.data()), std::streamsize(len));
      }
    if (!o) throw Error(TGS_ERR_IO, std::string("write failed: ") + path);
  });
}

int tgs_load_state(tgs_sim *h, const char *path) {
  return guard([&] {
    requireLoaded(h);
    if (!path) throw Error(TGS_ERR_ARG, "null path");
    std::ifstream in(path, std::ios::binary);
    if (!in) throw Error(TGS_ERR_IO, std::string("cannot read ") + path);
    StateHeader hd{};
    in.read(reinterpret_cast<char *>(&hd), sizeof(hd));
    if (!in || std::memcmp(hd.magic, kStateMagic, 8) != 0 || hd.version != kStateVersion)
      throw Error(TGS_ERR_FORMAT, std::string("not a state file: ") + path);
    if (hd.fingerprint != designFingerprint(h->design) || hd.regPoolSize != h->design.regPoolSize ||
        hd.memPoolSize != h->design.memPoolSize)
      throw Error(TGS_ERR_ARG, "state file of another design");
    if (hd.nStreams == 0) throw Error(TGS_ERR_FORMAT, "state file without streams");
    const uint32_t n = hd.nStreams;
    // the file must hold every stream the header announces before the
    // handle is reconfigured or its state touched: a truncated or corrupt
    // file leaves the handle as it was
    {
      const std::streampos here = in.tellg();
      in.seekg(0, std::ios::end);
      const uint64_t size = uint64_t(in.tellg());
      in.seekg(here);
      const uint64_t perStream = 16ull + hd.regPoolSize + hd.memPoolSize;
      if (!in || n > (size - sizeof(StateHeader)) / perStream || size != sizeof(StateHeader) + uint64_t(n) * perStream)
        throw Error(TGS_ERR_FORMAT, "state file size does not match its header");
    }
    std::vector<uint32_t> stop(n), stopCycle(n);
    std::vector<unsigned long long> roll(n);
    in.read(reinterpret_cast<char *>(stop.data()), n * 4ull);
    in.read(reinterpret_cast<char *>(stopCycle.data()), n * 4ull);
    in.read(reinterpret_cast<char *>(roll.data()), n * 8ull);
    if (!in) throw Error(TGS_ERR_FORMAT, "truncated state file");
    if (h->opt.n_streams != n) {
      h->opt.n_streams = n;
      configure(h);
    }
    resetState(h);  // padding slots and words take their initial values
    h->ioBytes.alloc(std::max<size_t>(h->ioBytes.n, h->regSlots));
    std::vector<uint8_t> buf(std::max<size_t>(h->regSlots, size_t(1) << 24));
    for (uint32_t st = 0; st < n; ++st) {
      uint32_t g, k;
      streamPos(h, st, g, k);
      in.read(reinterpret_cast<char *>(buf.data()), hd.regPoolSize);
      if (!in) throw Error(TGS_ERR_FORMAT, "truncated state file");
      // padding slots past regPoolSize keep their current (initial) values
      TGS_CUDA(launchGatherRegs(h->regs.p, h->regSlots, h->gpad, g, k, h->ioBytes.p, h->stream));
      TGS_CUDA(cudaMemcpyAsync(buf.data() + hd.regPoolSize, h->ioBytes.p + hd.regPoolSize,
                               h->regSlots - hd.regPoolSize, cudaMemcpyDeviceToHost, h->stream));
      TGS_CUDA(cudaStreamSynchronize(h->stream));
      TGS_CUDA(cudaMemcpyAsync(h->ioBytes.p, buf.data(), h->regSlots, cudaMemcpyHostToDevice, h->stream));
      TGS_CUDA(launchScatterRegs(h->regs.p, h->regSlots, h->gpad, g, k, h->ioBytes.p, h->stream));
      TGS_CUDA(cudaStreamSynchronize(h->stream));
    }
    for (uint32_t st = 0; st < n; ++st)
      for (uint64_t off = 0; off < hd.memPoolSize; off += buf.size()) {
        const size_t len = size_t(std::min<uint64_t>(buf.size(), hd.memPoolSize - off));
        in.read(reinterpret_cast<char *>(buf.data()), std::streamsize(len));
        if (!in) throw Error(TGS_ERR_FORMAT, "truncated state file");
        TGS_CUDA(cudaMemcpy(h->mems.p + size_t(st) * h->memStride + off, buf.data(), len, cudaMemcpyHostToDevice));
      }
    TGS_CUDA(cudaMemcpy(h->stop.p, stop.data(), n * 4ull, cudaMemcpyHostToDevice));
    TGS_CUDA(cudaMemcpy(h->stopCycle.p, stopCycle.data(), n * 4ull, cudaMemcpyHostToDevice));
    TGS_CUDA(cudaMemcpy(h->roll.p, roll.data(), n * 8ull, cudaMemcpyHostToDevice));
    TGS_CUDA(cudaMemcpy(h->realCycles.p, &hd.realCycles, 4, cudaMemcpyHostToDevice));
    h->cycleCnt = hd.cycleCnt;
    h->batchCycle = hd.batchCycle;
  });
}

int tgs_state_digest(tgs_sim *h, uint32_t s, uint64_t *rd, uint64_t *md) {
  return guard([&] {
    requireLoaded(h);
    if (s >= h->nStreams) throw Error(TGS_ERR_ARG, "stream index out of range");
    TGS_CUDA(cudaMemsetAsync(h->outA.p, 0, h->nStreams * 8, h->stream));
    TGS_CUDA(cudaMemsetAsync(h->outB.p, 0, h->nStreams * 8, h->stream));
    TGS_CUDA(launchRegDigest(int(h->spw), h->regs.p, h->design.regPoolSize, h->gpad, h->nStreams, h->outA.p, h->stream));
    TGS_CUDA(launchMemDigest(h->mems.p, h->memStride, h->design.memPoolSize, h->nStreams, h->outB.p, h->stream));
    unsigned long long a = 0, b = 0;
    TGS_CUDA(cudaMemcpyAsync(&a, h->outA.p + s, 8, cudaMemcpyDeviceToHost, h->stream));
    TGS_CUDA(cudaMemcpyAsync(&b, h->outB.p + s, 8, cudaMemcpyDeviceToHost, h->stream));
    TGS_CUDA(cudaStreamSynchronize(h->stream));
    if (rd) *rd = a;
    if (md) *md = b;
  });
}

int tgs_reset_state(tgs_sim *h) {
  return guard([&] {
    requireLoaded(h);
    resetState(h);
    h->cycleCnt = 0;
    h->batchCycle = 0;
  });
}

int tgs_batch_run(tgs_sim *h, const tgs_batch *job, tgs_batch_result *res) {
  return guard([&] {
    requireLoaded(h);
    batchRun(h, job, res);
  });
}

int tgs_default_gen_config(tgs_gen_config *c) {
  return guard([&] {
    if (!c) throw Error(TGS_ERR_ARG, "null config");
    std::memset(c, 0, sizeof(*c));
    c->seed = 1;
    c->n_lut = 4096;
    c->levels = 16;
    c->operands = 2;
    c->ff_bits = 512;
    c->pi_bits = 32;
    c->n_mems = 1;
    c->mem_depth = 1024;
    c->mem_width = 32;
    c->mem_read_ports = 1;
    c->mem_write_ports = 1;
    c->vec_nibbles = 8;
    c->max_fanout = 4096;
    c->luts_per_part = 2048;
    c->mpart_width = 32;
    c->cone_depth = 1;
  });
}

int tgs_generate(const tgs_gen_config *cfg, const char *design_path, const char *symbol_path, tgs_gen_info *info) {
  return guard([&] {
    if (!cfg || !design_path) throw Error(TGS_ERR_ARG, "null argument");
    SimDesignInfo d;
    SimDebugInfo s;
    generateDesign(*cfg, d, s, info);
    {
      std::ofstream o(design_path, std::ios::binary);
      if (!o) throw Error(TGS_ERR_IO, std::string("cannot write ") + design_path);
      serializeSimDesignInfo(o, d);
      if (!o) throw Error(TGS_ERR_IO, std::string("write failed: ") + design_path);
    }
    if (symbol_path) {
      std::ofstream o(symbol_path, std::ios::binary);
      if (!o) throw Error(TGS_ERR_IO, std::string("cannot write ") + symbol_path);
      serializeSimDebugInfo(o, s);
    }
  });
}

int tgs_validate_file(const char *design_path, const char *symbol_path, uint64_t *lut_ops) {
  return guard([&] {
    if (!design_path) throw Error(TGS_ERR_ARG, "null argument");
    auto bytes = readFileBytes(design_path);
    SimDesignInfo d;
    SimDebugInfo s;
    parseDesign(bytes.data(), bytes.size(), d);
    if (symbol_path) {
      auto sb = readFileBytes(symbol_path);
      parseSymbols(sb.data(), sb.size(), s);
    }
    d.Init();
    auto vi = validateDesign(d, symbol_path ? &s : nullptr);
    if (lut_ops) *lut_ops = vi.lutOps;
  });
}

}  // extern "C"

namespace tgs {

namespace {

void checkStimulus(tgs_sim *h, const tgs_stimulus *st) {
  for (auto &pd : h->img.parts)
    if (pd.copyKind == 1)
      for (uint32_t i = 0; i < st->n_inputs; ++i)
        if (st->reg[i] >= pd.copyDst && st->reg[i] < pd.copyDst + pd.copySlots)
          throw Error(TGS_ERR_ARG, "stimulus register " + std::to_string(st->reg[i]) + " is written by the design");
  for (uint32_t i = 0; i < st->n_inputs; ++i) {
    if (st->reg[i] >= h->design.regPoolSize) throw Error(TGS_ERR_RANGE, "stimulus register beyond regPool");
    if (st->bits[i] < 1 || st->bits[i] > 4) throw Error(TGS_ERR_RANGE, "stimulus bit width outside 1..4");
  }
}

// Stimulus and digests run beside the regions: registers must be read-only
// in region 0 and unread in region 1.
void checkRegionRoles(tgs_sim *h) {
  for (auto &pd : h->img.parts) {
    if (pd.region == 0 && pd.copyKind == 1)
      throw Error(TGS_ERR_INVALID_DESIGN, "region 0 writes registers: stimulus/digest runs need region-0 register writes to be absent");
    if (pd.region == 1 && pd.l0Exchange == 0 && pd.l0Count)
      throw Error(TGS_ERR_INVALID_DESIGN, "region 1 reads registers: stimulus/digest runs need region 1 to read only the exchange pool");
  }
}

float runTimed(tgs_sim *h, uint32_t c0, uint32_t n, uint32_t flags) {
  cudaEvent_t e0, e1;
  TGS_CUDA(cudaEventCreate(&e0));
  TGS_CUDA(cudaEventCreate(&e1));
  TGS_CUDA(cudaEventRecord(e0, h->stream));
  runCycles(h, c0, n, flags);
  TGS_CUDA(cudaEventRecord(e1, h->stream));
  TGS_CUDA(cudaEventSynchronize(e1));
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  TGS_CUDA(cudaStreamSynchronize(h->stream));
  checkDeviceError(h);
  return ms;
}

// Admission: streams queued onto S resident slots.  The kernel finds each
// cycle's retirements (length reached or, with stop exit, a stop in the
// previous cycle) and admits the next queued streams, longest first, in place.
void batchAdmission(tgs_sim *h, const tgs_batch *job, tgs_batch_result *res, uint32_t flags) {
  const uint32_t n = job->n_streams;
  // default slot count: enough that the queue's work fills the longest
  // stream's run (longest first keeps that stream from finishing late);
  // more slots only make every cycle wider
  uint64_t total = 0, longest = 1;
  for (uint32_t q = 0; q < n; ++q) {
    total += job->cycles[q];
    longest = std::max<uint64_t>(longest, job->cycles[q]);
  }
  uint32_t S = job->slots ? job->slots
                          : uint32_t(std::clamp<uint64_t>((total + longest - 1) / longest, 8, 4096));
  S = std::min(S, n);
  if (S > 1) S = (S + 7) / 8 * 8;
  if (S > 32u * kMaxSlotWords) throw Error(TGS_ERR_ARG, "queued batches run on at most 4096 slots");
  if (res && (res->final_regs || res->final_mems))
    throw Error(TGS_ERR_ARG, "final_regs / final_mems need every stream resident (slots >= n_streams, equal lengths)");
  if (job->stim && job->stim->table) throw Error(TGS_ERR_ARG, "stimulus tables need every stream resident and equally long");
  for (uint32_t q = 0; q < n; ++q)
    if (job->cycles[q] == 0) throw Error(TGS_ERR_ARG, "stream lengths must be at least one cycle");
  // retiring streams' memories are digested in region 0 and reset in region 1
  for (auto &pd : h->img.parts)
    if (pd.region == 0 && pd.memWCount)
      throw Error(TGS_ERR_INVALID_DESIGN, "region 0 writes memories: in-place admission needs memory writes in region 1 only");
  if (h->opt.n_streams != S) {
    h->opt.n_streams = S;
    configure(h);
  }
  // Streams are admitted longest first (LPT): every stream's results are
  // independent of when it runs, and the longest ones no longer start late
  // and run on alone.
  std::vector<uint32_t> order(n);
  std::iota(order.begin(), order.end(), 0u);
  std::stable_sort(order.begin(), order.end(), [&](uint32_t a, uint32_t b) { return job->cycles[a] > job->cycles[b]; });
  std::vector<uint32_t> slotStream(S, kNoStream), slotStart(S, 0), slotRetire(S, 0xFFFFFFFFu);
  // launch length: the queue's end without stops (min-heap of (retire
  // cycle, slot); a slot freed in cycle t takes its next stream from t + 1).
  // Shorter streams (stops) never end the queue later: a stream's start
  // cycle only grows with the lengths before it.
  using E = std::pair<uint64_t, uint32_t>;
  std::priority_queue<E, std::vector<E>, std::greater<E>> pq;
  uint32_t firstRetire = 0xFFFFFFFFu;
  for (uint32_t s = 0; s < S && s < n; ++s) {
    const uint32_t q = order[s];
    slotStream[s] = q;
    slotRetire[s] = job->cycles[q];
    firstRetire = std::min(firstRetire, job->cycles[q]);
    pq.push({job->cycles[q], s});
  }
  uint64_t last = 0;
  for (uint32_t nextQ = std::min(S, n); !pq.empty();) {
    auto [t, s] = pq.top();
    pq.pop();
    last = std::max(last, t);
    if (nextQ < n) pq.push({t + 1 + job->cycles[order[nextQ++]], s});
  }
  if (last >= 0xFFFFFFF0ull) throw Error(TGS_ERR_RANGE, "job too long for 32-bit cycle counters");
  std::vector<uint32_t> lens(job->cycles, job->cycles + n);
  std::vector<unsigned long long> seeds(n);
  for (uint32_t q = 0; q < n; ++q) seeds[q] = mix64((job->stim ? job->stim->base_seed : 0) ^ q);

  resetState(h);
  fillParams(h);
  KParams &p = h->kp;
  cudaStream_t st = h->stream;
  h->slotStream.upload(slotStream, st);
  h->slotStart.upload(slotStart, st);
  h->slotRetire.upload(slotRetire, st);
  h->jobLen.upload(lens, st);
  h->jobSeed.upload(seeds, st);
  h->queueOrder.upload(order, st);
  h->retList.alloc(S);
  const uint32_t admW[8] = {std::min(S, n), 0, 0, 0, firstRetire, firstRetire, 0xFFFFFFFFu, 0xFFFFFFFFu};
  h->admW.alloc(8);
  TGS_CUDA(cudaMemcpyAsync(h->admW.p, admW, sizeof(admW), cudaMemcpyHostToDevice, st));
  h->retireMask.alloc(h->gpad);
  h->memAcc.alloc(S);
  h->outReg.alloc(n);
  h->outMem.alloc(n);
  h->outRoll.alloc(n);
  h->outStop.alloc(n);
  TGS_CUDA(cudaMemsetAsync(h->retireMask.p, 0, h->gpad * 4, st));
  TGS_CUDA(cudaMemsetAsync(h->memAcc.p, 0, S * 8ull, st));
  TGS_CUDA(cudaMemsetAsync(h->digAcc.p, 0, S * 8ull, st));
  TGS_CUDA(cudaMemsetAsync(h->roll.p, 0, S * 8ull, st));
  p.slotStream = h->slotStream.p;
  p.slotStart = h->slotStart.p;
  p.slotRetire = h->slotRetire.p;
  p.jobLen = h->jobLen.p;
  p.jobSeed = h->jobSeed.p;
  p.queueOrder = h->queueOrder.p;
  p.queueHead = h->admW.p;
  p.queueSnap = h->admW.p + 1;
  p.retList = h->retList.p;
  p.retCount = h->admW.p + 2;
  p.nDone = h->admW.p + 3;
  p.eventHint = h->admW.p + 4;
  p.retireMask = h->retireMask.p;
  p.memAcc = h->memAcc.p;
  p.outReg = h->outReg.p;
  p.outMem = h->outMem.p;
  p.outRoll = h->outRoll.p;
  p.outStop = h->outStop.p;
  p.nJobs = n;
  p.streamSeed = h->jobSeed.p;
  if (flags & kFlagStimulus) {
    p.nStim = job->stim->n_inputs;
    p.stimReg = h->stimReg.p;
    p.stimBits = h->stimBits.p;
    p.stimToggle = job->stim->toggle ? h->stimToggle.p : nullptr;
  }
  const bool perCycle = (job->flags & TGS_BATCH_CYCLE_DIGESTS) && res && res->cycle_digest && res->cycle_stride;
  if (perCycle) {
    h->cycDig.alloc(size_t(n) * res->cycle_stride);
    TGS_CUDA(cudaMemsetAsync(h->cycDig.p, 0, size_t(n) * res->cycle_stride * 8, st));
    p.cycDig = h->cycDig.p;
    p.cycStride = res->cycle_stride;
  }
  const float ms = runTimed(h, 0, uint32_t(last) + 1, flags | kFlagSlots);
  h->cycleCnt = last + 1;
  if (!res) return;
  res->device_ms = ms;
  res->stream_cycles = total;
  if (flags & kFlagStopExit) {
    // a stream that stopped ran through its stop cycle
    std::vector<uint32_t> stops(n);
    TGS_CUDA(cudaMemcpyAsync(stops.data(), h->outStop.p, n * 4ull, cudaMemcpyDeviceToHost, st));
    TGS_CUDA(cudaStreamSynchronize(st));
    res->stream_cycles = 0;
    for (uint32_t q = 0; q < n; ++q)
      res->stream_cycles += stops[q] == 0xFFFFFFFFu ? job->cycles[q] : std::min<uint64_t>(job->cycles[q], stops[q] + 1ull);
  }
  res->launches = h->lastLaunches;
  if (res->final_reg_digest) TGS_CUDA(cudaMemcpyAsync(res->final_reg_digest, h->outReg.p, n * 8ull, cudaMemcpyDeviceToHost, st));
  if (res->final_mem_digest) TGS_CUDA(cudaMemcpyAsync(res->final_mem_digest, h->outMem.p, n * 8ull, cudaMemcpyDeviceToHost, st));
  if (res->rolling_digest) TGS_CUDA(cudaMemcpyAsync(res->rolling_digest, h->outRoll.p, n * 8ull, cudaMemcpyDeviceToHost, st));
  if (res->stop_cycle) TGS_CUDA(cudaMemcpyAsync(res->stop_cycle, h->outStop.p, n * 4ull, cudaMemcpyDeviceToHost, st));
  if (perCycle)
    TGS_CUDA(cudaMemcpyAsync(res->cycle_digest, h->cycDig.p, size_t(n) * res->cycle_stride * 8, cudaMemcpyDeviceToHost, st));
  TGS_CUDA(cudaStreamSynchronize(st));
}

}  // namespace

// Streams of a job run from the initial state (or, with TGS_BATCH_CONTINUE,
// from the previous call's state and cycle) for cycles[s] cycles each.
void batchRun(tgs_sim *h, const tgs_batch *job, tgs_batch_result *res) {
  if (!job || !job->cycles || job->n_streams == 0) throw Error(TGS_ERR_ARG, "empty batch");
  const uint32_t n = job->n_streams;
  const tgs_stimulus *st = job->stim;
  uint32_t flags = 0;
  if (st && st->n_inputs) {
    flags |= kFlagStimulus;
    checkStimulus(h, st);
  }
  const bool wantDigest = (job->flags & (TGS_BATCH_CYCLE_DIGESTS | TGS_BATCH_ROLLING)) != 0;
  if (wantDigest) flags |= kFlagDigest;
  if (job->flags & TGS_BATCH_STOP_EXIT) flags |= kFlagStopExit;
  if (flags) checkRegionRoles(h);
  if (flags & kFlagStimulus) {
    h->stimReg.upload(st->reg, st->n_inputs, h->stream);
    h->stimBits.upload(st->bits, st->n_inputs, h->stream);
    if (st->toggle) h->stimToggle.upload(st->toggle, st->n_inputs, h->stream);
  }
  bool equal = true;
  for (uint32_t s = 1; s < n; ++s) equal &= job->cycles[s] == job->cycles[0];
  const bool admission = !equal || (job->slots && job->slots < n);
  if (admission) {
    if (job->flags & TGS_BATCH_CONTINUE) throw Error(TGS_ERR_ARG, "TGS_BATCH_CONTINUE needs every stream resident");
    fillParams(h);  // refreshed below after any reconfiguration
    batchAdmission(h, job, res, flags);
    return;
  }
  const uint32_t cyc = job->cycles[0];
  const bool cont = (job->flags & TGS_BATCH_CONTINUE) != 0;
  if (cont && h->opt.n_streams != n) throw Error(TGS_ERR_STATE, "TGS_BATCH_CONTINUE with a different stream count");
  if (h->opt.n_streams != n) {
    h->opt.n_streams = n;
    configure(h);
  }
  if (!cont) {
    resetState(h);
    h->batchCycle = 0;
    TGS_CUDA(cudaMemsetAsync(h->roll.p, 0, n * 8ull, h->stream));
  }
  fillParams(h);
  KParams &p = h->kp;
  const uint32_t c0 = uint32_t(h->batchCycle);
  if (flags & kFlagStimulus) {
    p.nStim = st->n_inputs;
    p.stimReg = h->stimReg.p;
    p.stimBits = h->stimBits.p;
    p.stimToggle = st->toggle ? h->stimToggle.p : nullptr;
    std::vector<unsigned long long> seeds(n);
    for (uint32_t s = 0; s < n; ++s) seeds[s] = mix64(st->base_seed ^ s);
    h->seeds.upload(seeds, h->stream);
    p.streamSeed = h->seeds.p;
    if (st->table) {
      h->stimTable.upload(st->table, size_t(cyc) * st->n_inputs * n, h->stream);
      p.stimTable = h->stimTable.p;
      p.stimTableC0 = c0;
    }
  }
  TGS_CUDA(cudaMemsetAsync(h->digAcc.p, 0, n * 8ull, h->stream));
  const bool perCycle = (job->flags & TGS_BATCH_CYCLE_DIGESTS) && res && res->cycle_digest && res->cycle_stride;
  if (perCycle) {
    h->cycDig.alloc(size_t(n) * res->cycle_stride);
    TGS_CUDA(cudaMemsetAsync(h->cycDig.p, 0, size_t(n) * res->cycle_stride * 8, h->stream));
    p.cycDig = h->cycDig.p;
    p.cycStride = res->cycle_stride;
    p.cycBase = c0;
  }
  const float ms = runTimed(h, c0, cyc, flags);
  h->batchCycle += cyc;
  h->cycleCnt = h->batchCycle;
  if (!res) return;
  res->device_ms = ms;
  res->stream_cycles = uint64_t(cyc) * n;
  if (flags & kFlagStopExit) {
    // a stream that stopped ran up to and including its stop cycle
    std::vector<uint32_t> sc(n);
    TGS_CUDA(cudaMemcpy(sc.data(), h->stopCycle.p, n * 4ull, cudaMemcpyDeviceToHost));
    res->stream_cycles = 0;
    for (uint32_t q = 0; q < n; ++q)
      res->stream_cycles += sc[q] == 0xFFFFFFFFu ? cyc : (sc[q] >= c0 ? sc[q] + 1 - c0 : 0);
  }
  res->launches = h->lastLaunches;
  cudaStream_t s = h->stream;
  if (res->final_reg_digest || res->final_mem_digest) {
    TGS_CUDA(cudaMemsetAsync(h->outA.p, 0, n * 8ull, s));
    TGS_CUDA(cudaMemsetAsync(h->outB.p, 0, n * 8ull, s));
    if (res->final_reg_digest) {
      TGS_CUDA(launchRegDigest(int(h->spw), h->regs.p, h->design.regPoolSize, h->gpad, n, h->outA.p, s));
      TGS_CUDA(cudaMemcpyAsync(res->final_reg_digest, h->outA.p, n * 8ull, cudaMemcpyDeviceToHost, s));
    }
    if (res->final_mem_digest) {
      TGS_CUDA(launchMemDigest(h->mems.p, h->memStride, h->design.memPoolSize, n, h->outB.p, s));
      TGS_CUDA(cudaMemcpyAsync(res->final_mem_digest, h->outB.p, n * 8ull, cudaMemcpyDeviceToHost, s));
    }
  }
  if (res->rolling_digest) TGS_CUDA(cudaMemcpyAsync(res->rolling_digest, h->roll.p, n * 8ull, cudaMemcpyDeviceToHost, s));
  if (perCycle)
    TGS_CUDA(cudaMemcpyAsync(res->cycle_digest, h->cycDig.p, size_t(n) * res->cycle_stride * 8, cudaMemcpyDeviceToHost, s));
  if (res->stop_cycle) TGS_CUDA(cudaMemcpyAsync(res->stop_cycle, h->stopCycle.p, n * 4ull, cudaMemcpyDeviceToHost, s));
  TGS_CUDA(cudaStreamSynchronize(s));
  if (res->final_regs || res->final_mems) {
    for (uint32_t q = 0; q < n; ++q) {
      uint32_t g = q / h->spw, k = q % h->spw;
      if (res->final_regs) {
        h->ioBytes.alloc(std::max<size_t>(h->ioBytes.n, h->regSlots));
        TGS_CUDA(launchGatherRegs(h->regs.p, h->regSlots, h->gpad, g, k, h->ioBytes.p, s));
        TGS_CUDA(cudaMemcpyAsync(res->final_regs + size_t(q) * h->design.regPoolSize, h->ioBytes.p,
                                 h->design.regPoolSize, cudaMemcpyDeviceToHost, s));
        TGS_CUDA(cudaStreamSynchronize(s));
      }
      if (res->final_mems)
        TGS_CUDA(cudaMemcpy(res->final_mems + size_t(q) * h->design.memPoolSize, h->mems.p + size_t(q) * h->memStride,
                            h->design.memPoolSize, cudaMemcpyDeviceToHost));
    }
  }
}

}  // namespace tgs

namespace tgs {
const SimDesignInfo &designOf(const tgs_sim *h) { return h->design; }
const SimDebugInfo &symbolsOf(const tgs_sim *h) { return h->symbols; }
}  // namespace tgs

extern "C" int tgs_get_design_stats(const tgs_sim *h, tgs_design_stats *o) {
  return guard([&] {
    if (!h || !o) throw Error(TGS_ERR_ARG, "null argument");
    if (!h->loaded) throw Error(TGS_ERR_STATE, "simulator not initialised");
    std::memset(o, 0, sizeof(*o));
    uint64_t slots = 0;
    for (const auto &p : h->design.parts) {
      o->l0_reg_reads += p.ops_l0_regRead.size();
      o->l0_exg_reads += p.ops_l0_exchangeRead.size();
      o->max_exec_levels = std::max<uint32_t>(o->max_exec_levels, uint32_t(p.exec_mParts.size()));
      for (const auto &lvl : p.exec_mParts)
        for (const auto &m : lvl) {
          ++o->mparts;
          slots += 1;  // header word
          if (m.isLUTPart) {
            for (const auto &t : m.topLevel) (t.lutIndex ? o->lut_ops : o->nop_ops)++;
            for (const auto &l : m.middleLevels)
              for (const auto &op : l) (op.lutIndex() ? o->lut_ops : o->nop_ops)++;
            o->writeback_ops += m.lastLevel.size();
          }
          o->vec_read_ops += m.vecRead.size();
          o->vec_ops += m.vecArithAndLogic.size();
          o->mem_read_ops += m.memRead.size();
        }
      if (p.op_last_exchangeWrite.count) {
        o->exg_copy_slots += (lastLevelExchangeOp(p).count + 3) / 4 * 4;
      } else {
        if (p.op_last_regWrite.count) o->reg_copy_slots += (p.op_last_regWrite.count + 3) / 4 * 4;
        o->mem_write_ops += p.ops_last_memWrite.size();
        o->print_ops += p.ops_last_print.size();
        o->stop_ops += p.ops_last_stop.size();
      }
      slots += (p.op_last_regWrite.count || p.op_last_exchangeWrite.count) ? 1 : 0;
    }
    o->op_slots = slots + o->lut_ops + o->nop_ops + o->writeback_ops + o->l0_reg_reads + o->l0_exg_reads + o->mem_read_ops +
                  o->mem_write_ops + o->vec_ops + o->vec_read_ops + o->print_ops + o->stop_ops;
    o->partitions = uint32_t(h->design.parts.size());
    o->max_value_pool = h->img.maxVpSlots;
    o->blocks = h->lc.blocks;
    o->threads = h->lc.threads;
    o->groups_per_item = uint32_t(h->lc.G);
    o->streams_per_word = h->spw;
    o->block_barriers = h->sched.barriers;
    o->exec_levels = h->sched.levels;
    o->fused_levels = uint32_t(h->sched.fusedLevels);
    o->makespan[0] = h->sched.makespan[0];
    o->makespan[1] = h->sched.makespan[1];
    o->smem_per_block = uint32_t(h->lc.smem);
    o->stage_words = h->stageWords;
    o->resident_words = h->resWords;
  });
}

extern "C" int tgs_resave_design(const char *in, const char *out) {
  return guard([&] {
    if (!in || !out) throw Error(TGS_ERR_ARG, "null argument");
    auto bytes = readFileBytes(in);
    SimDesignInfo d;
    parseDesign(bytes.data(), bytes.size(), d);
    std::ofstream o(out, std::ios::binary);
    if (!o) throw Error(TGS_ERR_IO, std::string("cannot write ") + out);
    serializeSimDesignInfo(o, d);
  });
}

extern "C" int tgs_compact_design(const char *in, const char *out, uint32_t *maxBefore, uint32_t *maxAfter) {
  return guard([&] {
    if (!in || !out) throw Error(TGS_ERR_ARG, "null argument");
    auto bytes = readFileBytes(in);
    SimDesignInfo d;
    parseDesign(bytes.data(), bytes.size(), d);
    uint32_t before = 0, after = 0;
    for (auto &p : d.parts) {
      before = std::max(before, p.valuePoolSize);
      std::vector<uint32_t> newOf;
      const uint32_t n = planSlots(p, newOf);
      if (n <= 65534) renameSlots(p, newOf, n);
      after = std::max(after, p.valuePoolSize);
    }
    if (maxBefore) *maxBefore = before;
    if (maxAfter) *maxAfter = after;
    std::ofstream o(out, std::ios::binary);
    if (!o) throw Error(TGS_ERR_IO, std::string("cannot write ") + out);
    serializeSimDesignInfo(o, d);
  });
}

extern "C" int tgs_pack_design(const char *in, const char *out, uint32_t *mparts_before, uint32_t *mparts_after) {
  return guard([&] {
    if (!in || !out) throw Error(TGS_ERR_ARG, "null argument");
    auto bytes = readFileBytes(in);
    SimDesignInfo d;
    parseDesign(bytes.data(), bytes.size(), d);
    uint32_t before = 0, after = 0;
    for (auto &p : d.parts)
      for (auto &lvl : p.exec_mParts) {
        before += uint32_t(lvl.size());
        lvl = packLevel(lvl);
        after += uint32_t(lvl.size());
      }
    if (mparts_before) *mparts_before = before;
    if (mparts_after) *mparts_after = after;
    std::ofstream o(out, std::ios::binary);
    if (!o) throw Error(TGS_ERR_IO, std::string("cannot write ") + out);
    serializeSimDesignInfo(o, d);
  });
}

extern "C" int tgs_plan_schedule(const char *path, uint32_t warps, uint32_t groups, uint32_t mpartLanes,
                                 uint32_t levelsPerBarrier, int lanePacking, int fastLuts, uint32_t nStreams,
                                 tgs_schedule_stats *stats) {
  return guard([&] {
    if (!path || !stats) throw Error(TGS_ERR_ARG, "null argument");
    if (warps < 1 || warps > 32) throw Error(TGS_ERR_ARG, "warps must be 1 to 32");
    if (groups != 1 && groups != 2 && groups != 4 && groups != 8) throw Error(TGS_ERR_ARG, "groups must be 1, 2, 4 or 8");
    SchedOpts so;
    so.unitLanes = mpartLanes ? mpartLanes : 32u;
    so.levelsPerBarrier = levelsPerBarrier ? levelsPerBarrier : 1u;
    if (so.unitLanes != 32 && so.unitLanes != 64 && so.unitLanes != 128)
      throw Error(TGS_ERR_ARG, "mpart_lanes must be 32, 64 or 128");
    if (so.levelsPerBarrier != 1 && so.levelsPerBarrier != 2 && so.levelsPerBarrier != 4)
      throw Error(TGS_ERR_ARG, "levels_per_barrier must be 1, 2 or 4");
    auto bytes = readFileBytes(path);
    SimDesignInfo d;
    parseDesign(bytes.data(), bytes.size(), d);
    validateDesign(d, nullptr);  // the static checks tgs_init runs before building the image
    DeviceImage img;
    buildImage(d, img, true, nullptr, lanePacking == 0, fastLuts == 0 && nStreams > 1);
    Schedule s;
    buildSchedule(d, img, warps, groups, nullptr, 1, 1, s, so);
    tgs_schedule_stats st;
    std::memset(&st, 0, sizeof st);
    for (const auto &p : d.parts) st.exec_levels += p.exec_mParts.size();
    st.blocks = s.levels;
    st.barriers = s.barriers;
    st.fused_levels = s.fusedLevels;
    st.schedule_words = s.words.size();
    st.max_level_words = s.maxLevelWords;
    st.makespan = s.planMakespan;
    st.work = s.planWork;
    st.level_bound = s.planLower;
    st.list_bound = s.planUpper;
    *stats = st;
  });
}

extern "C" int tgs_repack_design(const char *in, const char *out, int lanePacking, int fastLuts,
                                 tgs_repack_stats *stats) {
  return guard([&] {
    if (!in || !out) throw Error(TGS_ERR_ARG, "null argument");
    auto bytes = readFileBytes(in);
    SimDesignInfo d;
    parseDesign(bytes.data(), bytes.size(), d);
    tgs_repack_stats st;
    std::memset(&st, 0, sizeof st);
    FastLuts fl(d.lut);
    FastLuts *fast = fastLuts && d.lut.size() == kLutSize ? &fl : nullptr;
    for (auto &p : d.parts)
      for (auto &lvl : p.exec_mParts) {
        st.exec_levels += 1;
        st.mparts_before += lvl.size();
        if (lanePacking) lvl = packLevel(lvl);
        if (fast) lvl = regroupLevel(lvl, fast);
        st.mparts_after += lvl.size();
        for (auto &m : lvl) {
          if (!m.isLUTPart) continue;
          uint64_t luts = 0;
          bool wordWide = fast && !m.topLevel.empty();
          for (auto &o : m.topLevel) {
            luts += o.lutIndex != 0;
            wordWide = wordWide && fast->code(o) != 0;
          }
          for (auto &lv : m.middleLevels)
            for (auto &o : lv) st.lut_ops += o.lutIndex() != 0;
          st.lut_ops += luts;
          if (wordWide) {
            st.fast_lut_ops += luts;
            st.fast_mparts += 1;
          }
        }
      }
    if (stats) *stats = st;
    std::ofstream o(out, std::ios::binary);
    if (!o) throw Error(TGS_ERR_IO, std::string("cannot write ") + out);
    serializeSimDesignInfo(o, d);
  });
}

extern "C" int tgs_resave_symbols(const char *in, const char *out) {
  return guard([&] {
    if (!in || !out) throw Error(TGS_ERR_ARG, "null argument");
    auto bytes = readFileBytes(in);
    SimDebugInfo s;
    parseSymbols(bytes.data(), bytes.size(), s);
    std::ofstream o(out, std::ios::binary);
    if (!o) throw Error(TGS_ERR_IO, std::string("cannot write ") + out);
    serializeSimDebugInfo(o, s);
  });
}

extern "C" int tgs_initial_state(const char *design_path, const char *symbol_path, int randomize, uint8_t *regs,
                                 size_t reg_bytes, uint8_t *mems, size_t mem_bytes) {
  return guard([&] {
    if (!design_path) throw Error(TGS_ERR_ARG, "null argument");
    auto bytes = readFileBytes(design_path);
    SimDesignInfo d;
    SimDebugInfo s;
    parseDesign(bytes.data(), bytes.size(), d);
    if (symbol_path) {
      auto sb = readFileBytes(symbol_path);
      parseSymbols(sb.data(), sb.size(), s);
    }
    d.Init();
    if (randomize) d.Randomize(0, s);
    if (reg_bytes != d.regPool.size() || mem_bytes != d.memPool.size())
      throw Error(TGS_ERR_ARG, "buffers must hold regPoolSize and memPoolSize bytes");
    if (regs && reg_bytes) std::memcpy(regs, d.regPool.data(), reg_bytes);
    if (mems && mem_bytes) std::memcpy(mems, d.memPool.data(), mem_bytes);
  });
}

extern "C" int tgs_host_alloc(size_t bytes, void **out) {
  return guard([&] {
    if (!out) throw Error(TGS_ERR_ARG, "null output");
    TGS_CUDA(cudaHostAlloc(out, bytes ? bytes : 1, cudaHostAllocDefault));
  });
}

extern "C" int tgs_host_free(void *p) {
  return guard([&] {
    if (p) TGS_CUDA(cudaFreeHost(p));
  });
}

extern "C" int tgs_device_reset(int device) {
  return guard([&] {
    TGS_CUDA(cudaSetDevice(device));
    TGS_CUDA(cudaDeviceReset());
  });
}

// ---- learned cost model ---------------------------------------------------------
namespace {
void requireModel(tgs_sim *h) {
  if (!h->model) h->model = std::make_unique<tgs::CostModel>();
}
}  // namespace

extern "C" int tgs_num_mparts(tgs_sim *h, uint32_t *n) {
  return guard([&] {
    requireLoaded(h);
    if (!n) throw Error(TGS_ERR_ARG, "null output");
    *n = h->img.nMParts;
  });
}

extern "C" int tgs_mpart_features(tgs_sim *h, float *features, uint32_t n) {
  return guard([&] {
    requireLoaded(h);
    if (!features || n != h->img.nMParts) throw Error(TGS_ERR_ARG, "features must hold n_mparts x 16 floats");
    for (auto &p : h->img.mp)
      for (auto &l : p)
        for (auto &r : l) featureVector(r.feat, features + size_t(r.id) * kFeatures);
  });
}

extern "C" int tgs_profile_mparts(tgs_sim *h, uint32_t cycles, float *mean_cycles, uint32_t n) {
  return guard([&] {
    requireLoaded(h);
    if (!mean_cycles || n != h->img.nMParts) throw Error(TGS_ERR_ARG, "mean_cycles must hold n_mparts floats");
    h->mpCycles.alloc(n);
    h->mpCount.alloc(n);
    TGS_CUDA(cudaMemsetAsync(h->mpCycles.p, 0, size_t(n) * 8, h->stream));
    TGS_CUDA(cudaMemsetAsync(h->mpCount.p, 0, size_t(n) * 4, h->stream));
    fillParams(h);
    h->kp.mpCycles = h->mpCycles.p;
    h->kp.mpCount = h->mpCount.p;
    runCycles(h, uint32_t(h->cycleCnt), cycles, kFlagProfileMP);
    TGS_CUDA(cudaStreamSynchronize(h->stream));
    checkDeviceError(h);
    h->cycleCnt += cycles;
    std::vector<unsigned long long> c(n);
    std::vector<uint32_t> k(n);
    TGS_CUDA(cudaMemcpy(c.data(), h->mpCycles.p, size_t(n) * 8, cudaMemcpyDeviceToHost));
    TGS_CUDA(cudaMemcpy(k.data(), h->mpCount.p, size_t(n) * 4, cudaMemcpyDeviceToHost));
    // counts are groups evaluated: a whole evaluation covers G of them
    const double G = double(h->lc.G);
    for (uint32_t i = 0; i < n; ++i) mean_cycles[i] = k[i] ? float(double(c[i]) * G / k[i]) : 0.f;
    fillParams(h);
  });
}

extern "C" int tgs_cost_model_train(tgs_sim *h, const float *features, const float *cycles, uint32_t n,
                                    const tgs_train_opts *o, tgs_train_report *rep) {
  return guard([&] {
    requireLoaded(h);
    if (!features || !cycles) throw Error(TGS_ERR_ARG, "null argument");
    requireModel(h);
    tgs_train_opts d{};
    d.epochs = 30;
    d.batch = 1024;
    d.lr = 2e-3f;
    d.seed = 1;
    d.val_frac = 0.2f;
    const tgs_train_opts &t = o ? *o : d;
    auto r = h->model->train(features, cycles, n, t.epochs ? t.epochs : d.epochs, t.batch ? t.batch : d.batch,
                             t.lr > 0 ? t.lr : d.lr, t.seed, t.val_frac);
    if (rep) {
      std::memset(rep, 0, sizeof(*rep));
      rep->train_mse = r.trainMse;
      rep->val_mse = r.valMse;
      rep->val_corr = r.valCorr;
      rep->gate_corr = r.gateCorr;
      rep->samples = r.samples;
      rep->epochs = r.epochs;
      rep->train_ms = r.ms;
    }
    if (h->opt.schedule == TGS_SCHED_LEARNED) {
      configure(h);
      resetState(h);
    }
  });
}

extern "C" int tgs_cost_model_state(tgs_sim *h, float *state, size_t n, int set) {
  return guard([&] {
    if (!h || !state) throw Error(TGS_ERR_ARG, "null argument");
    if (n != size_t(kMlpParams) + 2) throw Error(TGS_ERR_ARG, "cost model state holds 5,315 floats");
    requireModel(h);
    if (set) {
      h->model->setState(std::vector<float>(state, state + n));
      if (h->loaded && h->opt.schedule == TGS_SCHED_LEARNED) {
        TGS_CUDA(cudaSetDevice(h->device));
        configure(h);
        resetState(h);
      }
    } else {
      if (!h->model->trained()) throw Error(TGS_ERR_STATE, "cost model not trained");
      auto s = h->model->state();
      std::memcpy(state, s.data(), n * sizeof(float));
    }
  });
}

extern "C" int tgs_mlp_forward(const float *params, const float *X, uint32_t n, float *out) {
  return guard([&] {
    if (!params || !X || !out) throw Error(TGS_ERR_ARG, "null argument");
    DBuf<float> dp, dx, dy;
    dp.upload(params, kMlpParams, nullptr);
    dx.upload(X, size_t(n) * kFeatures, nullptr);
    dy.alloc(n);
    TGS_CUDA(mlpForward(dp.p, dx.p, n, dy.p, nullptr));
    TGS_CUDA(cudaMemcpy(out, dy.p, size_t(n) * 4, cudaMemcpyDeviceToHost));
  });
}

extern "C" int tgs_mlp_grad(const float *params, const float *X, const float *y, uint32_t n, float *grad, float *loss) {
  return guard([&] {
    if (!params || !X || !y || !grad) throw Error(TGS_ERR_ARG, "null argument");
    DBuf<float> dp, dx, dy, dg, dl;
    dp.upload(params, kMlpParams, nullptr);
    dx.upload(X, size_t(n) * kFeatures, nullptr);
    dy.upload(y, n, nullptr);
    dg.alloc(kMlpParams);
    dl.alloc(1);
    TGS_CUDA(cudaMemset(dg.p, 0, kMlpParams * 4));
    TGS_CUDA(cudaMemset(dl.p, 0, 4));
    TGS_CUDA(mlpGrad(dp.p, dx.p, dy.p, nullptr, n, n ? 1.f / float(n) : 0.f, dg.p, dl.p, nullptr));
    TGS_CUDA(cudaMemcpy(grad, dg.p, kMlpParams * 4, cudaMemcpyDeviceToHost));
    float l = 0;
    TGS_CUDA(cudaMemcpy(&l, dl.p, 4, cudaMemcpyDeviceToHost));
    if (loss) *loss = n ? l / float(n) : 0.f;
  });
}
