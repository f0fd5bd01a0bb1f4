// Drives the reference's own GPU kernels on the GB300.
//
// TEST INFRASTRUCTURE ONLY: generates the golden fixtures that pin the CPU
// oracle to the reference implementation.  oracle/Makefile compiles the
// reference's src/SimEval.cu (from its own tree, unmodified) into
// oracle/_ref/ref_simeval.cubin; this program loads that cubin through the
// CUDA driver API, builds the device netlist exactly as the reference's
// host code copy_netlist_to_gpu / copyMicroPartToNetlist lays it out
// (src/SimEval.cu:69-148,1114-1343; restated here field by field), sets the
// kernels' __device__ globals, and launches evalSingleCycle (one cycle per
// cooperative launch, as ToucanSimulator::eval does, src/ToucanSim.cu:206-230)
// or evalFreeRunningNCycles[_Large] (ToucanSim.cu:232-267).
//
// Stimulus is applied between cycles on the host, as a reference testbench
// does with setRegister (the hash is the oracle's, toucan_oracle.h).
//
//   refgpu <cubin> <design.bin> <symbols.bin|-> <randomize> <mode eval|free> <cycles> <streams>
//          <stimulus.txt|-> <out.jsonl>
//   stimulus.txt: "base_seed n" then n lines "reg bits toggle"
#include <cuda.h>

#include <cstddef>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iterator>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "ToucanGPUGenDataTypes.h"

using namespace toucanGPUSim;

namespace {

#define CK(x)                                                                         \
  do {                                                                                \
    CUresult r_ = (x);                                                                \
    if (r_ != CUDA_SUCCESS) {                                                         \
      const char *s_ = nullptr;                                                       \
      cuGetErrorString(r_, &s_);                                                      \
      throw std::runtime_error(std::string(#x) + ": " + (s_ ? s_ : "?"));             \
    }                                                                                 \
  } while (0)

// Device structs of the reference (src/SimEval.cu:152-187), pointer fields as
// 64-bit device addresses.
struct RefPartPtrs {
  uint64_t valuePool;
  uint16_t valuePoolSize;
  uint64_t constVecPool;
  uint64_t netlist;
  uint64_t lastLevelNetlistPtr;
  uint32_t numOpsL0RegRead;
  uint32_t numOpsL0ExgRead;
  uint32_t numExecLevels;
  uint64_t execMPartLevelInfo;
  uint32_t numOpsLastExgWrite;
  uint32_t numOpsLastRegWrite;
  uint32_t numOpsLastMemWrite;
  uint32_t numOpsLastPrint;
  uint32_t numOpsLastStop;
};
static_assert(sizeof(RefPartPtrs) == 88 && offsetof(RefPartPtrs, netlist) == 24 &&
                  offsetof(RefPartPtrs, execMPartLevelInfo) == 56 && offsetof(RefPartPtrs, numOpsLastStop) == 80,
              "SimPartitionPtrs layout");
struct RefLevelInfo {
  uint32_t numMParts;
  uint64_t mPartInfo;
};
static_assert(sizeof(RefLevelInfo) == 16, "SimMPartLevelInfo layout");
struct RefMPartPtr {
  uint32_t netlistOffset, netlistSize;
};

constexpr uint32_t kMagicLut = 0xfb709394u, kMagicVecRead = 0xfb809917u, kMagicMemRead = 0xccccccccu,
                   kMagicVecOp = 0xbeef1234u;
constexpr size_t kMaxLevels = 160, kLutSize = 4642;

uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
uint64_t digest(const std::vector<uint8_t> &p) {
  uint64_t s = 0;
  for (size_t i = 0; i < p.size(); ++i) s += mix64((uint64_t(i) << 8) | p[i]);
  return s;
}

template <typename T>
void appendRaw(std::vector<char> &b, const std::vector<T> &v) {
  const char *d = reinterpret_cast<const char *>(v.data());
  b.insert(b.end(), d, d + v.size() * sizeof(T));
}
void appendU32(std::vector<char> &b, uint32_t v) {
  const char *d = reinterpret_cast<const char *>(&v);
  b.insert(b.end(), d, d + 4);
}
// chunk padded to 16 bytes (appendToNetlistVec, SimEval.cu:1148-1154)
void appendPadded(std::vector<char> &net, const char *d, size_t n) {
  net.insert(net.end(), d, d + n);
  for (size_t i = 0; i < (16 - n % 16) % 16; ++i) net.push_back(0);
}

// copyMicroPartToNetlist (SimEval.cu:69-148)
std::vector<char> mpartBytes(const CGMicroPartInfo &m) {
  std::vector<char> b;
  if (m.isLUTPart) {
    appendU32(b, kMagicLut);
    appendU32(b, uint32_t(m.middleLevels.size()));
    std::vector<char> sizes(kMaxLevels, 0);
    sizes[0] = char(m.topLevel.size());
    for (size_t i = 0; i < m.middleLevels.size(); ++i) sizes[1 + i] = char(m.middleLevels[i].size());
    sizes[1 + m.middleLevels.size()] = char(m.lastLevel.size());
    b.insert(b.end(), sizes.begin(), sizes.end());
    appendRaw(b, m.topLevel);
    for (auto &l : m.middleLevels) appendRaw(b, l);
    appendRaw(b, m.lastLevel);
  } else if (!m.vecRead.empty()) {
    appendU32(b, kMagicVecRead);
    appendU32(b, uint32_t(m.vecRead.size()));
    appendRaw(b, m.vecRead);
  } else if (!m.vecArithAndLogic.empty()) {
    appendU32(b, kMagicVecOp);
    appendU32(b, uint32_t(m.vecArithAndLogic.size()));
    appendRaw(b, m.vecArithAndLogic);
  } else {
    appendU32(b, kMagicMemRead);
    appendU32(b, uint32_t(m.memRead.size()));
    appendRaw(b, m.memRead);
  }
  return b;
}

struct Module {
  CUmodule mod;
  CUfunction single, freeRun, freeLarge;
  CUdeviceptr global(const char *name, size_t expect = 0) {
    CUdeviceptr p;
    size_t n;
    CK(cuModuleGetGlobal(&p, &n, mod, name));
    if (expect && n != expect) throw std::runtime_error(std::string("global size mismatch: ") + name);
    return p;
  }
};

CUdeviceptr upload(const void *d, size_t n, std::vector<CUdeviceptr> &owned) {
  CUdeviceptr p;
  CK(cuMemAlloc(&p, n ? n : 16));
  if (n) CK(cuMemcpyHtoD(p, d, n));
  owned.push_back(p);
  return p;
}

struct Stim {
  uint64_t seed = 0;
  std::vector<uint32_t> reg;
  std::vector<uint8_t> bits;
  std::vector<uint16_t> toggle;
};

void applyStim(const Stim &st, uint64_t streamSeed, uint32_t c, std::vector<uint8_t> &regs) {
  for (uint32_t i = 0; i < st.reg.size(); ++i) {
    uint64_t h = mix64(streamSeed ^ mix64((uint64_t(c) << 32) | i));
    uint8_t mask = uint8_t((1u << st.bits[i]) - 1);
    if (st.toggle[i] == 0)
      regs[st.reg[i]] = uint8_t(h & mask);
    else if ((h >> 48) < st.toggle[i])
      regs[st.reg[i]] ^= mask;
  }
}

std::string hex(uint64_t v) {
  char b[24];
  std::snprintf(b, sizeof b, "\"%016llx\"", (unsigned long long)v);
  return b;
}

}  // namespace

int main(int argc, char **argv) {
  if (argc != 10) {
    std::fprintf(stderr, "usage: refgpu cubin design symbols randomize mode cycles streams stim out\n");
    return 2;
  }
  try {
    const std::string cubin = argv[1], designPath = argv[2], symPath = argv[3], mode = argv[5], stimPath = argv[8];
    const bool randomize = std::atoi(argv[4]) != 0;
    const uint32_t cycles = uint32_t(std::strtoul(argv[6], nullptr, 10)), streams = uint32_t(std::strtoul(argv[7], nullptr, 10));
    SimDesignInfo d;
    SimDebugInfo sym;
    {
      std::ifstream f(designPath, std::ios::binary);
      if (!f) throw std::runtime_error("cannot open design");
      deserializeSimDesignInfo(f, d);
    }
    if (symPath != "-") {
      std::ifstream f(symPath, std::ios::binary);
      if (!f) throw std::runtime_error("cannot open symbols");
      deserializeSimDebugInfo(f, sym);
    }
    d.Init();
    if (randomize) d.Randomize(0, sym);
    Stim st;
    if (stimPath != "-") {
      std::ifstream f(stimPath);
      size_t n;
      f >> st.seed >> n;
      for (size_t i = 0; i < n; ++i) {
        uint32_t r, b, t;
        f >> r >> b >> t;
        st.reg.push_back(r);
        st.bits.push_back(uint8_t(b));
        st.toggle.push_back(uint16_t(t));
      }
    }

    CK(cuInit(0));
    CUdevice dev;
    CK(cuDeviceGet(&dev, 0));
    CUcontext ctx;
    CK(cuDevicePrimaryCtxRetain(&ctx, dev));
    CK(cuCtxSetCurrent(ctx));
    Module M;
    CK(cuModuleLoad(&M.mod, cubin.c_str()));
    CK(cuModuleGetFunction(&M.single, M.mod, "_Z15evalSingleCyclev"));
    CK(cuModuleGetFunction(&M.freeRun, M.mod, "_Z22evalFreeRunningNCyclesj"));
    CK(cuModuleGetFunction(&M.freeLarge, M.mod, "_Z28evalFreeRunningNCycles_Largej"));
    std::vector<CUdeviceptr> owned;

    // ---- copy_netlist_to_gpu -------------------------------------------
    if (d.lut.size() != kLutSize) throw std::runtime_error("lut size");
    CK(cuMemcpyHtoD(M.global("lutContent", kLutSize), d.lut.data(), kLutSize));
    CUdeviceptr regDev = upload(d.regPool.data(), d.regPoolSize, owned);
    CUdeviceptr memDev = upload(d.memPool.data(), d.memPoolSize, owned);
    std::vector<uint8_t> zeros(d.exchangePoolSize, 0);
    CUdeviceptr exgDev = upload(zeros.data(), zeros.size(), owned);
    CK(cuMemcpyHtoD(M.global("regPool", 8), &regDev, 8));
    CK(cuMemcpyHtoD(M.global("memPool", 8), &memDev, 8));
    CK(cuMemcpyHtoD(M.global("exchangePool", 8), &exgDev, 8));

    std::vector<RefPartPtrs> parts;
    size_t maxVp = 0;
    for (const auto &p : d.parts) {
      RefPartPtrs pp;
      std::memset(&pp, 0, sizeof pp);
      std::vector<char> net;
      pp.valuePool = upload(p.valuePool.data(), p.valuePoolSize, owned);
      pp.valuePoolSize = uint16_t(p.valuePoolSize);
      maxVp = std::max<size_t>(maxVp, p.valuePoolSize);
      pp.constVecPool = p.constVecPool.empty() ? 0 : upload(p.constVecPool.data(), p.constVecPool.size(), owned);
      pp.numOpsL0RegRead = uint32_t(p.ops_l0_regRead.size());
      if (pp.numOpsL0RegRead)
        appendPadded(net, reinterpret_cast<const char *>(p.ops_l0_regRead.data()), p.ops_l0_regRead.size() * 8);
      pp.numOpsL0ExgRead = uint32_t(p.ops_l0_exchangeRead.size());
      if (pp.numOpsL0ExgRead)
        appendPadded(net, reinterpret_cast<const char *>(p.ops_l0_exchangeRead.data()), p.ops_l0_exchangeRead.size() * 8);
      std::vector<RefLevelInfo> levels;
      for (const auto &lvl : p.exec_mParts) {
        std::vector<RefMPartPtr> ptrs;
        for (const auto &m : lvl) {
          auto b = mpartBytes(m);
          ptrs.push_back({uint32_t(net.size()), uint32_t(b.size())});
          appendPadded(net, b.data(), b.size());
        }
        RefLevelInfo li;
        std::memset(&li, 0, sizeof li);
        li.numMParts = uint32_t(ptrs.size());
        li.mPartInfo = ptrs.empty() ? 0 : upload(ptrs.data(), ptrs.size() * sizeof(RefMPartPtr), owned);
        levels.push_back(li);
      }
      pp.numExecLevels = uint32_t(levels.size());
      pp.execMPartLevelInfo = levels.empty() ? 0 : upload(levels.data(), levels.size() * sizeof(RefLevelInfo), owned);
      pp.numOpsLastRegWrite = p.op_last_regWrite.count != 0;
      pp.numOpsLastExgWrite = p.op_last_exchangeWrite.count != 0;
      pp.numOpsLastMemWrite = uint32_t(p.ops_last_memWrite.size());
      pp.numOpsLastPrint = uint32_t(p.ops_last_print.size());
      pp.numOpsLastStop = uint32_t(p.ops_last_stop.size());
      size_t lastOff = net.size();
      if (pp.numOpsLastRegWrite) appendPadded(net, reinterpret_cast<const char *>(&p.op_last_regWrite), 8);
      if (pp.numOpsLastExgWrite) appendPadded(net, reinterpret_cast<const char *>(&p.op_last_exchangeWrite), 8);
      if (pp.numOpsLastMemWrite)
        appendPadded(net, reinterpret_cast<const char *>(p.ops_last_memWrite.data()), p.ops_last_memWrite.size() * 24);
      if (pp.numOpsLastPrint)
        appendPadded(net, reinterpret_cast<const char *>(p.ops_last_print.data()), p.ops_last_print.size() * 4);
      if (pp.numOpsLastStop)
        appendPadded(net, reinterpret_cast<const char *>(p.ops_last_stop.data()), p.ops_last_stop.size() * 2);
      pp.netlist = upload(net.data(), net.size(), owned);
      pp.lastLevelNetlistPtr = pp.netlist + lastOff;
      parts.push_back(pp);
    }
    CUdeviceptr partsDev = upload(parts.data(), parts.size() * sizeof(RefPartPtrs), owned);
    CK(cuMemcpyHtoD(M.global("partitions", 8), &partsDev, 8));
    if (d.regionPartitionIds.size() != 2) throw std::runtime_error("exactly two regions required");
    uint32_t n0 = uint32_t(d.regionPartitionIds[0].size()), n1 = uint32_t(d.regionPartitionIds[1].size()),
             nt = uint32_t(d.parts.size());
    CK(cuMemcpyHtoD(M.global("numParts_Region0", 4), &n0, 4));
    CK(cuMemcpyHtoD(M.global("numParts_Region1", 4), &n1, 4));
    CK(cuMemcpyHtoD(M.global("numTotalParts", 4), &nt, 4));
    std::vector<CUdeviceptr> msgPtrs;
    for (auto &s : d.printMsgs) msgPtrs.push_back(upload(s.c_str(), s.size() + 1, owned));
    CUdeviceptr msgsDev = upload(msgPtrs.data(), msgPtrs.size() * 8, owned);
    CK(cuMemcpyHtoD(M.global("printMsgs", 8), &msgsDev, 8));
    uint8_t enablePrint = 0;
    CK(cuMemcpyHtoD(M.global("enablePrint", 1), &enablePrint, 1));
    CUdeviceptr stopDev = M.global("shouldStop", 4), realDev = M.global("realCycles", 4);

    // ---- setupGPU / launch shape (ToucanSim.cu:16-100,188-191) ----------
    int sms = 0;
    CK(cuDeviceGetAttribute(&sms, CU_DEVICE_ATTRIBUTE_MULTIPROCESSOR_COUNT, dev));
    int threads = 1024, occ = 0;
    while (threads > 64) {
      CK(cuOccupancyMaxActiveBlocksPerMultiprocessor(&occ, M.single, threads, 0));
      if (occ > 0) break;
      threads >>= 1;
    }
    for (CUfunction f : {M.single, M.freeRun, M.freeLarge})
      CK(cuFuncSetAttribute(f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES, int(maxVp)));
    uint32_t maxParts = std::max(n0, n1);
    uint32_t gridSingle = std::min<uint32_t>(maxParts, uint32_t(occ * sms));
    uint32_t gridMulti = std::min<uint32_t>(maxParts, uint32_t(sms));

    std::ofstream out(argv[9]);
    std::vector<uint8_t> regs(d.regPoolSize), mems(d.memPoolSize);
    for (uint32_t s = 0; s < streams; ++s) {
      // fresh state for each stream (the reference runs one stimulus per init)
      CK(cuMemcpyHtoD(regDev, d.regPool.data(), d.regPoolSize));
      if (d.memPoolSize) CK(cuMemcpyHtoD(memDev, d.memPool.data(), d.memPoolSize));
      if (!zeros.empty()) CK(cuMemcpyHtoD(exgDev, zeros.data(), zeros.size()));
      uint32_t zero = 0;
      CK(cuMemcpyHtoD(stopDev, &zero, 4));
      CK(cuMemcpyHtoD(realDev, &zero, 4));
      const uint64_t streamSeed = mix64(st.seed ^ s);
      uint64_t roll = 0;
      uint32_t stopCycle = 0xFFFFFFFFu;
      std::ostringstream cyc;
      CUevent ev0, ev1;
      CK(cuEventCreate(&ev0, CU_EVENT_DEFAULT));
      CK(cuEventCreate(&ev1, CU_EVENT_DEFAULT));
      float kernelMs = 0.0f;
      if (mode == "eval") {
        for (uint32_t c = 0; c < cycles; ++c) {
          CK(cuMemcpyDtoH(regs.data(), regDev, regs.size()));
          applyStim(st, streamSeed, c, regs);
          CK(cuMemcpyHtoD(regDev, regs.data(), regs.size()));
          uint64_t dg = digest(regs);
          roll = mix64(roll + dg);
          cyc << (c ? "," : "") << hex(dg);
          void *args[] = {nullptr};
          CK(cuEventRecord(ev0, nullptr));
          CK(cuLaunchCooperativeKernel(M.single, gridSingle, 1, 1, threads, 1, 1, unsigned(maxVp), nullptr, args));
          CK(cuEventRecord(ev1, nullptr));
          CK(cuCtxSynchronize());
          float ms = 0;
          CK(cuEventElapsedTime(&ms, ev0, ev1));
          kernelMs += ms;
          uint32_t stop = 0;
          CK(cuMemcpyDtoH(&stop, stopDev, 4));
          if (stop && stopCycle == 0xFFFFFFFFu) stopCycle = c;
        }
      } else {
        uint32_t n = cycles;
        void *args[] = {&n};
        CUfunction f = maxParts > gridMulti ? M.freeLarge : M.freeRun;
        CK(cuEventRecord(ev0, nullptr));
        CK(cuLaunchCooperativeKernel(f, gridMulti, 1, 1, threads, 1, 1, unsigned(maxVp), nullptr, args));
        CK(cuEventRecord(ev1, nullptr));
        CK(cuCtxSynchronize());
        CK(cuEventElapsedTime(&kernelMs, ev0, ev1));
      }
      CK(cuMemcpyDtoH(regs.data(), regDev, regs.size()));
      if (!mems.empty()) CK(cuMemcpyDtoH(mems.data(), memDev, mems.size()));
      cuEventDestroy(ev0);
      cuEventDestroy(ev1);
      uint32_t real = 0, stop = 0;
      CK(cuMemcpyDtoH(&real, realDev, 4));
      CK(cuMemcpyDtoH(&stop, stopDev, 4));
      out << "{\"stream\": " << s << ", \"mode\": \"" << mode << "\", \"cycles\": " << cycles
          << ", \"final_reg_digest\": " << hex(digest(regs)) << ", \"final_mem_digest\": " << hex(digest(mems))
          << ", \"rolling_digest\": " << hex(roll) << ", \"stop\": " << stop << ", \"stop_cycle\": " << stopCycle
          << ", \"kernel_ms\": " << kernelMs << ", \"large_kernel\": " << (maxParts > gridMulti ? 1 : 0)
          << ", \"real_cycles\": " << real << ", \"threads\": " << threads << ", \"grid_single\": " << gridSingle
          << ", \"grid_multi\": " << gridMulti << ", \"cycle_digests\": [" << cyc.str() << "]";
      auto dump = [&](const char *key, const std::vector<uint8_t> &v) {
        if (v.size() > 65536) return;
        out << ", \"" << key << "\": \"";
        for (uint8_t x : v) out << "0123456789abcdef"[x & 15];
        out << "\"";
      };
      dump("final_regs", regs);
      dump("final_mems", mems);
      out << "}\n";
    }
    for (CUdeviceptr p : owned) cuMemFree(p);
    cuModuleUnload(M.mod);
    cuDevicePrimaryCtxRelease(dev);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "refgpu: %s\n", e.what());
    return 1;
  }
  return 0;
}
