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
// or evalFreeRunningNCycles[_Large] (ToucanSim.cu:232-267).  The layout
// (ref_layout.h) is checked on the CPU against the reference's own host code
// (ref_layout_main.cpp, tests/test_ref_layout.py).
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
#include "ref_layout.h"

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

// The layout on the GPU: device buffers and the cubin's __device__ globals.
struct CudaSink : reflayout::Sink {
  Module &M;
  std::vector<CUdeviceptr> &owned;
  CudaSink(Module &m, std::vector<CUdeviceptr> &o) : M(m), owned(o) {}
  uint64_t upload(const void *d, size_t n) override { return ::upload(d, n, owned); }
  void setGlobal(const char *name, const void *d, size_t n) override { CK(cuMemcpyHtoD(M.global(name, n), d, n)); }
};

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
    CudaSink sink(M, owned);
    const reflayout::Layout L = reflayout::build(d, sink);
    const CUdeviceptr regDev = L.reg, memDev = L.mem, exgDev = L.exg;
    const size_t maxVp = L.maxVp;
    const uint32_t n0 = L.n0, n1 = L.n1;
    std::vector<uint8_t> zeros(d.exchangePoolSize, 0);
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
