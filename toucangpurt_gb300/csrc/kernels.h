// Launch wrappers of the device code (cycle_kernel.cu).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "devimage.h"

namespace tgs {

struct LaunchCfg {
  int spw = 1, G = 1;
  bool res = false;  // exec levels resident in shared memory for the launch
  uint32_t blocks = 1, threads = 256;
  size_t smem = 0;
  cudaStream_t stream = nullptr;
};

void *cycleKernelFor(int spw, int G, bool resident);
void *regionKernelFor(int spw, int G, bool resident);
// instantiated one per translation unit (kernels_*.cu)
void *cycleKernelStaged(int spw, int G);
void *cycleKernelResident(int spw, int G);
void *regionKernelStaged(int spw, int G);
void *regionKernelResident(int spw, int G);
cudaError_t enqueueGraphChunk(const LaunchCfg &c, const KParams &p, uint32_t k, bool admit);
cudaError_t launchStimulus(int spw, const KParams &p, uint32_t cycle, cudaStream_t st);
cudaError_t launchCycles(const LaunchCfg &c, const KParams &p, uint32_t c0, uint32_t n);
cudaError_t launchInitState(int spw, const KParams &p, cudaStream_t st);
cudaError_t launchRegDigest(int spw, const uint32_t *regs, uint32_t slots, uint32_t gpad, uint32_t nStreams,
                            unsigned long long *out, cudaStream_t st);
cudaError_t launchMemDigest(const uint8_t *mems, unsigned long long stride, uint32_t size, uint32_t nStreams,
                            unsigned long long *out, cudaStream_t st);
cudaError_t launchGatherRegs(const uint32_t *regs, uint32_t slots, uint32_t gpad, uint32_t g, uint32_t k, uint8_t *out,
                             cudaStream_t st);
cudaError_t launchScatterRegs(uint32_t *regs, uint32_t slots, uint32_t gpad, uint32_t g, uint32_t k, const uint8_t *in,
                              cudaStream_t st);
cudaError_t launchPeekRegs(const uint32_t *regs, uint32_t gpad, uint32_t g, uint32_t k, const uint32_t *ids,
                           uint8_t *out, uint32_t n, cudaStream_t st);
cudaError_t launchPokeRegs(uint32_t *regs, uint32_t gpad, uint32_t g, uint32_t k, const uint32_t *ids,
                           const uint8_t *vals, uint32_t n, cudaStream_t st);

}  // namespace tgs
