// Small kernels of the cycle loop (graph-form admission, stimulus, cycle
// counter), state utilities, and the host-side launch wrappers.  The cycle
// and region kernels are instantiated in kernels_{persistent,region}_
// {staged,resident}.cu, one translation unit each, so the build compiles
// them in parallel.
#include "cycle_kernel.cuh"

namespace tgs {
namespace {

// Graph form, after region 1 (and the stop-exit inputs): admission (one
// block), cycle bookkeeping, the early-exit word.
template <int SPW>
__global__ void admitKernel(const KParams p, uint32_t k) {
  const uint32_t t = __ldcg(p.graphState) + k;
  // graphState[4] (exit) is written only here, after the cycle's regions
  if (t >= __ldcg(p.graphState + 2) || __ldcg(p.graphState + 4) || __ldcg(p.err)) return;
  const bool slots = (p.flags & kFlagSlots) != 0;
  const bool event = slots && __ldcg(p.retCount) != 0;
  if (event) eventAdmit<SPW>(p, t, threadIdx.x, blockDim.x);
  __syncthreads();
  if (threadIdx.x == 0) {
    if (p.flags & kFlagCountCycles) *p.realCycles += 1;
    if (slots) {
      if (event && __ldcg(p.nDone) >= p.nJobs) p.graphState[4] = 1;
    } else if ((p.flags & kFlagStopExit) && __ldcg(p.nStopped) >= p.nStreams) {
      p.graphState[4] = 1;
    }
  }
}

// Graph form, stop exit: the next cycle's inputs, after the region-1 launch.
template <int SPW>
__global__ void graphStimulusKernel(const KParams p, uint32_t k) {
  const uint32_t t = __ldcg(p.graphState) + k;
  if (t + 1 >= __ldcg(p.graphState + 2) || __ldcg(p.graphState + 4) || __ldcg(p.err)) return;
  applyStimulus<SPW>(p, t + 1, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

__global__ void advanceKernel(uint32_t *counter, uint32_t k) { *counter += k; }

template <int SPW>
__global__ void stimulusKernel(const KParams p, uint32_t cycle) {
  applyStimulus<SPW>(p, cycle, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}

// ---- state utilities -----------------------------------------------------------
template <int SPW>
__global__ void initStateKernel(const KParams p) {
  const size_t n = size_t(p.regSlots) * p.gpad;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < n; i += size_t(gridDim.x) * blockDim.x) {
    const uint32_t v = p.initRegs[i / p.gpad];
    p.regs[i] = SPW == 8 ? rep8(v) : v;
  }
  const size_t ne = size_t(p.exgSlots) * p.gpad;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < ne; i += size_t(gridDim.x) * blockDim.x) p.exg[i] = 0;
}

// Digest of one pool per stream: sum of mix64(i << 8 | v_i).
__global__ void memDigestKernel(const uint8_t *__restrict__ mems, unsigned long long stride, uint32_t size,
                                uint32_t nStreams, unsigned long long *__restrict__ out) {
  const uint32_t s = blockIdx.y;
  if (s >= nStreams) return;
  const uint8_t *m = mems + s * stride;
  unsigned long long acc = 0;
  for (size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x; i < size; i += size_t(gridDim.x) * blockDim.x)
    acc += dmix64((unsigned long long)i << 8 | m[i]);
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(kFull, acc, o);
  if ((threadIdx.x & 31u) == 0) atomicAdd(out + s, acc);
}

template <int SPW>
__global__ void regDigestKernel(const uint32_t *__restrict__ regs, uint32_t slots, uint32_t gpad, uint32_t nStreams,
                                unsigned long long *__restrict__ out) {
  const uint32_t g = blockIdx.y;
  unsigned long long acc[SPW];
#pragma unroll
  for (int k = 0; k < SPW; ++k) acc[k] = 0;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x) {
    const uint32_t w = regs[size_t(i) * gpad + g];
#pragma unroll
    for (int k = 0; k < SPW; ++k) acc[k] += dmix64((unsigned long long)i << 8 | nib(w, k));
  }
#pragma unroll
  for (int k = 0; k < SPW; ++k) {
    unsigned long long a = acc[k];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(kFull, a, o);
    const uint32_t s = g * SPW + k;
    if ((threadIdx.x & 31u) == 0 && s < nStreams) atomicAdd(out + s, a);
  }
}

// nibble k of every register word of group g <-> one byte per register
__global__ void gatherRegsKernel(const uint32_t *__restrict__ regs, uint32_t slots, uint32_t gpad, uint32_t g,
                                 uint32_t k, uint8_t *__restrict__ out) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x)
    out[i] = uint8_t(nib(regs[size_t(i) * gpad + g], k));
}

__global__ void scatterRegsKernel(uint32_t *__restrict__ regs, uint32_t slots, uint32_t gpad, uint32_t g, uint32_t k,
                                  const uint8_t *__restrict__ in) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < slots; i += gridDim.x * blockDim.x) {
    uint32_t *w = regs + size_t(i) * gpad + g;
    *w = (*w & ~(15u << (4 * k))) | ((uint32_t(in[i]) & 15u) << (4 * k));
  }
}

// Writes nibbles (id, value) of one stream.
__global__ void pokeRegsKernel(uint32_t *__restrict__ regs, uint32_t gpad, uint32_t g, uint32_t k,
                               const uint32_t *__restrict__ ids, const uint8_t *__restrict__ vals, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    uint32_t *w = regs + size_t(ids[i]) * gpad + g;
    *w = (*w & ~(15u << (4 * k))) | ((uint32_t(vals[i]) & 15u) << (4 * k));
  }
}

// The nibbles of the listed register ids of one stream (readRegister).
__global__ void peekRegsKernel(const uint32_t *__restrict__ regs, uint32_t gpad, uint32_t g, uint32_t k,
                               const uint32_t *__restrict__ ids, uint8_t *__restrict__ out, uint32_t n) {
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    out[i] = uint8_t(nib(regs[size_t(ids[i]) * gpad + g], k));
}

}  // namespace

void *cycleKernelFor(int spw, int G, bool resident) {
  return resident ? cycleKernelResident(spw, G) : cycleKernelStaged(spw, G);
}

cudaError_t launchCycles(const LaunchCfg &c, const KParams &p, uint32_t c0, uint32_t n) {
  void *fn = cycleKernelFor(c.spw, c.G, c.res);
  KParams pp = p;
  void *args[] = {&pp, &c0, &n};
  return cudaLaunchCooperativeKernel(fn, dim3(c.blocks), dim3(c.threads), args, c.smem, c.stream);
}

void *regionKernelFor(int spw, int G, bool resident) {
  return resident ? regionKernelResident(spw, G) : regionKernelStaged(spw, G);
}

// Enqueues one chunk of k cycles in graph form on the stream (captured by
// the caller): per cycle region 0, region 1 and (admission / cycle count)
// the admit kernel; then the cycle counter advance.
cudaError_t enqueueGraphChunk(const LaunchCfg &c, const KParams &p, uint32_t k, bool admit) {
  void *fn = regionKernelFor(c.spw, c.G, c.res);
  KParams pp = p;
  for (uint32_t i = 0; i < k; ++i) {
    for (uint32_t r = 0; r < 2; ++r) {
      uint32_t ki = i, ri = r;
      void *args[] = {&pp, &ki, &ri};
      cudaError_t e = cudaLaunchKernel(fn, dim3(c.blocks), dim3(c.threads), args, c.smem, c.stream);
      if (e != cudaSuccess) return e;
    }
    if ((p.flags & kFlagStopExit) && (p.flags & kFlagStimulus)) {
      const uint32_t n = std::max<uint32_t>(1, p.nStim * p.gpad);
      const uint32_t blocks = std::min<uint32_t>(1024, (n + 255) / 256);
      if (c.spw == 8)
        graphStimulusKernel<8><<<blocks, 256, 0, c.stream>>>(p, i);
      else
        graphStimulusKernel<1><<<blocks, 256, 0, c.stream>>>(p, i);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
    if (admit) {
      if (c.spw == 8)
        admitKernel<8><<<1, 256, 0, c.stream>>>(p, i);
      else
        admitKernel<1><<<1, 256, 0, c.stream>>>(p, i);
      cudaError_t e = cudaGetLastError();
      if (e != cudaSuccess) return e;
    }
  }
  advanceKernel<<<1, 1, 0, c.stream>>>(p.graphState, k);
  return cudaGetLastError();
}

cudaError_t launchStimulus(int spw, const KParams &p, uint32_t cycle, cudaStream_t st) {
  const uint32_t n = std::max<uint32_t>(1, p.nStim * p.gpad);
  const uint32_t blocks = std::min<uint32_t>(1024, (n + 255) / 256);
  if (spw == 8)
    stimulusKernel<8><<<blocks, 256, 0, st>>>(p, cycle);
  else
    stimulusKernel<1><<<blocks, 256, 0, st>>>(p, cycle);
  return cudaGetLastError();
}

cudaError_t launchInitState(int spw, const KParams &p, cudaStream_t st) {
  const size_t n = size_t(p.regSlots) * p.gpad;
  const uint32_t blocks = uint32_t(std::min<size_t>(4096, (n + 255) / 256 + 1));
  if (spw == 8)
    initStateKernel<8><<<blocks, 256, 0, st>>>(p);
  else
    initStateKernel<1><<<blocks, 256, 0, st>>>(p);
  return cudaGetLastError();
}

cudaError_t launchRegDigest(int spw, const uint32_t *regs, uint32_t slots, uint32_t gpad, uint32_t nStreams,
                            unsigned long long *out, cudaStream_t st) {
  dim3 grid(std::max<uint32_t>(1, std::min<uint32_t>(64, (slots + 255) / 256)), gpad);
  if (spw == 8)
    regDigestKernel<8><<<grid, 256, 0, st>>>(regs, slots, gpad, nStreams, out);
  else
    regDigestKernel<1><<<grid, 256, 0, st>>>(regs, slots, gpad, nStreams, out);
  return cudaGetLastError();
}

cudaError_t launchMemDigest(const uint8_t *mems, unsigned long long stride, uint32_t size, uint32_t nStreams,
                            unsigned long long *out, cudaStream_t st) {
  if (size == 0 || nStreams == 0) return cudaSuccess;
  dim3 grid(std::max<uint32_t>(1, std::min<uint32_t>(1024, (size + 255) / 256)), nStreams);
  memDigestKernel<<<grid, 256, 0, st>>>(mems, stride, size, nStreams, out);
  return cudaGetLastError();
}

cudaError_t launchGatherRegs(const uint32_t *regs, uint32_t slots, uint32_t gpad, uint32_t g, uint32_t k, uint8_t *out,
                             cudaStream_t st) {
  gatherRegsKernel<<<std::max<uint32_t>(1, std::min<uint32_t>(1024, (slots + 255) / 256)), 256, 0, st>>>(regs, slots, gpad, g, k, out);
  return cudaGetLastError();
}

cudaError_t launchScatterRegs(uint32_t *regs, uint32_t slots, uint32_t gpad, uint32_t g, uint32_t k, const uint8_t *in,
                              cudaStream_t st) {
  scatterRegsKernel<<<std::max<uint32_t>(1, std::min<uint32_t>(1024, (slots + 255) / 256)), 256, 0, st>>>(regs, slots, gpad, g, k, in);
  return cudaGetLastError();
}

cudaError_t launchPeekRegs(const uint32_t *regs, uint32_t gpad, uint32_t g, uint32_t k, const uint32_t *ids,
                           uint8_t *out, uint32_t n, cudaStream_t st) {
  if (!n) return cudaSuccess;
  peekRegsKernel<<<std::max<uint32_t>(1, std::min<uint32_t>(1024, (n + 255) / 256)), 256, 0, st>>>(regs, gpad, g, k, ids, out, n);
  return cudaGetLastError();
}

cudaError_t launchPokeRegs(uint32_t *regs, uint32_t gpad, uint32_t g, uint32_t k, const uint32_t *ids,
                           const uint8_t *vals, uint32_t n, cudaStream_t st) {
  if (!n) return cudaSuccess;
  pokeRegsKernel<<<std::max<uint32_t>(1, std::min<uint32_t>(1024, (n + 255) / 256)), 256, 0, st>>>(regs, gpad, g, k, ids, vals, n);
  return cudaGetLastError();
}

}  // namespace tgs
