// A test double of the CUDA runtime's host interface, for running the
// reference's host code (copy_netlist_to_gpu) on a machine without a GPU.
//
// TEST INFRASTRUCTURE ONLY: ref_layout_main.cpp links the reference's
// SimEval.cu host code against this library instead of the CUDA runtime.
// "Device" memory is host memory: cudaMalloc allocates and records a buffer,
// copies are memmove, and a __device__ variable is its host shadow object
// (recorded by name when the module registers it), so after the reference's
// host code ran, every buffer and global it wrote can be read back and put in
// canonical form.  Kernel launches are refused; nothing else is provided.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace {

struct Buf {
  uint8_t *p;
  size_t n;
};
std::vector<Buf> &bufs() {
  static std::vector<Buf> b;
  return b;
}
struct Var {
  char *host;
  size_t n;
};
std::map<std::string, Var> &vars() {
  static std::map<std::string, Var> v;
  return v;
}

}  // namespace

extern "C" {

// ---- queries for the test driver ----------------------------------------------
bool fakecuda_resolve(uint64_t addr, const uint8_t **p, size_t *n, size_t *off) {
  for (const Buf &b : bufs()) {
    const uint64_t base = uint64_t(reinterpret_cast<uintptr_t>(b.p));
    if (addr >= base && addr <= base + b.n) {
      *p = b.p;
      *n = b.n;
      *off = size_t(addr - base);
      return true;
    }
  }
  return false;
}
bool fakecuda_global(const char *name, const uint8_t **p, size_t *n) {
  auto it = vars().find(name);
  if (it == vars().end()) return false;
  *p = reinterpret_cast<const uint8_t *>(it->second.host);
  *n = it->second.n;
  return true;
}

// ---- the runtime calls the reference's host code makes ------------------------
cudaError_t cudaMalloc(void **devPtr, size_t size) {
  // 16 bytes at least and never the same address twice, so that an address
  // names one buffer
  auto *p = static_cast<uint8_t *>(std::calloc(size ? size : 16, 1));
  if (!p) return cudaErrorMemoryAllocation;
  bufs().push_back({p, size});
  *devPtr = p;
  return cudaSuccess;
}
cudaError_t cudaFree(void *) { return cudaSuccess; }  // buffers live until exit
cudaError_t cudaMemcpy(void *dst, const void *src, size_t count, enum cudaMemcpyKind) {
  if (count) std::memmove(dst, src, count);
  return cudaSuccess;
}
cudaError_t cudaMemcpyToSymbol(const void *symbol, const void *src, size_t count, size_t offset,
                               enum cudaMemcpyKind) {
  if (count) std::memmove(static_cast<char *>(const_cast<void *>(symbol)) + offset, src, count);
  return cudaSuccess;
}
cudaError_t cudaMemcpyFromSymbol(void *dst, const void *symbol, size_t count, size_t offset, enum cudaMemcpyKind) {
  if (count) std::memmove(dst, static_cast<const char *>(symbol) + offset, count);
  return cudaSuccess;
}
cudaError_t cudaDeviceSynchronize(void) { return cudaSuccess; }
cudaError_t cudaGetLastError(void) { return cudaSuccess; }
const char *cudaGetErrorString(cudaError_t) { return "test-double runtime"; }

// ---- module registration (emitted by nvcc into the host object) ---------------
void **__cudaRegisterFatBinary(void *) {
  static void *handle = nullptr;
  return &handle;
}
void __cudaRegisterFatBinaryEnd(void **) {}
void __cudaUnregisterFatBinary(void **) {}
void __cudaRegisterFunction(void **, const char *, char *, const char *, int, uint3 *, uint3 *, dim3 *, dim3 *,
                            int *) {}
void __cudaRegisterVar(void **, char *hostVar, char *, const char *deviceName, int, size_t size, int, int) {
  vars()[deviceName] = {hostVar, size};
}
char __cudaInitModule(void **) { return 0; }
cudaError_t __cudaPopCallConfiguration(dim3 *, dim3 *, size_t *, void *) { return cudaErrorNotSupported; }
cudaError_t __cudaGetKernel(cudaKernel_t *, const void *) { return cudaErrorNotSupported; }
cudaError_t __cudaLaunchKernel(cudaKernel_t, dim3, dim3, void **, size_t, cudaStream_t) {
  return cudaErrorNotSupported;
}

}  // extern "C"
