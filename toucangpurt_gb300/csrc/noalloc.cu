// State digests of caller-owned device memory, without any allocation.
//
// tgs_state_digest reduces a simulator's pools into device accumulators the
// library allocates.  Some callers cannot allocate device memory at all: a
// host application whose allocator owns every device byte, or code running
// while a memory pool is frozen.  For them tgs_pool_digests_noalloc takes
// the pools from the caller and keeps its per-pool accumulators in the
// fixed-size array below, which lives as long as the library is loaded
// (every GPU that loads the library holds it until exit).
#include <cuda_runtime.h>

#include <new>
#include <string>

#include "kernels.h"
#include "tgs_internal.h"

namespace tgs {
namespace {

constexpr uint32_t kNoAllocMaxPools = 4096;  // 32 KiB of accumulators per device

__device__ __align__(256) unsigned long long gPoolDigestScratch[kNoAllocMaxPools];

// Device address of the accumulator array in the current device's context.
// Resolved on every call, with that device current: the lookup allocates
// nothing, and a context the caller re-created (cudaDeviceReset) places the
// array at a new address that a cached pointer would miss.  The first call
// on a device loads the library's device code into its context.
unsigned long long *scratchForCurrentDevice() {
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, gPoolDigestScratch);
  if (e != cudaSuccess) throw Error(TGS_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  return static_cast<unsigned long long *>(p);
}

}  // namespace
}  // namespace tgs

extern "C" int tgs_pool_digests_noalloc(const uint8_t *pools, uint64_t stride, uint64_t bytes, uint32_t n_pools,
                                        uint64_t *digests) {
  using namespace tgs;
  try {
    if (n_pools == 0) return TGS_OK;
    if (!pools || !digests) throw Error(TGS_ERR_ARG, "null pools or digests");
    if (n_pools > kNoAllocMaxPools)
      throw Error(TGS_ERR_RANGE, "at most " + std::to_string(kNoAllocMaxPools) + " pools per call");
    if (bytes > 0xFFFFFFFFull) throw Error(TGS_ERR_RANGE, "pool larger than 4 GiB");
    if (n_pools > 1 && stride < bytes) throw Error(TGS_ERR_ARG, "stride smaller than the pool");
    unsigned long long *acc = scratchForCurrentDevice();
    // the array keeps the previous call's sums: clear the part this call uses
    cudaError_t e = cudaMemsetAsync(acc, 0, size_t(n_pools) * sizeof(unsigned long long), nullptr);
    if (e == cudaSuccess) e = launchMemDigest(pools, stride, uint32_t(bytes), n_pools, acc, nullptr);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(digests, acc, size_t(n_pools) * sizeof(unsigned long long), cudaMemcpyDeviceToHost, nullptr);
    if (e == cudaSuccess) e = cudaStreamSynchronize(nullptr);
    if (e != cudaSuccess) throw Error(TGS_ERR_CUDA, std::string("pool digest: ") + cudaGetErrorString(e));
    return TGS_OK;
  } catch (const Error &err) {
    setLastError(err.what());
    return err.code;
  } catch (const std::bad_alloc &) {
    setLastError("host out of memory");
    return TGS_ERR_RESOURCES;
  } catch (const std::exception &err) {
    setLastError(err.what());
    return TGS_ERR_ARG;
  }
}
