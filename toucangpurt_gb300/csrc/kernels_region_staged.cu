// Instantiates the graph-form region kernel (regionKernel, one launch per region) for every
// (streams per word, groups per item) pair, with exec levels staged per level into shared memory, or read from global memory.
#include "cycle_kernel.cuh"

namespace tgs {

void *regionKernelStaged(int spw, int G) { return regionKernelPtrT<false>(spw, G); }

}  // namespace tgs
