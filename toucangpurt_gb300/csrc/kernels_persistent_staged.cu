// Instantiates the persistent cooperative cycle kernel (cycleKernel) for every
// (streams per word, groups per item) pair, with exec levels staged per level into shared memory, or read from global memory.
#include "cycle_kernel.cuh"

namespace tgs {

void *cycleKernelStaged(int spw, int G) { return cycleKernelPtrT<false>(spw, G); }

}  // namespace tgs
