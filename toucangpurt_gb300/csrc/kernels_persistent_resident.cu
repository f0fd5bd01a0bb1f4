// Instantiates the persistent cooperative cycle kernel (cycleKernel) for every
// (streams per word, groups per item) pair, with exec levels resident in shared memory for the whole launch.
#include "cycle_kernel.cuh"

namespace tgs {

void *cycleKernelResident(int spw, int G) { return cycleKernelPtrT<true>(spw, G); }

}  // namespace tgs
