// Instantiates the graph-form region kernel (regionKernel, one launch per region) for every
// (streams per word, groups per item) pair, with exec levels resident in shared memory for the whole launch.
#include "cycle_kernel.cuh"

namespace tgs {

void *regionKernelResident(int spw, int G) { return regionKernelPtrT<true>(spw, G); }

}  // namespace tgs
