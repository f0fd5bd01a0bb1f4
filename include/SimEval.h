// Free-function host API of the reference evaluator (include/SimEval.h:11-40
// of ucsc-vama/toucanGPURT).  The reference keeps one simulator as global
// device state; here the functions act on the simulator most recently
// initialised through toucanGPUSim::ToucanSimulator::init or
// copy_netlist_to_gpu.  The reference's __global__ kernels are not part of
// this header: the GB300 kernels are internal to the library.
#pragma once

#include <cuda_runtime_api.h>

#include <cstdio>
#include <cstdlib>
#include <tuple>
#include <vector>

#include "SimConfigs.h"
#include "ToucanGPUGenDataTypes.h"

#define gpuErrchk(ans) \
  { gpuAssert((ans), __FILE__, __LINE__); }
inline void gpuAssert(cudaError_t code, const char *file, int line, bool abort = true) {
  if (code != cudaSuccess) {
    fprintf(stderr, "GPUassert: %s, file: %s, line: %d\n", cudaGetErrorString(code), file, line);
    if (abort) exit(code);
  }
}

uint64_t read_reg_from_gpu(const std::vector<std::tuple<uint32_t, uint32_t>> &signalLocs);
void write_reg_to_gpu(const std::vector<std::tuple<uint32_t, uint32_t>> &signalLocs, uint64_t signalValue);
void copy_netlist_to_gpu(toucanGPUSim::SimDesignInfo &design);
bool get_eval_done();
uint32_t get_real_cycles();
void setEnablePrint(bool print_en);
#ifdef ENABLE_SIM_PROFILE
void copy_profile_data(int64_t *usefulTicks, int64_t *totalTicks, size_t count);
#endif
