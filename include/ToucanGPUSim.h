// C++ host API of the simulator, source compatible with the reference's
// toucanGPUSim::ToucanSimulator (include/ToucanGPUSim.h:10-74 of
// ucsc-vama/toucanGPURT): same public members and signatures, so a testbench
// written against the reference (e.g. its main.cpp) builds unchanged.
// Each instance owns one handle of the C ABI in toucan_gb300.h.
#pragma once

#include <cstddef>
#include <fstream>
#include <string>
#include <vector>

#include "GPUConsts.h"
#include "SimConfigs.h"
#include "ToucanGPUGenDataTypes.h"

struct tgs_sim;

namespace toucanGPUSim {

class ToucanSimulator {
 public:
  SimDesignInfo design;
  SimDebugInfo symbols;

  // 0 on success, -1 when a file cannot be opened or the design does not fit
  // the GPU (ToucanSim.cu:102-204).
  int init(const int gpu_id, const std::string designBinFilename, const std::string symbolBinFilename,
           bool shouldRandomize, bool enablePrint);

  void enableVCDDump(const std::string vcdFilename);

  // One cycle; returns the sticky stop flag.
  bool eval();

  // max_cycles cycles in one launch; returns the sticky stop flag.
  bool eval_free_running(uint32_t max_cycles);

  void setRegister(const std::string &signalName, uint64_t signalValue);
  uint64_t readRegister(const std::string &signalName);
  uint64_t readSignal(const std::string &signalName);

  // Releases all device memory (the reference's cleanup is empty).
  void cleanup();

#ifdef ENABLE_SIM_PROFILE
  void printProfile();
#endif

  ToucanSimulator();
  ~ToucanSimulator() { cleanup(); }
  ToucanSimulator(const ToucanSimulator &) = delete;
  ToucanSimulator &operator=(const ToucanSimulator &) = delete;

  uint64_t cycle_cnt = 0;

  // Underlying C-ABI handle (null before init).
  tgs_sim *handle() const { return sim_; }

 private:
  tgs_sim *sim_ = nullptr;
  bool dumpVCD = false;
  std::string vcdFile;
};

}  // namespace toucanGPUSim
