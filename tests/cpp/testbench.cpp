// A testbench written against the reference's C++ API only
// (toucanGPUSim::ToucanSimulator, include/ToucanGPUSim.h:10-74, and the
// SimEval.h free functions, include/SimEval.h:21-40), built against this
// library.  Usage: testbench <design.bin> <symbols.bin> <eval cycles> <free cycles>
// Prints "name=value" for every register after the run, sorted by name;
// built with ENABLE_SIM_PROFILE it then prints the per-partition profile.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "SimConfigs.h"
#include "SimEval.h"
#include "ToucanGPUSim.h"

int main(int argc, char **argv) {
  if (argc != 5) return 2;
  toucanGPUSim::ToucanSimulator sim;
  if (sim.init(0, argv[1], argv[2], true, false) != 0) return 3;
  const int evalCycles = std::atoi(argv[3]), freeCycles = std::atoi(argv[4]);
  // drive pi_0 from the testbench between eval() calls, like a reference testbench
  for (int c = 0; c < evalCycles; ++c) {
    sim.setRegister("pi_0", uint64_t(0x9E3779B1u * (c + 1)) & 0xFFFFFFFFu);
    sim.eval();
  }
  bool stop = sim.eval_free_running(uint32_t(freeCycles));
  std::vector<std::string> names;
  for (auto &kv : sim.symbols.regDebugInfo) names.push_back(kv.first);
  std::sort(names.begin(), names.end());
  for (auto &n : names) std::printf("%s=%llu\n", n.c_str(), (unsigned long long)sim.readRegister(n));
  // the free-function API reads the same state
  const auto &locs = sim.symbols.regDebugInfo.at("pi_0");
  std::printf("#read_reg_from_gpu=%llu\n", (unsigned long long)read_reg_from_gpu(locs));
  std::printf("#cycle_cnt=%llu real_cycles=%u stop=%d eval_done=%d\n", (unsigned long long)sim.cycle_cnt,
              get_real_cycles(), int(stop), int(get_eval_done()));
#ifdef ENABLE_SIM_PROFILE
  // the reference driver's profile report after a free-running call (main.cpp:62-64)
  sim.printProfile();
#endif
  return 0;
}
