// toucanGPUSim::ToucanSimulator and the SimEval.h free functions on top of
// the C ABI.  Behaviour follows the reference host code
// (src/ToucanSim.cu:102-326, src/SimEval.cu:1058-1104): init returns -1 on a
// missing file or a design that does not fit, other failures print the error
// and exit like the reference's gpuErrchk (SimEval.h:11-19).
// The library always carries the profile entry points; the header declares
// them only when the including code enables the profile.
#define ENABLE_SIM_PROFILE

#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <sstream>

#include "SimEval.h"
#include "ToucanGPUSim.h"
#include "tgs_internal.h"

namespace tgs {
const toucanGPUSim::SimDesignInfo &designOf(const tgs_sim *h);
const toucanGPUSim::SimDebugInfo &symbolsOf(const tgs_sim *h);
}

namespace {
tgs_sim *gCurrent = nullptr;  // simulator the SimEval.h free functions act on

void dieOn(int rc, const char *what) {
  if (rc == TGS_OK) return;
  std::fprintf(stderr, "toucan: %s failed: %s\n", what, tgs_last_error());
  std::exit(1);
}

tgs_sim *current() {
  if (!gCurrent) {
    std::fprintf(stderr, "toucan: no simulator initialised\n");
    std::exit(1);
  }
  return gCurrent;
}
}  // namespace

namespace toucanGPUSim {

ToucanSimulator::ToucanSimulator() = default;

int ToucanSimulator::init(const int gpu_id, const std::string designBinFilename, const std::string symbolBinFilename,
                          bool shouldRandomize, bool enablePrint) {
  cycle_cnt = 0;
  dumpVCD = false;
  if (!sim_ && tgs_create(&sim_) != TGS_OK) return -1;
  int rc = tgs_init(sim_, gpu_id, designBinFilename.c_str(), symbolBinFilename.c_str(), shouldRandomize ? 1 : 0,
                    enablePrint ? 1 : 0);
  if (rc != TGS_OK) {
    std::cerr << "Error: " << tgs_last_error() << std::endl;
    return -1;
  }
  std::cout << "Load design complete" << std::endl;
  std::cout << "Load symbols complete" << std::endl;
  design = tgs::designOf(sim_);
  symbols = tgs::symbolsOf(sim_);
  std::cout << "Region 0 has " << design.regionPartitionIds[0].size() << " partitions\n";
  std::cout << "Region 1 has " << design.regionPartitionIds[1].size() << " partitions\n";
  gCurrent = sim_;
  return 0;
}

void ToucanSimulator::enableVCDDump(const std::string vcdFilename) {
  dumpVCD = true;
  vcdFile = vcdFilename;
  if (sim_ && tgs_enable_vcd(sim_, vcdFilename.c_str()) != TGS_OK) {
    std::cerr << "enableVCDDump: " << tgs_last_error() << std::endl;
    dumpVCD = false;
  }
}

bool ToucanSimulator::eval() {
  int stop = 0;
  dieOn(tgs_eval(sim_, &stop), "eval");
  cycle_cnt++;
  return stop != 0;
}

bool ToucanSimulator::eval_free_running(uint32_t max_cycles) {
  int stop = 0;
  dieOn(tgs_eval_free_running(sim_, max_cycles, &stop), "eval_free_running");
  cycle_cnt += max_cycles;
  return stop != 0;
}

void ToucanSimulator::setRegister(const std::string &name, uint64_t value) {
  dieOn(tgs_set_register(sim_, name.c_str(), value), "setRegister");
}

uint64_t ToucanSimulator::readRegister(const std::string &name) {
  uint64_t v = 0;
  dieOn(tgs_read_register(sim_, name.c_str(), &v), "readRegister");
  return v;
}

// UINT64_MAX with a message when the value is not available (signal capture
// off, unknown name, wider than 64 bits), as the reference always answers.
uint64_t ToucanSimulator::readSignal(const std::string &name) {
  uint64_t v = 0;
  if (!sim_ || tgs_read_signal(sim_, name.c_str(), &v) != TGS_OK) {
    std::cerr << "readSignal: " << (sim_ ? tgs_last_error() : "simulator not initialised") << std::endl;
    return UINT64_MAX;
  }
  return v;
}

void ToucanSimulator::cleanup() {
  if (!sim_) return;
  if (gCurrent == sim_) gCurrent = nullptr;
  tgs_destroy(sim_);
  sim_ = nullptr;
}

#ifdef ENABLE_SIM_PROFILE
void ToucanSimulator::printProfile() {
  size_t n = design.parts.size();
  std::vector<int64_t> useful(n), total(n);
  dieOn(tgs_copy_profile_data(sim_, useful.data(), total.data(), n), "copy_profile_data");
  for (size_t p = 0; p < n; ++p) {
    float ratio = total[p] ? float(useful[p] * 100.0 / total[p]) : 0.0f;
    std::cout << "Part " << p << ", useful " << ratio << "%, ticks " << useful[p] << ", total ticks " << total[p] << "\n";
  }
}
#endif

}  // namespace toucanGPUSim

uint64_t read_reg_from_gpu(const std::vector<std::tuple<uint32_t, uint32_t>> &locs) {
  tgs_sim *h = current();
  uint32_t regPool = 0;
  dieOn(tgs_get_pool_sizes(h, &regPool, nullptr, nullptr), "read_reg_from_gpu");
  std::vector<uint8_t> pool(regPool);
  dieOn(tgs_read_reg_pool(h, 0, pool.data(), pool.size()), "read_reg_from_gpu");
  uint64_t r = 0;
  for (auto &l : locs) r = (r << 4) | (pool.at(std::get<0>(l)) & 0xF);
  return r;
}

void write_reg_to_gpu(const std::vector<std::tuple<uint32_t, uint32_t>> &locs, uint64_t value) {
  tgs_sim *h = current();
  uint32_t regPool = 0;
  dieOn(tgs_get_pool_sizes(h, &regPool, nullptr, nullptr), "write_reg_to_gpu");
  std::vector<uint8_t> pool(regPool);
  dieOn(tgs_read_reg_pool(h, 0, pool.data(), pool.size()), "write_reg_to_gpu");
  for (auto it = locs.rbegin(); it != locs.rend(); ++it) {
    pool.at(std::get<0>(*it)) = uint8_t(value & 0xF);
    value >>= 4;
  }
  if (value != 0) {
    std::fprintf(stderr, "toucan: given value is wider than register\n");
    std::exit(1);
  }
  dieOn(tgs_write_reg_pool(h, 0, pool.data(), pool.size()), "write_reg_to_gpu");
}

void copy_netlist_to_gpu(toucanGPUSim::SimDesignInfo &design) {
  if (!gCurrent) dieOn(tgs_create(&gCurrent), "copy_netlist_to_gpu");
  std::ostringstream os;
  toucanGPUSim::serializeSimDesignInfo(os, design);
  std::string bytes = os.str();
  dieOn(tgs_init_from_memory(gCurrent, 0, bytes.data(), bytes.size(), nullptr, 0, 0, 0), "copy_netlist_to_gpu");
}

bool get_eval_done() {
  int stop = 0;
  dieOn(tgs_get_eval_done(current(), &stop), "get_eval_done");
  return stop != 0;
}

uint32_t get_real_cycles() {
  uint32_t c = 0;
  dieOn(tgs_get_real_cycles(current(), &c), "get_real_cycles");
  return c;
}

void setEnablePrint(bool en) { dieOn(tgs_set_enable_print(current(), en ? 1 : 0), "setEnablePrint"); }

#ifdef ENABLE_SIM_PROFILE
void copy_profile_data(int64_t *useful, int64_t *total, size_t count) {
  dieOn(tgs_copy_profile_data(current(), useful, total, count), "copy_profile_data");
}
#endif
