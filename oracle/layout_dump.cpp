// Prints the canonical form (layout_canon.h) of the device netlist layout
// that refgpu_harness.cpp builds for the reference's kernels (ref_layout.h),
// laid out in host memory instead of on a GPU.
//
// TEST INFRASTRUCTURE ONLY: tests/test_ref_layout.py compares it with the
// canonical form of the reference's own copy_netlist_to_gpu
// (ref_layout_main.cpp) on the same design files.
//
//   layout_dump <design.bin>
#include <cstdio>
#include <fstream>
#include <map>
#include <string>
#include <vector>

#include "layout_canon.h"
#include "ref_layout.h"

namespace {

// Buffers at synthetic addresses: buffer k spans [(k + 1) << 32, + n).
struct HostSink : reflayout::Sink {
  std::vector<std::vector<uint8_t>> bufs;
  std::map<std::string, std::vector<uint8_t>> globals;
  uint64_t upload(const void *d, size_t n) override {
    const auto *b = static_cast<const uint8_t *>(d);
    bufs.emplace_back(b, b + n);
    return uint64_t(bufs.size()) << 32;
  }
  void setGlobal(const char *name, const void *d, size_t n) override {
    const auto *b = static_cast<const uint8_t *>(d);
    globals[name].assign(b, b + n);
  }
};

}  // namespace

int main(int argc, char **argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: layout_dump design.bin\n");
    return 2;
  }
  try {
    toucanGPUSim::SimDesignInfo d;
    std::ifstream f(argv[1], std::ios::binary);
    if (!f) throw std::runtime_error("cannot open design");
    toucanGPUSim::deserializeSimDesignInfo(f, d);
    d.Init();
    HostSink s;
    reflayout::build(d, s);
    const std::string c = reflayout::canonical(
        [&](uint64_t a, reflayout::Found &r) {
          const uint64_t k = a >> 32;
          if (k == 0 || k > s.bufs.size()) return false;
          const auto &b = s.bufs[k - 1];
          r.p = b.data();
          r.n = b.size();
          r.off = size_t(a & 0xFFFFFFFFull);
          return r.off <= r.n;
        },
        [&](const char *name, std::vector<uint8_t> &out) {
          auto it = s.globals.find(name);
          if (it == s.globals.end()) return false;
          out = it->second;
          return true;
        });
    std::fwrite(c.data(), 1, c.size(), stdout);
  } catch (const std::exception &e) {
    std::fprintf(stderr, "layout_dump: %s\n", e.what());
    return 1;
  }
  return 0;
}
