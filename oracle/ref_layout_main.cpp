// Runs the reference's own copy_netlist_to_gpu (src/SimEval.cu:1114-1343,
// built from the reference's tree) against the test-double runtime
// (fake_cudart.cpp) and prints the canonical form of the layout it wrote
// (layout_canon.h).
//
// TEST INFRASTRUCTURE ONLY: tests/test_ref_layout.py compares the output
// with layout_dump, the restated layout that drives the reference's cubin in
// refgpu_harness.cpp.  The design file is read with the reference's own
// Serializer and initialised with its own SimInit.
//
//   ref_layout <design.bin>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "ToucanGPUGenDataTypes.h"
#include "layout_canon.h"

// src/SimEval.cu (declared in the reference's include/SimEval.h, which also
// pulls in the CUDA device headers)
void copy_netlist_to_gpu(toucanGPUSim::SimDesignInfo &design);

extern "C" bool fakecuda_resolve(uint64_t addr, const uint8_t **p, size_t *n, size_t *off);
extern "C" bool fakecuda_global(const char *name, const uint8_t **p, size_t *n);

int main(int argc, char **argv) {
  if (argc != 2) {
    std::fprintf(stderr, "usage: ref_layout design.bin\n");
    return 2;
  }
  toucanGPUSim::SimDesignInfo d;
  {
    std::ifstream f(argv[1], std::ios::binary);
    if (!f) {
      std::fprintf(stderr, "ref_layout: cannot open design\n");
      return 1;
    }
    toucanGPUSim::deserializeSimDesignInfo(f, d);
  }
  d.Init();
  copy_netlist_to_gpu(d);
  const std::string c = reflayout::canonical(
      [](uint64_t a, reflayout::Found &r) { return fakecuda_resolve(a, &r.p, &r.n, &r.off); },
      [](const char *name, std::vector<uint8_t> &out) {
        const uint8_t *p;
        size_t n;
        if (!fakecuda_global(name, &p, &n)) return false;
        out.assign(p, p + n);
        return true;
      });
  std::fwrite(c.data(), 1, c.size(), stdout);
  return 0;
}
