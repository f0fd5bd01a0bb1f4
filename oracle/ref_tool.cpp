// Command-line driver around the reference's own host code.
//
// TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
// src/Serializer.cpp and src/SimInit.cpp taken from the reference checkout
// (never copied into this repository) into oracle/_ref/ref_tool, which the
// format tests use as the ground truth for the design/symbol file format and
// for the initial state.
//
//   ref_tool roundtrip  <design.bin> <out.bin>     deserialize + serialize
//   ref_tool symtrip    <symbols.bin> <out.bin>    same for a symbol file
//   ref_tool identical  <a.bin> <b.bin>            isSimDesignInfoIdentical
//   ref_tool initstate  <design.bin> <symbols.bin> <randomize 0|1> <regs.out> <mems.out>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>

#include "ToucanGPUGenDataTypes.h"

using namespace toucanGPUSim;

static bool loadDesign(const char *p, SimDesignInfo &d) {
  std::ifstream f(p, std::ios::binary);
  if (!f) return false;
  deserializeSimDesignInfo(f, d);
  return true;
}

int main(int argc, char **argv) {
  if (argc < 2) return 2;
  std::string cmd = argv[1];
  if (cmd == "roundtrip" && argc == 4) {
    SimDesignInfo d;
    if (!loadDesign(argv[2], d)) return 3;
    std::ofstream o(argv[3], std::ios::binary);
    serializeSimDesignInfo(o, d);
    return 0;
  }
  if (cmd == "symtrip" && argc == 4) {
    SimDebugInfo s;
    std::ifstream f(argv[2], std::ios::binary);
    if (!f) return 3;
    deserializeSimDebugInfo(f, s);
    std::ofstream o(argv[3], std::ios::binary);
    serializeSimDebugInfo(o, s);
    std::cout << s.regDebugInfo.size() << " " << s.signalDebugInfo.size() << " " << s.memDebugInfo.size() << "\n";
    return 0;
  }
  if (cmd == "identical" && argc == 4) {
    SimDesignInfo a, b;
    if (!loadDesign(argv[2], a) || !loadDesign(argv[3], b)) return 3;
    std::cout << (isSimDesignInfoIdentical(a, b) ? "identical" : "different") << "\n";
    return 0;
  }
  if (cmd == "initstate" && argc == 7) {
    SimDesignInfo d;
    SimDebugInfo s;
    if (!loadDesign(argv[2], d)) return 3;
    std::ifstream f(argv[3], std::ios::binary);
    if (!f) return 3;
    deserializeSimDebugInfo(f, s);
    d.Init();
    if (std::atoi(argv[4])) d.Randomize(0, s);
    std::ofstream r(argv[5], std::ios::binary), m(argv[6], std::ios::binary);
    r.write(reinterpret_cast<const char *>(d.regPool.data()), d.regPool.size());
    m.write(reinterpret_cast<const char *>(d.memPool.data()), d.memPool.size());
    return 0;
  }
  return 2;
}
