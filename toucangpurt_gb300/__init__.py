"""GB300-native (sm_103a) Toucan netlist simulator.

A drop-in for the per-cycle netlist evaluation of ucsc-vama/toucanGPURT: the
reference's design/symbol file format, its ToucanSimulator API (C++ header in
include/, Python mirror in ``sim``), hand-written CUDA kernels behind a C ABI
(include/toucan_gb300.h).  Build with ``toucangpurt_gb300.build.build()``.
"""
from .capi import TgsError, library_path  # noqa: F401
from .sim import BatchOutput, Simulator, StimulusSpec, gen_config, generate, validate_file  # noqa: F401
