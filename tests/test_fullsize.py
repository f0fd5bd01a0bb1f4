"""Bit-exactness on the benchmarked configurations at full size.

The designs the benchmark measures (the seeded 1M-LUT, mixed 4M-LUT and
16M-LUT netlists of toucangpurt_gb300.workloads) run through the benchmark's
own configuration (workloads.bench_simulator: learned schedule for batched
runs, default groups per item, exec levels resident or staged as the
library picks, CUDA-graph form for staged levels, lane packing and the
compact value pool) and are compared with the CPU oracle, 64 streams (and a
single stream, the plain form) for a few cycles: per-cycle register digests
of every stream, final register, memory and rolling digests and stop
cycles.  The workloads' own primary-input statistics are used (toggle rates
included).
"""
import os

import numpy as np
import pytest

from oracle import pyoracle
from toucangpurt_gb300 import sim, workloads

pytestmark = pytest.mark.gpu

CASES = ["scale", "learned", "largest"]


@pytest.fixture(scope="module", params=CASES)
def full_design(request, tmp_path_factory, built):
    name = request.param
    d = tmp_path_factory.mktemp(name)
    dp, sp = d / f"{name}.bin", d / f"{name}.sym"
    info = sim.generate(dp, sp, **workloads.design_config(name))
    od = pyoracle.OracleDesign(dp, sp)
    yield name, dp, sp, info, od
    dp.unlink()


def _stim(name, info, seed):
    return sim.StimulusSpec(seed, info["pi_ids"], info["pi_bits"], workloads.toggles(name, info["pi_bits"]))


@pytest.mark.parametrize("streams,cycles", [(64, 4), (1, 6)])
def test_fullsize_bench_configuration_matches_oracle(full_design, streams, cycles):
    name, dp, sp, info, od = full_design
    stim = _stim(name, info, 1000)
    cyc = np.full(streams, cycles, np.uint32)
    s, notes = workloads.bench_simulator(name, dp, sp, streams=streams, profile_cycles=4, epochs=8)
    try:
        st = s.design_stats()
        got = s.batch_run(cyc, stim, cycle_digests=True)
        # a second launch of the same run (graph chunks replayed, levels restaged)
        again = s.batch_run(cyc, stim, cycle_digests=True)
    finally:
        s.cleanup()
    ref = od.run(cyc, stim, threads=min(os.cpu_count() or 1, max(streams, 16)), cycle_digests=True)
    for out in (got, again):
        np.testing.assert_array_equal(out.cycle_digest, ref["cycle_digest"], err_msg=f"{name}: per-cycle digests")
        for k in ("final_reg_digest", "final_mem_digest", "rolling_digest", "stop_cycle"):
            np.testing.assert_array_equal(getattr(out, k), ref[k], err_msg=f"{name}: {k}")
    assert st["lut_ops"] == info["lut_ops"]
    if streams > 1:
        assert notes["schedule"] == "learned"
