"""The benchmarked configurations at full size against the reference's own
GPU kernel.

tests/golden/refgpu_fullsize.json holds the reference kernel's results
(src/SimEval.cu compiled unmodified, driven through its race-free eval()
path by oracle/refgpu_harness.cpp, tests/golden/make_refgpu_fullsize.py) for
one stream of each benchmarked workload: the seeded 1M-LUT, mixed 4M-LUT and
16M-LUT designs, regenerated here from their seeds.  The CPU oracle must
reproduce every per-cycle register digest and the final register, memory
and rolling digests; so must (marked gpu) this library, both as a single
stream and as stream 0 of a 64-stream batch in the benchmark's
configuration (stream 0's inputs are the fixture's: seed_s = mix64(base ^ s)).
"""
import json
import os
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle
from toucangpurt_gb300 import sim, workloads

FIX_PATH = Path(__file__).parent / "golden" / "refgpu_fullsize.json"
FIX = json.loads(FIX_PATH.read_text()) if FIX_PATH.exists() else []


def _h(x):
    return np.uint64(int(x, 16))


@pytest.fixture(scope="module", params=FIX, ids=[f["case"] for f in FIX])
def case(request, tmp_path_factory, built):
    f = request.param
    d = tmp_path_factory.mktemp(f["case"])
    dp, sp = d / "d.bin", d / "s.bin"
    info = sim.generate(dp, sp, **workloads.design_config(f["case"]))
    assert workloads.DESIGN_SEEDS[f["case"]] == f["design_seed"] and info["lut_ops"] == f["lut_ops"]
    stim = sim.StimulusSpec(f["stim_seed"], info["pi_ids"], info["pi_bits"],
                            workloads.toggles(f["case"], info["pi_bits"]))
    yield f, dp, sp, stim
    dp.unlink()


def _check(f, cycle_digest, final_reg, final_mem, rolling, stop):
    r = f["results"][0]
    np.testing.assert_array_equal(cycle_digest, np.array([int(x, 16) for x in r["cycle_digests"]], np.uint64))
    assert final_reg == _h(r["final_reg_digest"])
    assert final_mem == _h(r["final_mem_digest"])
    assert rolling == _h(r["rolling_digest"])
    assert int(stop) == r["stop_cycle"]


def test_oracle_matches_reference_kernel_fullsize(case):
    f, dp, sp, stim = case
    od = pyoracle.OracleDesign(dp, sp)
    out = od.run(np.full(1, f["cycles"], np.uint32), stim, threads=os.cpu_count() or 1, cycle_digests=True)
    _check(f, out["cycle_digest"][0], out["final_reg_digest"][0], out["final_mem_digest"][0], out["rolling_digest"][0],
           out["stop_cycle"][0])


@pytest.mark.gpu
@pytest.mark.parametrize("streams", [1, 64])
def test_gpu_matches_reference_kernel_fullsize(case, streams):
    f, dp, sp, stim = case
    s, _ = workloads.bench_simulator(f["case"], dp, sp, streams=streams, profile_cycles=4, epochs=8)
    try:
        got = s.batch_run(np.full(streams, f["cycles"], np.uint32), stim, cycle_digests=True)
    finally:
        s.cleanup()
    _check(f, got.cycle_digest[0], got.final_reg_digest[0], got.final_mem_digest[0], got.rolling_digest[0],
           got.stop_cycle[0])
