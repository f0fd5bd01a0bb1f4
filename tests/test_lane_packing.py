"""Lane packing of narrow LUT micro-partitions (csrc/emit.cpp packLevel).

tgs_pack_design writes the packed design as an ordinary design file, so the
CPU oracle (an independent evaluator of the reference semantics) checks the
transformation: the packed file must evaluate bit for bit like the original
— on the reference kernel's own golden fixtures and on generated designs
with narrow and deep cones.  On the GPU, the simulator with packing on and
off must both match the oracle."""
import ctypes as C
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle
from tests.test_golden import EVAL, _h, _ids, _stim
from toucangpurt_gb300 import capi, sim, workloads

G = Path(__file__).parent / "golden"

# narrow micro-partitions (4-16 lanes) with deep middle-level chains
NARROW = {
    "cones16": dict(workloads.design_config("small"), seed=21, cone_depth=4, mpart_width=16, n_lut=6000, levels=16),
    "cones4": dict(workloads.design_config("small"), seed=22, cone_depth=9, mpart_width=4, n_lut=3000, levels=18,
                   operands=3),
    "mixed": dict(seed=14, n_lut=40000, levels=64, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=65536,
                  ff_bits=8192, pi_bits=64, n_mems=16, mem_depth=1024, mem_width=64, mem_read_ports=2,
                  mem_write_ports=1, luts_per_part=4000, mpart_width=32, cone_depth=1, mixed=1),
}


def pack(src, dst):
    before, after = C.c_uint32(), C.c_uint32()
    capi.check(capi.lib().tgs_pack_design(str(src).encode(), str(dst).encode(), C.byref(before), C.byref(after)))
    return before.value, after.value


@pytest.mark.parametrize("f", EVAL, ids=_ids(EVAL))
def test_packed_design_reproduces_reference_kernel(built, tmp_path, f):
    dst = tmp_path / "p.bin"
    pack(G / f"{f['case']}.bin", dst)
    od = pyoracle.OracleDesign(dst, G / f"{f['case']}.sym", randomize=bool(f["randomize"]))
    out = od.run(np.full(f["streams"], f["cycles"], np.uint32), _stim(f), cycle_digests=True)
    for s, r in enumerate(f["results"]):
        np.testing.assert_array_equal(out["cycle_digest"][s], np.array([int(x, 16) for x in r["cycle_digests"]], np.uint64))
        assert out["final_reg_digest"][s] == _h(r["final_reg_digest"])
        assert out["final_mem_digest"][s] == _h(r["final_mem_digest"])
        assert int(out["stop_cycle"][s]) == r["stop_cycle"]


@pytest.fixture(scope="module")
def narrow(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("narrow")
    out = {}
    for name, cfg in NARROW.items():
        dp, sp = d / f"{name}.bin", d / f"{name}.sym"
        out[name] = (dp, sp, sim.generate(dp, sp, **cfg))
    return out


@pytest.mark.parametrize("name", list(NARROW))
def test_packed_design_evaluates_like_original(narrow, tmp_path, name):
    dp, sp, info = narrow[name]
    dst = tmp_path / "p.bin"
    before, after = pack(dp, dst)
    assert after < before  # something was packed
    capi.check(capi.lib().tgs_validate_file(str(dst).encode(), str(sp).encode(), None))  # still a valid design
    cycles = np.full(3, 40, np.uint32)
    stim = sim.StimulusSpec(31, info["pi_ids"], info["pi_bits"])
    a = pyoracle.OracleDesign(dp, sp).run(cycles, stim, cycle_digests=True)
    b = pyoracle.OracleDesign(dst, sp).run(cycles, stim, cycle_digests=True)
    for k in ("cycle_digest", "final_reg_digest", "final_mem_digest", "rolling_digest", "stop_cycle"):
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(NARROW))
@pytest.mark.parametrize("packing", [0, 1])
@pytest.mark.parametrize("mode", [0, 1])
def test_gpu_packing_matches_oracle(narrow, name, packing, mode):
    dp, sp, info = narrow[name]
    cycles = np.full(24, 30, np.uint32)
    stim = sim.StimulusSpec(33, info["pi_ids"], info["pi_bits"])
    with sim.Simulator(n_streams=24, groups_per_item=2, lane_packing=packing, mode=mode) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cycles, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim, cycle_digests=True)
    for k in ("final_reg_digest", "final_mem_digest", "rolling_digest", "stop_cycle"):
        np.testing.assert_array_equal(getattr(got, k), ref[k], err_msg=k)
    np.testing.assert_array_equal(got.cycle_digest, ref["cycle_digest"])
