"""Value-pool slot renumbering by live range (csrc/slotalloc.cpp).

The renumbered design is an ordinary design file: it must pass the static
checks, need no larger a pool, and evaluate bit for bit like the original —
on the reference kernel's own golden fixtures and on every known-answer
design — through the CPU oracle.  On the GPU, both numberings must match the
oracle."""
import ctypes as C
import json
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle
from tests.test_golden import EVAL, _h, _ids, _stim
from toucangpurt_gb300 import capi, sim, workloads

G = Path(__file__).parent / "golden"


def compact(src, dst):
    before, after = C.c_uint32(), C.c_uint32()
    capi.check(capi.lib().tgs_compact_design(str(src).encode(), str(dst).encode(), C.byref(before), C.byref(after)))
    capi.check(capi.lib().tgs_validate_file(str(dst).encode(), None, None))
    assert after.value <= before.value
    return before.value, after.value


@pytest.mark.parametrize("f", EVAL, ids=_ids(EVAL))
def test_compacted_design_reproduces_reference_kernel(built, tmp_path, f):
    dst = tmp_path / "c.bin"
    compact(G / f"{f['case']}.bin", dst)
    od = pyoracle.OracleDesign(dst, G / f"{f['case']}.sym", randomize=bool(f["randomize"]))
    out = od.run(np.full(f["streams"], f["cycles"], np.uint32), _stim(f), cycle_digests=True)
    for s, r in enumerate(f["results"]):
        np.testing.assert_array_equal(out["cycle_digest"][s], np.array([int(x, 16) for x in r["cycle_digests"]], np.uint64))
        assert out["final_reg_digest"][s] == _h(r["final_reg_digest"])
        assert out["final_mem_digest"][s] == _h(r["final_mem_digest"])
        assert int(out["stop_cycle"][s]) == r["stop_cycle"]


KATS = sorted(p.stem for p in G.glob("kat_*.bin"))


@pytest.mark.parametrize("name", KATS)
def test_compacted_known_answer_designs(built, tmp_path, name):
    dst = tmp_path / "c.bin"
    compact(G / f"{name}.bin", dst)
    a = pyoracle.OracleDesign(G / f"{name}.bin").run(np.full(2, 6, np.uint32), cycle_digests=True, final_state=True)
    b = pyoracle.OracleDesign(dst).run(np.full(2, 6, np.uint32), cycle_digests=True, final_state=True)
    for k in ("cycle_digest", "final_reg_digest", "final_mem_digest", "stop_cycle"):
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_generated_design_shrinks(built, tmp_path):
    dp, sp = tmp_path / "d.bin", tmp_path / "d.sym"
    info = sim.generate(dp, sp, **workloads.design_config("scale", n_lut=1 << 16, ff_bits=4096, n_mems=2,
                                                          mem_depth=1024))
    before, after = compact(dp, tmp_path / "c.bin")
    assert after < before
    stim = sim.StimulusSpec(3, info["pi_ids"], info["pi_bits"])
    cyc = np.full(4, 5, np.uint32)
    a = pyoracle.OracleDesign(dp, sp).run(cyc, stim, cycle_digests=True)
    b = pyoracle.OracleDesign(tmp_path / "c.bin", sp).run(cyc, stim, cycle_digests=True)
    np.testing.assert_array_equal(a["cycle_digest"], b["cycle_digest"])
    np.testing.assert_array_equal(a["final_mem_digest"], b["final_mem_digest"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["mixed", "vec16", "stop", "deep"])
@pytest.mark.parametrize("value_pool", [0, 1])
def test_gpu_both_numberings_match_oracle(built, case, value_pool):
    f = next(x for x in EVAL if x["case"] == case)
    stim = _stim(f)
    cyc = np.full(16, min(f["cycles"], 60), np.uint32)
    with sim.Simulator(n_streams=16, value_pool=value_pool) as s:
        s.init(0, G / f"{case}.bin", G / f"{case}.sym", bool(f["randomize"]), False)
        got = s.batch_run(cyc, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(G / f"{case}.bin", G / f"{case}.sym", randomize=bool(f["randomize"])).run(
        cyc, stim, cycle_digests=True)
    np.testing.assert_array_equal(got.cycle_digest, ref["cycle_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])
    np.testing.assert_array_equal(got.stop_cycle, ref["stop_cycle"])
