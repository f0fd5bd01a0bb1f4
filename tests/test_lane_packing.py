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


def _packing_kat():
    """One exec level of four narrow micro-partitions: A references a lane
    beyond its width (not packable: that lane is idle, value 0, in A alone);
    B has two middle levels, an immediate write-back and a shuffle id >= 64;
    C has fewer write-back entries than lanes; D has one middle level."""
    from tests import designlib as dl
    from tests.test_kat import IN, OUT, frame, table

    lut = table(100, lambda a, b, c: a * 7 + b * 3 + c * 5 + (a & b), rows=16)
    A = dl.MPart(top=[dl.top(100, IN + 0, IN + 1, IN + 2), dl.top(100, IN + 3, IN + 4, IN + 5),
                      dl.top(100, 1, IN + 6, IN + 7)],
                 mids=[[dl.mid(100, 33, 34, 37), dl.mid(100, 32, 32, 33), dl.mid(0, 0, 0, 34)]],
                 wbs=[dl.wb(32, OUT + 0), dl.wb(33, OUT + 1), dl.wb(34, OUT + 2)])
    B = dl.MPart(top=[dl.top(100, IN + 8, IN + 9, IN + 10), dl.top(100, 2, IN + 11, IN + 12),
                      dl.top(100, IN + 13, 4, IN + 14), dl.top(0, 0, 0, IN + 15)],
                 mids=[[dl.mid(100, 33, 34, 35), dl.mid(100, 32, 35, 34), dl.mid(100, 34, 33, 32), dl.mid(0, 0, 0, 35)],
                       [dl.mid(100, 32, 33, 34), dl.mid(100, 35, 34, 33), dl.mid(0, 0, 0, 33), dl.mid(100, 3, 32, 35)]],
                 wbs=[dl.wb(32, OUT + 3), dl.wb(7, OUT + 4), dl.wb(64 + 2, OUT + 5), dl.wb(35, OUT + 6)])
    C = dl.MPart(top=[dl.top(100, IN + 1, IN + 3, IN + 5), dl.top(100, IN + 2, IN + 4, IN + 6)],
                 wbs=[dl.wb(33, OUT + 7)])
    D = dl.MPart(top=[dl.top(100, IN + k, IN + (k + 5) % 16, IN + (k + 9) % 16) for k in range(5)],
                 mids=[[dl.mid(100, 32 + (k + 1) % 5, 32 + k, 32 + (k + 3) % 5) for k in range(5)]],
                 wbs=[dl.wb(32 + k, OUT + 8 + k) for k in range(5)])
    return frame([[A, B, C, D]], lut=lut)


def test_packing_known_answer_design(tmp_path, built):
    dp = tmp_path / "kat.bin"
    _packing_kat().write(dp)
    dst = tmp_path / "packed.bin"
    before, after = pack(dp, dst)
    assert (before, after) == (5, 3)  # B, C and D packed into one; A and the zeroing level kept
    capi.check(capi.lib().tgs_validate_file(str(dst).encode(), None, None))
    stim = sim.StimulusSpec(5, np.arange(16, dtype=np.uint32), np.full(16, 4, np.uint8))
    cycles = np.full(2, 50, np.uint32)
    a = pyoracle.OracleDesign(dp).run(cycles, stim, cycle_digests=True, final_state=True)
    b = pyoracle.OracleDesign(dst).run(cycles, stim, cycle_digests=True, final_state=True)
    for k in ("cycle_digest", "final_regs", "final_mems", "stop_cycle"):
        np.testing.assert_array_equal(b[k], a[k], err_msg=k)


@pytest.mark.gpu
@pytest.mark.parametrize("packing", [0, 1])
def test_packing_known_answer_design_gpu(tmp_path, built, packing):
    dp = tmp_path / "kat.bin"
    _packing_kat().write(dp)
    stim = sim.StimulusSpec(5, np.arange(16, dtype=np.uint32), np.full(16, 4, np.uint8))
    cycles = np.full(16, 50, np.uint32)
    ref = pyoracle.OracleDesign(dp).run(cycles, stim, cycle_digests=True)
    with sim.Simulator(n_streams=16, lane_packing=packing) as s:
        s.init(0, dp, None, False, False)
        got = s.batch_run(cycles, stim, cycle_digests=True)
    np.testing.assert_array_equal(got.cycle_digest, ref["cycle_digest"])
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])
