"""GPU parity: the sm_103a kernels through the C ABI against the CPU oracle.

Bit-exact equality on the same seeded inputs: per-cycle register digests,
rolling digests, final register/memory digests, full final state, stop cycles.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle
from toucangpurt_gb300 import sim, workloads

pytestmark = pytest.mark.gpu

# name -> generator overrides (small cases the oracle finishes in seconds)
DESIGNS = {
    "small": workloads.design_config("small"),
    "deep_cones": dict(workloads.design_config("small"), seed=11, cone_depth=4, mpart_width=16, n_lut=6000, levels=16),
    "wide3op": dict(seed=12, n_lut=20000, levels=12, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=64,
                    ff_bits=2048, pi_bits=64, n_vec_ops=24, vec_nibbles=8, n_mems=3, mem_depth=4096, mem_width=32,
                    mem_read_ports=2, mem_write_ports=2, mem_multi_writer=1, luts_per_part=2500, mpart_width=32,
                    cone_depth=2),
    "vec16": dict(seed=13, n_lut=8000, levels=8, operands=3, ff_bits=4096, pi_bits=64, n_vec_ops=40, vec_nibbles=16,
                  n_mems=2, mem_depth=256, mem_width=64, mem_read_ports=1, mem_write_ports=1, luts_per_part=2000,
                  mpart_width=32, cone_depth=1),
    "mixed": dict(seed=14, n_lut=40000, levels=64, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=65536,
                  ff_bits=8192, pi_bits=64, n_mems=16, mem_depth=1024, mem_width=64, mem_read_ports=2,
                  mem_write_ports=1, luts_per_part=4000, mpart_width=32, cone_depth=1, mixed=1),
    "stop": dict(workloads.design_config("small"), seed=15, with_stop=1),
}


@pytest.fixture(scope="module")
def designs(tmp_path_factory, built):
    out = {}
    d = tmp_path_factory.mktemp("designs")
    for name, cfg in DESIGNS.items():
        dp, sp = d / f"{name}.bin", d / f"{name}.sym"
        info = sim.generate(dp, sp, **cfg)
        out[name] = (dp, sp, info)
    return out


def _stim(info, seed=77, toggle=None):
    return sim.StimulusSpec(seed, info["pi_ids"], info["pi_bits"], toggle)


def _compare(got, ref, cycle_digests=True):
    for k in ("final_reg_digest", "final_mem_digest", "rolling_digest", "stop_cycle"):
        np.testing.assert_array_equal(getattr(got, k), ref[k], err_msg=k)
    if cycle_digests:
        np.testing.assert_array_equal(got.cycle_digest, ref["cycle_digest"], err_msg="cycle digests")


@pytest.mark.parametrize("name", list(DESIGNS))
@pytest.mark.parametrize("streams,groups", [(1, 1), (8, 1), (16, 2), (32, 4), (40, 4), (64, 8), (72, 8)])
def test_batch_parity(designs, name, streams, groups):
    dp, sp, info = designs[name]
    cycles = np.full(streams, 40, np.uint32)
    stim = _stim(info)
    with sim.Simulator(n_streams=streams, groups_per_item=groups) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cycles, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim, cycle_digests=True)
    _compare(got, ref)


@pytest.mark.parametrize("name", ["small", "wide3op", "mixed", "deep_cones"])
@pytest.mark.parametrize("levels", [0, 1, 2, 3])  # auto, resident, global, staged
@pytest.mark.parametrize("mode", [0, 1])  # persistent, graph
def test_exec_level_sources(designs, name, levels, mode):
    """Exec levels resident in shared memory for the launch, staged per level,
    or read from global memory: the same bit-exact results."""
    dp, sp, info = designs[name]
    cycles = np.full(24, 30, np.uint32)
    stim = _stim(info, seed=9)
    with sim.Simulator(n_streams=24, groups_per_item=2, resident_netlist=levels, mode=mode) as s:
        s.init(0, dp, sp, False, False)
        st = s.design_stats()
        if levels == 1:
            assert st["resident_words"] > 0 and st["stage_words"] == 0
        elif levels == 2:
            assert st["resident_words"] == 0 and st["stage_words"] == 0
        elif levels == 3:
            assert st["resident_words"] == 0 and st["stage_words"] > 0
        got = s.batch_run(cycles, stim, cycle_digests=True)
        got2 = s.batch_run(cycles, stim, cycle_digests=True)  # a second launch reloads the levels
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim, cycle_digests=True)
    _compare(got, ref)
    _compare(got2, ref)


@pytest.mark.parametrize("name", ["small", "wide3op", "mixed", "deep_cones"])
@pytest.mark.parametrize("levels", [0, 1, 3])  # auto, resident, staged
@pytest.mark.parametrize("mode", [0, 1])  # persistent, graph
@pytest.mark.parametrize("value_pool", [0, 1])  # renumbered (slot immediates), the design's numbering
@pytest.mark.parametrize("streams", [1, 8])  # one stream per word / 8 streams in one group
def test_single_stream_levels(designs, name, levels, mode, value_pool, streams):
    """One stream group per item: resident exec levels take the path that
    reads and decodes each warp's next unit during the current level (one-
    level compact LUT records over slot immediates; every other unit, and the
    design's own slot numbering, through the general path); staged and global
    ones the general loop.  Bit-exact in every form."""
    dp, sp, info = designs[name]
    cycles = np.full(streams, 40, np.uint32)
    stim = _stim(info, seed=21)
    with sim.Simulator(n_streams=streams, groups_per_item=1, resident_netlist=levels, mode=mode,
                       value_pool=value_pool) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cycles, stim, cycle_digests=True)
        got2 = s.batch_run(cycles, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim, cycle_digests=True)
    _compare(got, ref)
    _compare(got2, ref)


@pytest.mark.parametrize("name", ["wide3op", "mixed", "deep_cones"])
@pytest.mark.parametrize("streams,groups", [(1, 1), (8, 1), (24, 2)])
@pytest.mark.parametrize("mode", [0, 1])
def test_small_stage_buffers(designs, name, streams, groups, mode):
    """Stage buffers capped below the largest exec levels (stage_words):
    those levels are read from global memory, the others staged; one-group
    and multi-group items, both forms."""
    dp, sp, info = designs[name]
    cycles = np.full(streams, 30, np.uint32)
    stim = _stim(info, seed=23)
    with sim.Simulator(n_streams=streams, groups_per_item=groups, resident_netlist=3, mode=mode,
                       stage_words=256) as s:
        s.init(0, dp, sp, False, False)
        st = s.design_stats()
        assert 0 < st["stage_words"] <= 256
        if name == "wide3op":
            assert st["stage_words"] == 256  # some of its levels are larger
        got = s.batch_run(cycles, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim, cycle_digests=True)
    _compare(got, ref)


@pytest.mark.parametrize("warps", [0, 3, 4, 6, 12, 16, 32])
def test_warps_per_block(designs, warps):
    dp, sp, info = designs["wide3op"]
    cycles = np.full(16, 30, np.uint32)
    stim = _stim(info, seed=5)
    with sim.Simulator(n_streams=16, warps_per_block=warps) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cycles, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim, cycle_digests=True)
    _compare(got, ref)


def test_final_state_full(designs):
    dp, sp, info = designs["wide3op"]
    cycles = np.full(24, 25, np.uint32)
    stim = _stim(info, seed=9)
    with sim.Simulator(n_streams=24) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cycles, stim, final_state=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim, final_state=True)
    np.testing.assert_array_equal(got.final_regs, ref["final_regs"])
    np.testing.assert_array_equal(got.final_mems, ref["final_mems"][:, : got.final_mems.shape[1]])


def test_toggle_inputs(designs):
    dp, sp, info = designs["small"]
    tog = np.full(info["pi_ids"].size, 3277, np.uint16)  # 5 % per cycle
    stim = _stim(info, seed=31, toggle=tog)
    cycles = np.full(8, 60, np.uint32)
    with sim.Simulator(n_streams=8) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cycles, stim, cycle_digests=True)
    _compare(got, pyoracle.OracleDesign(dp, sp).run(cycles, stim, cycle_digests=True))


@pytest.mark.parametrize("randomize", [False, True])
def test_eval_per_cycle_matches_oracle(designs, randomize):
    """The reference's eval() flow: one cycle per call, full state each cycle."""
    dp, sp, _ = designs["wide3op"]
    od = pyoracle.OracleDesign(dp, sp, randomize=randomize)
    st = pyoracle.OracleState(od)
    with sim.Simulator() as s:
        s.init(0, dp, sp, randomize, False)
        np.testing.assert_array_equal(s.reg_pool(), st.regs())
        for c in range(12):
            stop = s.eval()
            ostop = st.eval(1)
            assert stop == ostop
            np.testing.assert_array_equal(s.reg_pool(), st.regs(), err_msg=f"regs after cycle {c}")
            np.testing.assert_array_equal(s.mem_pool(), st.mems(), err_msg=f"mems after cycle {c}")
        assert s.cycle_cnt() == 12
        assert s.real_cycles() == 0  # only free-running launches count (SimEval.cu:985-989)


def test_free_running_matches_oracle(designs):
    dp, sp, _ = designs["mixed"]
    od = pyoracle.OracleDesign(dp, sp, randomize=True)
    st = pyoracle.OracleState(od)
    with sim.Simulator() as s:
        s.init(0, dp, sp, True, False)
        s.eval_free_running(150)
        st.eval(150)
        np.testing.assert_array_equal(s.reg_pool(), st.regs())
        np.testing.assert_array_equal(s.mem_pool(), st.mems())
        assert s.real_cycles() == 150
        assert s.cycle_cnt() == 150


def test_register_io_roundtrip(designs):
    dp, sp, info = designs["small"]
    with sim.Simulator(n_streams=16) as s:
        s.init(0, dp, sp, False, False)
        s.set_register("ff_3", 0x12345678, stream=5)
        s.set_register("ff_3", 0x0BADF00D, stream=6)
        assert s.read_register("ff_3", stream=5) == 0x12345678
        assert s.read_register("ff_3", stream=6) == 0x0BADF00D
        with pytest.raises(sim.capi.TgsError) as e:
            s.set_register("ff_3", 1 << 40)
        assert e.value.code == sim.capi.ERR_RANGE
        with pytest.raises(sim.capi.TgsError) as e:
            s.read_register("no_such_reg")
        assert e.value.code == sim.capi.ERR_NOT_FOUND


def test_register_poke_then_eval(designs):
    """setRegister between cycles, as a reference testbench drives inputs:
    pi_0 holds primary-input nibbles 0..7, least significant first."""
    dp, sp, info = designs["small"]
    od = pyoracle.OracleDesign(dp, sp)
    st = pyoracle.OracleState(od)
    ids = info["pi_ids"][:8]
    with sim.Simulator() as s:
        s.init(0, dp, sp, False, False)
        rng = np.random.default_rng(3)
        for c in range(10):
            v = int(rng.integers(0, 2**32))
            s.set_register("pi_0", v)
            regs = st.regs()
            for j, rid in enumerate(ids):
                regs[rid] = (v >> (4 * j)) & 0xF
            assert s.read_register("pi_0") == v
            s.eval()
            st.eval(1)
            np.testing.assert_array_equal(s.reg_pool(), st.regs(), err_msg=f"cycle {c}")


def test_stop_and_print(designs, capfd):
    dp, sp, info = designs["stop"]
    stim = _stim(info, seed=3)
    cycles = np.full(8, 30, np.uint32)
    with sim.Simulator(n_streams=8) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cycles, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim, cycle_digests=True)
    _compare(got, ref)
    assert (got.stop_cycle != 0xFFFFFFFF).any()
    with sim.Simulator() as s:
        s.init(0, dp, sp, False, True)
        fired = False
        for _ in range(30):
            fired = s.eval() or fired
        od = pyoracle.OracleState(pyoracle.OracleDesign(dp, sp))
        assert fired == od.eval(30)
    out = capfd.readouterr().out
    if fired:
        assert "Toucan first stop" in out


def test_digest_matches_host(designs):
    dp, sp, _ = designs["vec16"]
    with sim.Simulator(n_streams=8) as s:
        s.init(0, dp, sp, True, False)
        s.eval_free_running(20)
        for stream in (0, 3, 7):
            r, m = s.digest(stream)
            assert r == pyoracle.digest(s.reg_pool(stream))
            assert m == pyoracle.digest(s.mem_pool(stream))


def test_read_registers_matches_oracle(designs):
    """Every register of the symbol file, read after a run for several
    streams: tgs_read_registers (one gather and one copy for all names) and
    tgs_read_register equal the oracle's register pools, most significant
    nibble first."""
    dp, sp, info = designs["wide3op"]
    regs = sim.symbol_registers(sp)
    names = sorted(n for n in regs if len(regs[n]) <= 16)  # at most 64 bits (SimEval.cu:1062)
    cycles = np.full(16, 21, np.uint32)
    stim = _stim(info, seed=41)
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim, final_state=True)
    with sim.Simulator(n_streams=16) as s:
        s.init(0, dp, sp, False, False)
        s.batch_run(cycles, stim)
        for stream in (0, 5, 15):
            pool = ref["final_regs"][stream]
            expect = []
            for n in names:
                v = 0
                for rid, _w in regs[n]:
                    v = (v << 4) | int(pool[rid])
                expect.append(v)
            assert s.read_registers(names, stream=stream) == expect
            for n, e in list(zip(names, expect))[:: max(1, len(names) // 16)]:
                assert s.read_register(n, stream=stream) == e
        assert s.read_registers([]) == []
        with pytest.raises(sim.capi.TgsError) as e:
            s.read_registers([names[0], "no_such_reg"])
        assert e.value.code == sim.capi.ERR_NOT_FOUND


@pytest.mark.parametrize("name", ["small", "mixed"])
def test_copy_profile_data(designs, name):
    """tgs_copy_profile_data (copy_profile_data, src/SimEval.cu:1101-1104):
    after a free-running call of at least 200 cycles every partition has a
    mean useful tick count in (0, total], totals covering the partition's
    region (src/SimEval.cu:894-983); values stay bit-exact."""
    dp, sp, _ = designs[name]
    od = pyoracle.OracleDesign(dp, sp, randomize=True)
    st = pyoracle.OracleState(od)
    with sim.Simulator() as s:
        s.init(0, dp, sp, True, False)
        s.eval_free_running(230)
        n = od.n_parts
        useful, total = s.profile(n)
        assert (useful > 0).all() and (useful <= total).all(), (useful[:8], total[:8])
        st.eval(230)
        np.testing.assert_array_equal(s.reg_pool(), st.regs())


def _design_levels(dp) -> int:
    import ctypes as C
    import tempfile

    st = sim.capi.RepackStats()
    with tempfile.TemporaryDirectory() as td:
        sim.capi.check(sim.capi.lib().tgs_repack_design(str(dp).encode(), str(Path(td) / "r.bin").encode(), 0, 0,
                                                        C.byref(st)))
    return st.exec_levels


@pytest.mark.parametrize("name", ["mixed", "deep_cones", "wide3op", "small"])
@pytest.mark.parametrize("lanes", [32, 64, 128])
@pytest.mark.parametrize("lpb", [1, 2, 4])
def test_schedule_knobs(designs, name, lanes, lpb):
    """Micro-partition size (LUTs a warp takes at once: 32, 64, 128) and
    levels per barrier (1, 2, 4 exec levels merged into one block where every
    dependency stays on one warp) only move the schedule: bit-exact results
    for batched streams (resident and staged levels, both forms) and a single
    stream."""
    dp, sp, info = designs[name]
    stim = _stim(info, seed=23)
    ref = None
    for streams, levels, mode in ((24, 0, 0), (24, 3, 1), (1, 0, 0)):
        cyc = np.full(streams, 24, np.uint32)
        with sim.Simulator(n_streams=streams, groups_per_item=2 if streams > 1 else 0, resident_netlist=levels,
                           mode=mode, mpart_lanes=lanes, levels_per_barrier=lpb) as s:
            s.init(0, dp, sp, False, False)
            st = s.design_stats()
            # every exec level of the design is a block of its own or merged into one
            assert st["exec_levels"] + st["fused_levels"] == _design_levels(dp)
            if lpb == 1:
                assert st["fused_levels"] == 0
            got = s.batch_run(cyc, stim, cycle_digests=True)
        r = pyoracle.OracleDesign(dp, sp).run(cyc, stim, cycle_digests=True)
        _compare(got, r)
