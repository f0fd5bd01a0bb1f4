"""CUDA-graph form of the cycle loop (one launch per region, replayed chunks)
against the CPU oracle: batched streams, admission, free-running state and
the per-cycle eval() flow."""
import numpy as np
import pytest

from oracle import pyoracle
from toucangpurt_gb300 import capi, sim, workloads

pytestmark = pytest.mark.gpu

GRAPH = dict(mode=capi.MODE_GRAPH)


@pytest.fixture(scope="module")
def small(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("graph")
    dp, sp = d / "d.bin", d / "s.bin"
    return dp, sp, sim.generate(dp, sp, **workloads.design_config("small"))


@pytest.fixture(scope="module")
def mixed(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("graphmixed")
    dp, sp = d / "d.bin", d / "s.bin"
    cfg = dict(seed=14, n_lut=40000, levels=64, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=65536,
               ff_bits=8192, pi_bits=64, n_mems=16, mem_depth=1024, mem_width=64, mem_read_ports=2,
               mem_write_ports=1, luts_per_part=4000, mpart_width=32, cone_depth=1, mixed=1)
    return dp, sp, sim.generate(dp, sp, **cfg)


@pytest.mark.parametrize("streams,groups,cycles", [(64, 4, 75), (64, 8, 40), (16, 2, 33), (8, 1, 1)])
def test_graph_batch_matches_oracle(small, streams, groups, cycles):
    """Chunks of 32 cycles replayed; lengths off the chunk boundary skip the tail."""
    dp, sp, info = small
    cyc = np.full(streams, cycles, np.uint32)
    stim = sim.StimulusSpec(4242, info["pi_ids"], info["pi_bits"])
    with sim.Simulator(n_streams=streams, groups_per_item=groups, **GRAPH) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cyc, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cyc, stim, cycle_digests=True)
    np.testing.assert_array_equal(got.cycle_digest, ref["cycle_digest"])
    np.testing.assert_array_equal(got.rolling_digest, ref["rolling_digest"])
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])


def test_graph_admission_matches_oracle(small):
    dp, sp, info = small
    rng = np.random.default_rng(5)
    cyc = rng.integers(3, 70, 41).astype(np.uint32)
    stim = sim.StimulusSpec(17, info["pi_ids"], info["pi_bits"])
    with sim.Simulator(n_streams=8, **GRAPH) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cyc, stim, cycle_digests=True, slots=16)
    ref = pyoracle.OracleDesign(dp, sp).run(cyc, stim, cycle_digests=True)
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])
    np.testing.assert_array_equal(got.rolling_digest, ref["rolling_digest"])
    for q in range(cyc.size):
        np.testing.assert_array_equal(got.cycle_digest[q, : cyc[q]], ref["cycle_digest"][q, : cyc[q]])


def test_graph_free_running_matches_oracle(mixed):
    dp, sp, _ = mixed
    st = pyoracle.OracleState(pyoracle.OracleDesign(dp, sp, randomize=True))
    with sim.Simulator(**GRAPH) as s:
        s.init(0, dp, sp, True, False)
        s.eval_free_running(70)
        st.eval(70)
        np.testing.assert_array_equal(s.reg_pool(), st.regs())
        np.testing.assert_array_equal(s.mem_pool(), st.mems())
        assert s.real_cycles() == 70
        for _ in range(3):
            assert s.eval() == st.eval(1)
        np.testing.assert_array_equal(s.reg_pool(), st.regs())
        np.testing.assert_array_equal(s.mem_pool(), st.mems())
        assert s.real_cycles() == 70


def test_autotune_then_parity(small):
    """The tuner's choice (any launch shape or mode) keeps results bit-exact."""
    dp, sp, info = small
    cyc = np.full(24, 40, np.uint32)
    stim = sim.StimulusSpec(8, info["pi_ids"], info["pi_bits"])
    with sim.Simulator(n_streams=24) as s:
        s.init(0, dp, sp, False, False)
        best, trials = s.autotune(cycles=8, warmup=1)
        assert best["ms_per_cycle"] > 0 and len(trials) >= 2
        assert {t["mode"] for t in trials} == {0, 1}
        assert best["ms_per_cycle"] == min(t["ms_per_cycle"] for t in trials if t["ms_per_cycle"] > 0)
        # the schedule axes: micro-partition size x levels per barrier
        assert {(t["mpart_lanes"], t["levels_per_barrier"]) for t in trials} == {
            (a, b) for a in (32, 64, 128) for b in (1, 2, 4)}
        o = s.options()
        assert (o["groups_per_item"], o["warps_per_block"], o["mode"]) == (
            best["groups_per_item"], best["warps_per_block"], best["mode"])
        assert (o["mpart_lanes"], o["levels_per_barrier"]) == (best["mpart_lanes"], best["levels_per_barrier"])
        got = s.batch_run(cyc, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cyc, stim, cycle_digests=True)
    np.testing.assert_array_equal(got.cycle_digest, ref["cycle_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])
