"""Early exit on stop (TGS_BATCH_STOP_EXIT, tgs_eval_until_stop): a stream
that executes a stop op freezes after that cycle.  Its results must equal the
oracle run for exactly (stop cycle + 1) cycles; streams that never stop run
the full length; the launch ends when every stream stopped.  Queued streams
retire at their stop and free their slot for the next queued stream."""
import numpy as np
import pytest

from oracle import pyoracle
from toucangpurt_gb300 import capi, sim, workloads

pytestmark = pytest.mark.gpu

NO_STOP = 0xFFFFFFFF


@pytest.fixture(scope="module")
def stop_design(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("stopexit")
    dp, sp = d / "d.bin", d / "s.bin"
    return dp, sp, sim.generate(dp, sp, **workloads.design_config("small", seed=15, with_stop=2))


def _expected(dp, sp, info, n, cycles, stim):
    od = pyoracle.OracleDesign(dp, sp)
    full = od.run(np.full(n, cycles, np.uint32), stim)
    sc = full["stop_cycle"].astype(np.int64)
    lens = np.where(sc == NO_STOP, cycles, np.minimum(sc + 1, cycles)).astype(np.uint32)
    return lens, od.run(lens, stim, cycle_digests=True)


@pytest.mark.parametrize("mode", [capi.MODE_PERSISTENT, capi.MODE_GRAPH])
def test_batch_stop_exit_matches_truncated_oracle(stop_design, mode):
    dp, sp, info = stop_design
    n, cycles = 24, 60
    stim = sim.StimulusSpec(3, info["pi_ids"], info["pi_bits"])
    lens, ref = _expected(dp, sp, info, n, cycles, stim)
    assert (lens < cycles).any(), "the design should stop some streams"
    with sim.Simulator(n_streams=n, mode=mode) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(np.full(n, cycles, np.uint32), stim, cycle_digests=True, stop_exit=True)
    np.testing.assert_array_equal(got.stop_cycle, ref["stop_cycle"])
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])
    np.testing.assert_array_equal(got.rolling_digest, ref["rolling_digest"])
    for q in range(n):
        np.testing.assert_array_equal(got.cycle_digest[q, : lens[q]], ref["cycle_digest"][q, : lens[q]])
        assert not got.cycle_digest[q, lens[q]:].any()
    assert got.stream_cycles == int(lens.sum())


@pytest.mark.parametrize("mode", [capi.MODE_PERSISTENT, capi.MODE_GRAPH])
def test_eval_until_stop_single_stream(stop_design, mode):
    dp, sp, info = stop_design
    # find a register start value that makes stream 0 stop: run the oracle
    st = pyoracle.OracleState(pyoracle.OracleDesign(dp, sp, randomize=True))
    stopped_at = None
    for c in range(200):
        if st.eval(1):
            stopped_at = c
            break
    if stopped_at is None:
        pytest.skip("no stop within 200 free-running cycles for this start state")
    ref = pyoracle.OracleState(pyoracle.OracleDesign(dp, sp, randomize=True))
    ref.eval(stopped_at + 1)
    with sim.Simulator(mode=mode) as s:
        s.init(0, dp, sp, True, False)
        stop, ran = s.eval_until_stop(500)
        assert stop and ran == stopped_at + 1
        assert s.real_cycles() == ran and s.cycle_cnt() == ran
        np.testing.assert_array_equal(s.reg_pool(), ref.regs())
        np.testing.assert_array_equal(s.mem_pool(), ref.mems())
        # every stream stopped: a second call runs nothing
        assert s.eval_until_stop(10) == (True, 0)


@pytest.mark.parametrize("mode", [capi.MODE_PERSISTENT, capi.MODE_GRAPH])
def test_queued_stop_exit_retires_stopped_streams(stop_design, mode):
    """Queued streams (ragged lengths, 8 slots): a stream that stops retires
    after its stop cycle and frees its slot for the next queued stream."""
    dp, sp, info = stop_design
    n = 40
    cycles = (3 + (np.arange(n) * 7) % 45).astype(np.uint32)
    stim = sim.StimulusSpec(5, info["pi_ids"], info["pi_bits"])
    od = pyoracle.OracleDesign(dp, sp)
    full = od.run(cycles, stim)
    sc = full["stop_cycle"].astype(np.int64)
    lens = np.where(sc == NO_STOP, cycles, np.minimum(sc + 1, cycles)).astype(np.uint32)
    assert (lens < cycles).any() and (lens == cycles).any()
    ref = od.run(lens, stim, cycle_digests=True)
    with sim.Simulator(n_streams=8, mode=mode) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cycles, stim, cycle_digests=True, stop_exit=True, slots=8)
        plain = s.batch_run(cycles, stim, slots=8)
    np.testing.assert_array_equal(got.stop_cycle, full["stop_cycle"])
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])
    np.testing.assert_array_equal(got.rolling_digest, ref["rolling_digest"])
    for q in range(n):
        np.testing.assert_array_equal(got.cycle_digest[q, : lens[q]], ref["cycle_digest"][q, : lens[q]])
        assert not got.cycle_digest[q, lens[q]:].any()
    assert got.stream_cycles == int(lens.sum())
    # without stop exit the same queue runs every stream to its length
    np.testing.assert_array_equal(plain.final_reg_digest, full["final_reg_digest"])
    np.testing.assert_array_equal(plain.stop_cycle, full["stop_cycle"])
    assert plain.stream_cycles == int(cycles.sum())


def test_queued_slot_limit(stop_design):
    dp, sp, info = stop_design
    with sim.Simulator(n_streams=8) as s:
        s.init(0, dp, sp, False, False)
        with pytest.raises(capi.TgsError):
            s.batch_run(np.arange(5, 5 + 4200, dtype=np.uint32) % 30 + 1, None, slots=4104)
