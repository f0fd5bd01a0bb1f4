"""Batched runs: in-place retirement / admission of queued streams, host
stimulus tables, continued runs.  All compared bit-exact with the oracle."""
import numpy as np
import pytest

from oracle import pyoracle
from toucangpurt_gb300 import sim, workloads


def _design(tmp_path_factory, name, **cfg):
    d = tmp_path_factory.mktemp(name)
    dp, sp = d / "d.bin", d / "s.bin"
    return dp, sp, sim.generate(dp, sp, **cfg)


@pytest.fixture(scope="module")
def batch_design(tmp_path_factory, built):
    return _design(tmp_path_factory, "batch", **workloads.design_config("batch"))


def test_host_table_matches_device_hash(batch_design):
    """The host-side table generator reproduces the seeded device values."""
    from oracle import pyoracle as po

    dp, sp, info = batch_design
    spec = sim.StimulusSpec(77, info["pi_ids"], info["pi_bits"])
    tab = sim.stimulus_table(spec, 3, 5, 2)
    seeds = [po.lib().orc_mix64(77 ^ s) for s in range(3)]
    for c in range(2):
        for i in range(len(info["pi_ids"])):
            for s in range(3):
                h = po.lib().orc_mix64(seeds[s] ^ po.lib().orc_mix64(((5 + c) << 32) | i))
                assert tab[c, i, s] == h & ((1 << int(info["pi_bits"][i])) - 1)


def test_host_table_toggles_follow_device_rule(batch_design):
    """Toggle inputs in the host table flip the previous value exactly when
    the device would (h >> 48 < toggle)."""
    from oracle import pyoracle as po

    dp, sp, info = batch_design
    ids, bits = info["pi_ids"], info["pi_bits"]
    tog = np.where(np.arange(len(ids)) % 2 == 0, 20000, 0).astype(np.uint16)
    spec = sim.StimulusSpec(9, ids, bits, tog)
    n, c0, cyc = 3, 4, 5
    prev = (np.arange(len(ids) * n, dtype=np.uint8).reshape(len(ids), n) & 15)
    tab = sim.stimulus_table(spec, n, c0, cyc, prev=prev)
    seeds = [po.lib().orc_mix64(9 ^ s) for s in range(n)]
    cur = prev.astype(int).copy()
    for c in range(cyc):
        for i in range(len(ids)):
            mask = (1 << int(bits[i])) - 1
            for s in range(n):
                h = po.lib().orc_mix64(seeds[s] ^ po.lib().orc_mix64(((c0 + c) << 32) | i))
                if tog[i]:
                    cur[i, s] = cur[i, s] ^ mask if (h >> 48) < tog[i] else cur[i, s]
                else:
                    cur[i, s] = h & mask
                assert tab[c, i, s] == cur[i, s]


@pytest.mark.gpu
def test_toggle_tables_match_seeded_run(batch_design):
    """Continued calls fed by toggle-aware host tables equal one seeded run."""
    dp, sp, info = batch_design
    n, steps, per = 16, 3, 11
    tog = workloads.toggles("batch", info["pi_bits"])
    spec = sim.StimulusSpec(21, info["pi_ids"], info["pi_bits"], tog)
    with sim.Simulator(n_streams=n) as s:
        s.init(0, dp, sp, False, False)
        prev = np.repeat(s.reg_pool(0)[info["pi_ids"]][:, None], n, axis=1)
        for k in range(steps):
            tab = sim.stimulus_table(spec, n, k * per, per, prev=prev)
            prev = tab[-1]
            tspec = sim.StimulusSpec(21, info["pi_ids"], info["pi_bits"], table=tab)
            got = s.batch_run(np.full(n, per, np.uint32), tspec, continue_=k > 0, final_digests=k == steps - 1)
    ref = pyoracle.OracleDesign(dp, sp).run(np.full(n, steps * per, np.uint32), spec)
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])
    np.testing.assert_array_equal(got.rolling_digest, ref["rolling_digest"])


@pytest.mark.gpu
@pytest.mark.parametrize("n,slots", [(20, 8), (37, 16), (64, 64), (100, 24)])
def test_admission_matches_oracle(batch_design, n, slots):
    dp, sp, info = batch_design
    rng = np.random.default_rng(n)
    cycles = rng.integers(5, 60, n).astype(np.uint32)
    tog = workloads.toggles("batch", info["pi_bits"])
    stim = sim.StimulusSpec(99, info["pi_ids"], info["pi_bits"], tog)
    with sim.Simulator(n_streams=8) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cycles, stim, cycle_digests=True, slots=slots)
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim, cycle_digests=True)
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])
    np.testing.assert_array_equal(got.rolling_digest, ref["rolling_digest"])
    np.testing.assert_array_equal(got.stop_cycle, ref["stop_cycle"])
    for q in range(n):
        np.testing.assert_array_equal(got.cycle_digest[q, : cycles[q]], ref["cycle_digest"][q, : cycles[q]])
    assert got.stream_cycles == int(cycles.sum())


@pytest.mark.gpu
def test_admission_without_cycle_digests(batch_design):
    """Final digests come from the retire cycle even without per-cycle digests."""
    dp, sp, info = batch_design
    cycles = np.array([7, 30, 3, 19, 44, 2, 11, 25, 9, 13], np.uint32)
    stim = sim.StimulusSpec(5, info["pi_ids"], info["pi_bits"])
    with sim.Simulator(n_streams=8) as s:
        s.init(0, dp, sp, True, False)
        got = s.batch_run(cycles, stim, rolling=False, slots=8)
    ref = pyoracle.OracleDesign(dp, sp, randomize=True).run(cycles, stim)
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])


@pytest.mark.gpu
def test_admission_stop_cycles(tmp_path_factory, built):
    dp, sp, info = _design(tmp_path_factory, "stop", **workloads.design_config("small", seed=15, with_stop=1))
    cycles = np.array([3, 9, 1, 14, 6, 2, 8, 12, 5, 4, 7], np.uint32)
    stim = sim.StimulusSpec(3, info["pi_ids"], info["pi_bits"])
    with sim.Simulator(n_streams=8) as s:
        s.init(0, dp, sp, False, False)
        got = s.batch_run(cycles, stim, slots=8)
    ref = pyoracle.OracleDesign(dp, sp).run(cycles, stim)
    np.testing.assert_array_equal(got.stop_cycle, ref["stop_cycle"])
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])


@pytest.mark.gpu
def test_table_and_continue_match_single_run(batch_design):
    """A run split into continued calls fed by host tables equals one seeded
    run of the same length (and the oracle)."""
    dp, sp, info = batch_design
    n, steps, per = 24, 4, 15
    spec = sim.StimulusSpec(11, info["pi_ids"], info["pi_bits"])
    with sim.Simulator(n_streams=n) as s:
        s.init(0, dp, sp, False, False)
        one = s.batch_run(np.full(n, steps * per, np.uint32), spec)
        pinned = sim.PinnedBuffer((per, len(info["pi_ids"]), n))
        for k in range(steps):
            sim.stimulus_table(spec, n, k * per, per, out=pinned.array)
            tspec = sim.StimulusSpec(11, info["pi_ids"], info["pi_bits"], table=pinned.array)
            got = s.batch_run(np.full(n, per, np.uint32), tspec, continue_=k > 0, final_digests=(k == steps - 1))
        pinned.free()
    ref = pyoracle.OracleDesign(dp, sp).run(np.full(n, steps * per, np.uint32), spec)
    np.testing.assert_array_equal(one.final_reg_digest, ref["final_reg_digest"])
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])
    np.testing.assert_array_equal(got.rolling_digest, ref["rolling_digest"])
