"""Checkpoint / restore (tgs_dump_state, tgs_load_state): a run continued
from a checkpoint, in another handle with other launch options, equals the
uninterrupted run and the oracle."""
import numpy as np
import pytest

from oracle import pyoracle
from toucangpurt_gb300 import capi, sim, workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def design(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("ckpt")
    dp, sp = d / "d.bin", d / "s.bin"
    cfg = workloads.design_config("small", seed=31, n_mems=2)
    return dp, sp, sim.generate(dp, sp, **cfg)


def test_batch_continue_across_checkpoint(design, tmp_path):
    dp, sp, info = design
    n, first, second = 24, 17, 23
    stim = sim.StimulusSpec(5, info["pi_ids"], info["pi_bits"])
    with sim.Simulator(n_streams=n, groups_per_item=4) as s:
        s.init(0, dp, sp, True, False)
        s.batch_run(np.full(n, first, np.uint32), stim)
        s.dump_state(tmp_path / "ck.bin")
    with sim.Simulator(n_streams=8, groups_per_item=2, warps_per_block=4, mode=capi.MODE_GRAPH) as s2:
        s2.init(0, dp, sp, True, False)
        s2.load_state(tmp_path / "ck.bin")
        assert s2.options()["n_streams"] == n
        got = s2.batch_run(np.full(n, second, np.uint32), stim, continue_=True)
    ref = pyoracle.OracleDesign(dp, sp, randomize=True).run(np.full(n, first + second, np.uint32), stim)
    np.testing.assert_array_equal(got.final_reg_digest, ref["final_reg_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])
    np.testing.assert_array_equal(got.rolling_digest, ref["rolling_digest"])


def test_free_running_across_checkpoint(design, tmp_path):
    dp, sp, _ = design
    st = pyoracle.OracleState(pyoracle.OracleDesign(dp, sp))
    with sim.Simulator() as s:
        s.init(0, dp, sp, False, False)
        s.eval_free_running(40)
        s.dump_state(tmp_path / "ck.bin")
        s.eval_free_running(5)  # diverge, then restore
        s.load_state(tmp_path / "ck.bin")
        assert s.real_cycles() == 40 and s.cycle_cnt() == 40
        s.eval_free_running(30)
        st.eval(70)
        np.testing.assert_array_equal(s.reg_pool(), st.regs())
        np.testing.assert_array_equal(s.mem_pool(), st.mems())
        assert s.real_cycles() == 70 and s.cycle_cnt() == 70


def test_checkpoint_of_another_design_is_refused(design, tmp_path_factory, tmp_path):
    dp, sp, _ = design
    d2 = tmp_path_factory.mktemp("other")
    sim.generate(d2 / "d.bin", d2 / "s.bin", **workloads.design_config("small", seed=32))
    with sim.Simulator() as s:
        s.init(0, dp, sp, False, False)
        s.dump_state(tmp_path / "ck.bin")
    with sim.Simulator() as s2:
        s2.init(0, d2 / "d.bin", d2 / "s.bin", False, False)
        with pytest.raises(capi.TgsError):
            s2.load_state(tmp_path / "ck.bin")
        (tmp_path / "junk.bin").write_bytes(b"not a state file at all, nope.")
        with pytest.raises(capi.TgsError):
            s2.load_state(tmp_path / "junk.bin")


def test_truncated_checkpoint_leaves_handle_unchanged(design, tmp_path):
    """A state file shorter than its header announces is refused before the
    handle is reconfigured: stream count and state stay as they were."""
    dp, sp, info = design
    stim = sim.StimulusSpec(5, info["pi_ids"], info["pi_bits"])
    with sim.Simulator(n_streams=24) as s:
        s.init(0, dp, sp, True, False)
        s.batch_run(np.full(24, 9, np.uint32), stim)
        s.dump_state(tmp_path / "ck.bin")
    raw = (tmp_path / "ck.bin").read_bytes()
    (tmp_path / "short.bin").write_bytes(raw[:-1])
    (tmp_path / "long.bin").write_bytes(raw + b"\0")
    with sim.Simulator(n_streams=8) as s2:
        s2.init(0, dp, sp, True, False)
        s2.batch_run(np.full(8, 5, np.uint32), stim)
        before = [s2.digest(k) for k in range(8)]
        for name in ("short.bin", "long.bin"):
            with pytest.raises(capi.TgsError) as e:
                s2.load_state(tmp_path / name)
            assert e.value.code == capi.ERR_FORMAT
            assert s2.options()["n_streams"] == 8
            assert [s2.digest(k) for k in range(8)] == before
