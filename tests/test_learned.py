"""Learned cost model: the GPU forward / backward kernels against a NumPy
reference, training, and the learned schedule (bit-exact values, gain over
the gate-count schedule)."""
import numpy as np
import pytest

from tests import mlp_ref
from toucangpurt_gb300 import sim, workloads


def _params(seed=0):
    rng = np.random.default_rng(seed)
    p = rng.normal(0, 0.2, mlp_ref.N_PARAMS).astype(np.float32)
    return p


def test_reference_gradient_matches_finite_differences():
    rng = np.random.default_rng(1)
    p = _params(1).astype(np.float64)
    X = rng.uniform(0, 3, (40, 16))
    y = rng.normal(0, 1, 40)
    g, _ = mlp_ref.grad(p, X, y)
    for i in rng.choice(p.size, 25, replace=False):
        e = np.zeros_like(p)
        e[i] = 1e-6
        num = (mlp_ref.grad(p + e, X, y)[1] - mlp_ref.grad(p - e, X, y)[1]) / 2e-6
        assert abs(num - g[i]) <= 1e-5 + 1e-4 * abs(num), i


@pytest.mark.gpu
def test_forward_kernel_matches_reference(built):
    rng = np.random.default_rng(2)
    p = _params(2)
    X = rng.uniform(0, 4, (777, 16)).astype(np.float32)
    got = sim.mlp_forward(p, X)
    ref, _ = mlp_ref.forward(p.astype(np.float64), X.astype(np.float64))
    np.testing.assert_allclose(got, ref, rtol=1e-4, atol=1e-4)


@pytest.mark.gpu
def test_gradient_kernel_matches_reference(built):
    rng = np.random.default_rng(3)
    p = _params(3)
    X = rng.uniform(0, 4, (1000, 16)).astype(np.float32)
    y = rng.normal(0, 1, 1000).astype(np.float32)
    g, loss = sim.mlp_grad(p, X, y)
    gr, lr = mlp_ref.grad(p.astype(np.float64), X.astype(np.float64), y.astype(np.float64))
    np.testing.assert_allclose(loss, lr, rtol=1e-4)
    scale = np.abs(gr).max()
    np.testing.assert_allclose(g, gr, rtol=2e-3, atol=2e-5 * scale)


@pytest.fixture(scope="module")
def mixed_design(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("mixed")
    dp, sp = d / "d.bin", d / "s.bin"
    info = sim.generate(dp, sp, **workloads.design_config("learned", n_lut=300_000, n_mems=64, ff_bits=32768,
                                                             luts_per_part=4000))
    return dp, sp, info


@pytest.mark.gpu
def test_training_learns_costs_and_keeps_values_exact(mixed_design):
    from oracle import pyoracle

    dp, sp, info = mixed_design
    n = 32
    with sim.Simulator(n_streams=n) as s:
        s.init(0, dp, sp, False, False)
        X = s.mpart_features()
        c = s.profile_mparts(20)
        assert (c > 0).all()
        rep = s.train_cost_model(X, c, epochs=40, seed=5)
        assert rep["val_mse"] < 0.5            # standardised: well below the variance (1.0)
        assert rep["val_corr"] > rep["gate_corr"]
        state = s.cost_model_state()
        stim = sim.StimulusSpec(8, info["pi_ids"], info["pi_bits"])
        cyc = np.full(n, 25, np.uint32)
        s.set_options(schedule=sim.capi.SCHED_LEARNED)
        got = s.batch_run(cyc, stim, cycle_digests=True)
    ref = pyoracle.OracleDesign(dp, sp).run(cyc, stim, cycle_digests=True)
    np.testing.assert_array_equal(got.cycle_digest, ref["cycle_digest"])
    np.testing.assert_array_equal(got.final_mem_digest, ref["final_mem_digest"])
    # the state round-trips into a fresh handle
    with sim.Simulator(n_streams=n, schedule=sim.capi.SCHED_LEARNED) as s2:
        s2.set_cost_model_state(state)
        s2.init(0, dp, sp, False, False)
        np.testing.assert_array_equal(s2.cost_model_state(), state)


@pytest.mark.gpu
@pytest.mark.parametrize("packing", [0, 1])
def test_learned_schedule_no_regression(mixed_design, packing):
    """On a small heterogeneous design, where every exec level holds about
    as many units as a block has warps, the schedule has little to balance:
    the learned one must not be slower than the gate-count one beyond 4 %
    (measured 0.98-1.01x over runs; the gain itself is asserted on the
    benchmarked design below)."""
    dp, sp, info = mixed_design
    n, cycles = 64, 60
    stim = sim.StimulusSpec(8, info["pi_ids"], info["pi_bits"])
    cyc = np.full(n, cycles, np.uint32)
    with sim.Simulator(n_streams=n, lane_packing=packing) as s:
        s.init(0, dp, sp, False, False)
        s.train_cost_model(s.mpart_features(), s.profile_mparts(20), epochs=40, seed=5)
        t = {"greedy": [], "learned": []}
        # the two schedules alternate, so clock drift does not favour either
        for _ in range(5):
            for name, sched in (("greedy", sim.capi.SCHED_GREEDY), ("learned", sim.capi.SCHED_LEARNED)):
                s.set_options(schedule=sched)
                s.batch_run(cyc, stim, rolling=False)  # warm
                t[name].append(min(s.batch_run(cyc, stim, rolling=False).device_ms for _ in range(2)))
    g, l = min(t["greedy"]), min(t["learned"])
    print(f"lane_packing={packing}: greedy {g:.2f} ms, learned {l:.2f} ms, gain {g / l:.3f}x")
    assert l <= g * 1.04


@pytest.mark.gpu
def test_learned_schedule_gain_on_benchmarked_design(tmp_path, built):
    """The benchmarked learned-partitioning workload: the mixed 4M-LUT design
    (datapath, deep control, memory-heavy and high-fan-out regions) with 256
    streams, about 8 items per partition spread over the blocks.  Gate count
    mispredicts the cost of its micro-partitions (memory ports, vector ops,
    word-wide palette ops, deep cones); the network, trained on about 200K
    clock64 samples (every micro-partition, over several profiling passes),
    balances blocks and warps by predicted cost.
    Measured: 1.06x (31.0 ms against 33.0 ms for 40 cycles); asserted: a real
    gain of at least 3 %."""
    from toucangpurt_gb300 import workloads

    dp, sp = tmp_path / "d.bin", tmp_path / "s.bin"
    info = sim.generate(dp, sp, **workloads.design_config("learned"))
    streams, cycles = 256, 40
    stim = sim.StimulusSpec(8, info["pi_ids"], info["pi_bits"])
    cyc = np.full(streams, cycles, np.uint32)
    s, notes = workloads.bench_simulator("learned", dp, sp, streams=streams)
    try:
        cm = notes["cost_model"]
        assert cm["samples"] >= 150_000  # per-micro-partition clock64 samples of several profiling passes
        assert cm["val_corr"] > 0.9 and cm["val_corr"] > cm["gate_corr"]
        t = {"greedy": [], "learned": []}
        for _ in range(3):
            for name, sched in (("greedy", sim.capi.SCHED_GREEDY), ("learned", sim.capi.SCHED_LEARNED)):
                s.set_options(schedule=sched)
                s.batch_run(cyc, stim, rolling=False)  # warm
                t[name].append(min(s.batch_run(cyc, stim, rolling=False).device_ms for _ in range(2)))
    finally:
        s.cleanup()
    g, l = min(t["greedy"]), min(t["learned"])
    print(f"mixed 4M-LUT x {streams}: greedy {g:.2f} ms, learned {l:.2f} ms, gain {g / l:.3f}x, {cm}")
    assert g / l >= 1.03
