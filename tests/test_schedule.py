"""The exec-level scheduler on the host (tgs_plan_schedule, no GPU): the
gate-count plan of every level block against the bounds any schedule and
any list schedule obey, the schedule knobs (micro-partition size, levels per
barrier), and argument checks."""
import ctypes as C

import pytest

from toucangpurt_gb300 import capi, sim, workloads

DESIGNS = {
    "small": workloads.design_config("small"),
    "deep_cones": dict(workloads.design_config("small"), seed=11, cone_depth=4, mpart_width=16, n_lut=6000, levels=16),
    "mixed": dict(seed=14, n_lut=40000, levels=64, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=65536,
                  ff_bits=8192, pi_bits=64, n_mems=16, mem_depth=1024, mem_width=64, mem_read_ports=2,
                  mem_write_ports=1, luts_per_part=4000, mpart_width=32, cone_depth=1, mixed=1),
}


@pytest.fixture(scope="module")
def designs(tmp_path_factory, built):
    d = tmp_path_factory.mktemp("sched")
    out = {}
    for name, cfg in DESIGNS.items():
        dp, sp = d / f"{name}.bin", d / f"{name}.sym"
        sim.generate(dp, sp, **cfg)
        out[name] = dp
    return out


def plan(dp, warps=6, groups=4, lanes=0, lpb=0, packing=0, fast=0, streams=64):
    return sim.plan_schedule(dp, warps, groups, lanes, lpb, packing, fast, streams)


def test_c_abi_and_python_agree(designs):
    st = capi.ScheduleStats()
    capi.check(capi.lib().tgs_plan_schedule(str(designs["mixed"]).encode(), 6, 4, 0, 2, 0, 0, 64, C.byref(st)))
    assert {f: getattr(st, f) for f, _ in st._fields_ if not f.startswith("reserved")} == plan(designs["mixed"], lpb=2)


def test_repack_then_plan(designs, tmp_path):
    """A design rewritten the way tgs_init rewrites it plans like the original
    (the image is built from it with the same transforms, which are
    idempotent), with the same work."""
    out = tmp_path / "r.bin"
    st = sim.repack_design(designs["mixed"], out)
    assert st["exec_levels"] > 0
    a, b = plan(designs["mixed"]), plan(out)
    assert a["exec_levels"] == b["exec_levels"] and abs(a["work"] - b["work"]) <= 1e-6 * a["work"]


@pytest.mark.parametrize("name", list(DESIGNS))
@pytest.mark.parametrize("warps", [4, 6, 8, 16])
@pytest.mark.parametrize("groups", [1, 4])
def test_plan_within_bounds(designs, name, warps, groups):
    s = plan(designs[name], warps, groups)
    eps = 1e-6 * max(1.0, s["work"])
    assert s["blocks"] == s["exec_levels"] and s["fused_levels"] == 0
    assert 0 < s["barriers"] <= s["blocks"]
    assert s["level_bound"] - eps <= s["makespan"] <= s["list_bound"] + eps
    assert s["makespan"] >= s["work"] / warps - eps
    assert s["max_level_words"] * s["blocks"] >= s["schedule_words"] - 16 * s["blocks"]


@pytest.mark.parametrize("name", list(DESIGNS))
def test_work_independent_of_launch_shape(designs, name):
    works = {round(plan(designs[name], w, g)["work"], 6) for w in (4, 6, 8) for g in (1, 2, 4, 8)}
    assert len(works) == 1


@pytest.mark.parametrize("name", list(DESIGNS))
@pytest.mark.parametrize("lpb", [2, 4])
def test_fused_levels(designs, name, lpb):
    """Levels merge only where the merged block plans no longer than the
    levels apart: the plan's makespan never grows."""
    base = plan(designs[name], 6, 4)
    s = plan(designs[name], 6, 4, lpb=lpb)
    assert s["blocks"] + s["fused_levels"] == s["exec_levels"] == base["exec_levels"]
    assert s["makespan"] <= base["makespan"] * (1 + 1e-9)
    assert abs(s["work"] - base["work"]) <= 1e-6 * base["work"]


@pytest.mark.parametrize("name", list(DESIGNS))
@pytest.mark.parametrize("lanes", [64, 128])
def test_bundled_units(designs, name, lanes):
    """Bundling 32-lane units by two or four changes how work is split, not
    how much there is; no schedule beats the per-block bound."""
    base = plan(designs[name], 8, 1)
    s = plan(designs[name], 8, 1, lanes=lanes)
    assert abs(s["work"] - base["work"]) <= 1e-6 * base["work"]
    assert s["makespan"] >= s["level_bound"] * (1 - 1e-9)


def test_deterministic(designs):
    assert plan(designs["mixed"], 6, 4, lpb=2) == plan(designs["mixed"], 6, 4, lpb=2)


@pytest.mark.parametrize("kw", [dict(warps=0), dict(warps=33), dict(groups=3), dict(lanes=48), dict(lpb=3)])
def test_bad_arguments(designs, kw):
    with pytest.raises(capi.TgsError) as e:
        plan(designs["small"], **kw)
    assert e.value.code == capi.ERR_ARG


def test_missing_design(tmp_path):
    with pytest.raises(capi.TgsError) as e:
        plan(tmp_path / "none.bin")
    assert e.value.code == capi.ERR_IO


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(DESIGNS))
@pytest.mark.parametrize("streams,groups,lpb", [(64, 4, 0), (64, 4, 2), (8, 1, 0), (1, 1, 0)])
def test_plan_matches_live_schedule(designs, name, streams, groups, lpb):
    """The host-side plan is the schedule tgs_init builds: the same level
    blocks, barriers and fused levels."""
    dp = designs[name]
    with sim.Simulator(n_streams=streams, groups_per_item=groups, warps_per_block=6, levels_per_barrier=lpb) as s:
        s.init(0, dp, None, False, False)
        st = s.design_stats()
    p = plan(dp, 6, groups, 0, lpb, 0, 0, streams)
    assert (st["exec_levels"], st["block_barriers"], st["fused_levels"]) == (p["blocks"], p["barriers"],
                                                                              p["fused_levels"])
