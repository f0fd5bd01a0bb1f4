"""Synthetic design generator: determinism, legality, configuration mapping."""
import hashlib

import numpy as np
import pytest

from toucangpurt_gb300 import sim, workloads


def _gen(tmp_path, name, **cfg):
    dp, sp = tmp_path / f"{name}.bin", tmp_path / f"{name}.sym"
    info = sim.generate(dp, sp, **cfg)
    return dp, sp, info


def test_deterministic(tmp_path, built):
    a = _gen(tmp_path, "a", **workloads.design_config("small"))
    b = _gen(tmp_path, "b", **workloads.design_config("small"))
    assert a[0].read_bytes() == b[0].read_bytes()
    c = _gen(tmp_path, "c", **workloads.design_config("small", seed=999))
    assert c[0].read_bytes() != a[0].read_bytes()


# sha256 prefixes of generated designs, computed on x86-64; the gpu-marked
# twin checks the same bytes on the aarch64 GPU host.
STABLE = {
    "small": (dict(workloads.design_config("small")), "482ab3ad1eba6da2"),
    "powerlaw": (dict(seed=12, n_lut=20000, levels=12, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=64,
                      ff_bits=2048, pi_bits=64, n_vec_ops=24, vec_nibbles=8, n_mems=3, mem_depth=4096, mem_width=32,
                      mem_read_ports=2, mem_write_ports=2, mem_multi_writer=1, luts_per_part=2500, cone_depth=2),
                 "cd639344cc83bac5"),
}


def _check_stable(tmp_path):
    for name, (cfg, sha) in STABLE.items():
        dp, _, _ = _gen(tmp_path, name, **cfg)
        assert hashlib.sha256(dp.read_bytes()).hexdigest()[:16] == sha, name


def test_designs_are_byte_stable(tmp_path, built):
    _check_stable(tmp_path)


@pytest.mark.gpu
def test_designs_are_byte_stable_on_gpu_host(tmp_path, built):
    _check_stable(tmp_path)


@pytest.mark.parametrize("name", ["small", "scale"])
def test_workload_designs_validate(tmp_path, built, name):
    cfg = workloads.design_config(name)
    if name == "scale":
        cfg.update(n_lut=200_000, n_mems=4, n_vec_ops=64)  # scaled down for the CPU suite
    dp, sp, info = _gen(tmp_path, name, **cfg)
    assert sim.validate_file(dp, sp) == info["lut_ops"]
    assert info["lut_ops"] >= cfg["n_lut"] * 0.98


def test_mixed_regions_validate(tmp_path, built):
    cfg = workloads.design_config("learned", n_lut=200_000, n_mems=64, ff_bits=32768)
    dp, sp, info = _gen(tmp_path, "mixed", **cfg)
    assert sim.validate_file(dp, sp) == info["lut_ops"]
    assert info["mem_read_ops"] > 0


@pytest.mark.parametrize("depth,width", [(1, 32), (2, 32), (4, 16), (8, 8), (40, 4)])
def test_cone_shapes(tmp_path, built, depth, width):
    cfg = dict(seed=3, n_lut=8000, levels=80, operands=3, ff_bits=1024, pi_bits=32, n_mems=1, mem_depth=256,
               mem_width=32, mem_read_ports=1, mem_write_ports=1, luts_per_part=4000, cone_depth=depth,
               mpart_width=width)
    dp, sp, info = _gen(tmp_path, f"c{depth}", **cfg)
    assert sim.validate_file(dp, sp) == info["lut_ops"]


def test_primary_inputs_layout(tmp_path, built):
    dp, sp, info = _gen(tmp_path, "pi", **workloads.design_config("batch"))
    ids, bits = info["pi_ids"], info["pi_bits"]
    assert ids.size == 8 + 1  # 32 input bits + one reset line
    assert (np.diff(ids) == 1).all()
    assert bits[-1] == 1 and (bits[:-1] == 4).all()
    assert ids.max() < info["reg_pool"]


def test_stream_lengths_log_uniform():
    c = workloads.stream_lengths("batch")
    assert c.size == 4096 and c.min() >= 1000 and c.max() <= 100_000
    # mean of a log-uniform on [1e3, 1e5] is (1e5 - 1e3) / ln(100) ~ 21.5K
    assert 19_000 < c.mean() < 24_000
