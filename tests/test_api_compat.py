"""Source compatibility of the C++ host API with the reference.

The reference's own driver (main.cpp, unmodified) and a testbench written
against the reference API compile and link against include/ and the library;
on a GPU the testbench's results equal the oracle's.
"""
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from oracle import pyoracle

ROOT = Path(__file__).resolve().parents[1]
REF_DIR = pyoracle.reference_dir()  # where oracle/Makefile finds the reference checkout, or None
REF_MAIN = REF_DIR / "main.cpp" if REF_DIR else None
CUDA_INC = "/usr/local/cuda/include"


def _compile(src: Path, out: Path, extra=()):
    from toucangpurt_gb300 import build

    lib = build.build()
    cmd = ["g++", "-std=c++20", "-O1", f"-I{ROOT / 'include'}", f"-I{CUDA_INC}", str(src), *extra,
           f"-L{lib.parent}", "-ltoucan_gb300", f"-Wl,-rpath,{lib.parent}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


@pytest.mark.skipif(REF_MAIN is None or not REF_MAIN.exists(), reason="reference checkout not present")
@pytest.mark.parametrize("profile", [False, True])
def test_reference_main_compiles_unmodified(tmp_path, built, profile):
    extra = ["-DENABLE_SIM_PROFILE"] if profile else []
    _compile(REF_MAIN, tmp_path / "test_run", extra)


def test_testbench_compiles(tmp_path, built):
    _compile(ROOT / "tests" / "cpp" / "testbench.cpp", tmp_path / "tb")


@pytest.mark.gpu
def test_testbench_matches_oracle(tmp_path, small_design):
    from oracle import pyoracle

    dp, sp, info = small_design
    exe = _compile(ROOT / "tests" / "cpp" / "testbench.cpp", tmp_path / "tb")
    r = subprocess.run([str(exe), str(dp), str(sp), "7", "50"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = dict(l.split("=", 1) for l in r.stdout.splitlines() if "=" in l and not l.startswith("#"))
    # oracle: same testbench flow
    od = pyoracle.OracleDesign(dp, sp, randomize=True)
    st = pyoracle.OracleState(od)
    ids = info["pi_ids"][:8]
    for c in range(7):
        v = (0x9E3779B1 * (c + 1)) & 0xFFFFFFFF
        regs = st.regs()
        for j, rid in enumerate(ids):
            regs[rid] = (v >> (4 * j)) & 0xF
        st.eval(1)
    st.eval(50)
    regs = st.regs()
    # ff_k: nibbles 8k..8k+7 (most significant = highest id)
    for name, val in got.items():
        if name.startswith("ff_"):
            k = int(name[3:])
            exp = 0
            for j in reversed(range(8)):
                if 8 * k + j < info["reg_pool"]:
                    exp = (exp << 4) | int(regs[8 * k + j])
            assert int(val) == exp, name
    assert "#cycle_cnt=57 real_cycles=50" in r.stdout


@pytest.mark.gpu
def test_testbench_print_profile(tmp_path, small_design):
    """ToucanSimulator::printProfile after eval_free_running (the reference's
    profiling hook, src/ToucanSim.cu:307-315 over src/SimEval.cu:894-983):
    one line per partition with 0 < useful ticks <= total ticks."""
    dp, sp, info = small_design
    exe = _compile(ROOT / "tests" / "cpp" / "testbench.cpp", tmp_path / "tbp", ["-DENABLE_SIM_PROFILE"])
    r = subprocess.run([str(exe), str(dp), str(sp), "2", "250"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("Part ")]
    assert len(lines) == info["partitions"], r.stdout[-2000:]
    for l in lines:
        # "Part p, useful X%, ticks U, total ticks T"
        f = l.replace(",", "").split()
        useful, total = int(f[5]), int(f[8])
        assert 0 < useful <= total, l
