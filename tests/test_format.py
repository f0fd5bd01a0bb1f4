"""Design / symbol file format: byte compatibility with the reference
serializer (src/Serializer.cpp) and initial state (src/SimInit.cpp)."""
import ctypes as C
import shutil
import subprocess

import numpy as np
import pytest

from oracle import pyoracle
from toucangpurt_gb300 import capi, sim, workloads

REF_TOOL = pyoracle.REF_TOOL
need_ref = pytest.mark.skipif(not REF_TOOL.exists(), reason="reference checkout not built here (oracle/_ref)")

CFGS = {
    "small": workloads.design_config("small"),
    "vec_mem": dict(seed=12, n_lut=6000, levels=12, operands=3, palette_pct=40, ff_bits=2048, pi_bits=64,
                    n_vec_ops=24, vec_nibbles=8, n_mems=3, mem_depth=512, mem_width=32, mem_read_ports=2,
                    mem_write_ports=2, mem_multi_writer=1, luts_per_part=2500, cone_depth=2, with_stop=1),
}


@pytest.fixture(scope="module", params=list(CFGS))
def design(request, tmp_path_factory, built):
    d = tmp_path_factory.mktemp("fmt")
    dp, sp = d / "d.bin", d / "s.bin"
    info = sim.generate(dp, sp, **CFGS[request.param])
    return dp, sp, info


def _resave(fn, src, dst):
    capi.check(fn(str(src).encode(), str(dst).encode()))


def test_product_resave_is_byte_identical(design, tmp_path):
    dp, sp, _ = design
    _resave(capi.lib().tgs_resave_design, dp, tmp_path / "d2.bin")
    assert (tmp_path / "d2.bin").read_bytes() == dp.read_bytes()
    _resave(capi.lib().tgs_resave_symbols, sp, tmp_path / "s2.bin")
    assert len((tmp_path / "s2.bin").read_bytes()) == len(sp.read_bytes())


@need_ref
def test_reference_serializer_roundtrip_byte_identical(design, tmp_path):
    dp, sp, _ = design
    out = tmp_path / "ref.bin"
    subprocess.run([str(REF_TOOL), "roundtrip", str(dp), str(out)], check=True)
    assert out.read_bytes() == dp.read_bytes()
    r = subprocess.run([str(REF_TOOL), "identical", str(dp), str(out)], check=True, capture_output=True, text=True)
    assert r.stdout.strip() == "identical"


@need_ref
def test_reference_reads_symbols(design, tmp_path):
    dp, sp, _ = design
    out = tmp_path / "sym.bin"
    r = subprocess.run([str(REF_TOOL), "symtrip", str(sp), str(out)], check=True, capture_output=True, text=True)
    n_regs, n_sig, n_mem = map(int, r.stdout.split())
    assert n_regs > 0
    # the product reads the reference's re-serialization (hash-map order may differ)
    capi.check(capi.lib().tgs_resave_symbols(str(out).encode(), str(tmp_path / "again.bin").encode()))


def _initial(dp, sp, randomize):
    o = pyoracle.OracleDesign(dp, sp)
    regs = np.zeros(o.reg_pool, np.uint8)
    mems = np.zeros(o.mem_pool, np.uint8)
    capi.check(capi.lib().tgs_initial_state(str(dp).encode(), str(sp).encode(), randomize,
                                            regs.ctypes.data_as(capi.u8p), regs.size,
                                            mems.ctypes.data_as(capi.u8p), mems.size))
    return regs, mems


@pytest.mark.parametrize("randomize", [0, 1])
def test_initial_state_product_matches_oracle(design, randomize):
    dp, sp, _ = design
    regs, mems = _initial(dp, sp, randomize)
    od = pyoracle.OracleDesign(dp, sp, randomize=bool(randomize))
    np.testing.assert_array_equal(regs, od.initial_regs())
    np.testing.assert_array_equal(mems, od.initial_mems())
    if randomize:
        assert regs.any()


@need_ref
def test_initial_state_matches_reference_randomize(design, tmp_path):
    dp, sp, _ = design
    r, m = tmp_path / "r.bin", tmp_path / "m.bin"
    subprocess.run([str(REF_TOOL), "initstate", str(dp), str(sp), "1", str(r), str(m)], check=True)
    regs, mems = _initial(dp, sp, 1)
    np.testing.assert_array_equal(np.fromfile(r, np.uint8), regs)
    np.testing.assert_array_equal(np.fromfile(m, np.uint8), mems)


def test_truncated_and_corrupt_files(design, tmp_path):
    dp, sp, _ = design
    data = dp.read_bytes()
    for cut in (3, 20, len(data) // 2, len(data) - 1):
        p = tmp_path / f"cut{cut}.bin"
        p.write_bytes(data[:cut])
        with pytest.raises(capi.TgsError) as e:
            sim.validate_file(p)
        assert e.value.code == capi.ERR_FORMAT
    # absurd vector count: rejected before any allocation
    bad = bytearray(data)
    bad[13:21] = (2**62).to_bytes(8, "little")  # lut vector count
    p = tmp_path / "bad.bin"
    p.write_bytes(bytes(bad))
    with pytest.raises(capi.TgsError) as e:
        sim.validate_file(p)
    assert e.value.code == capi.ERR_FORMAT


def test_missing_file(tmp_path):
    with pytest.raises(capi.TgsError) as e:
        sim.validate_file(tmp_path / "nope.bin")
    assert e.value.code == capi.ERR_IO


def test_oracle_parser_agrees_on_sizes(design):
    dp, sp, info = design
    od = pyoracle.OracleDesign(dp, sp)
    assert od.reg_pool == info["reg_pool"]
    assert od.mem_pool == info["mem_pool"]
    assert od.lut_ops == info["lut_ops"]
    assert od.lut_ops == sim.validate_file(dp, sp)


_FUZZ_CHILD = r"""
import ctypes as C, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from toucangpurt_gb300 import capi, sim
from pathlib import Path
src, work, seed, n = Path(sys.argv[2]), Path(sys.argv[3]), int(sys.argv[4]), int(sys.argv[5])
data = src.read_bytes()
rng = np.random.default_rng(seed)
accepted = rejected = 0
for k in range(n):
    b = bytearray(data)
    mode = rng.integers(3)
    if mode == 0:  # a few random bytes
        for _ in range(rng.integers(1, 8)):
            b[rng.integers(len(b))] = rng.integers(256)
    elif mode == 1:  # a huge 64-bit count or offset
        pos = int(rng.integers(len(b) - 8))
        b[pos:pos + 8] = int(rng.integers(1 << 62)).to_bytes(8, "little")
    else:  # a large 32-bit field
        pos = int(rng.integers(len(b) - 4))
        b[pos:pos + 4] = int(rng.integers(1 << 31)).to_bytes(4, "little")
    p = work / "m.bin"
    p.write_bytes(bytes(b))
    try:
        sim.validate_file(p)
        accepted += 1
        st = capi.RepackStats()
        capi.check(capi.lib().tgs_repack_design(str(p).encode(), str(work / "r.bin").encode(), 0, 0, C.byref(st)))
        ss = capi.ScheduleStats()
        capi.check(capi.lib().tgs_plan_schedule(str(p).encode(), 6, 4, 0, 2, 0, 0, 64, C.byref(ss)))
    except capi.TgsError:
        rejected += 1
print("fuzz", accepted, rejected)
"""


def test_mutated_design_files_never_crash(design, tmp_path):
    """Random byte, 32-bit and 64-bit field mutations of a design file: the
    bulk loader and the static checks reject it with an error code or accept
    it (and then repacking it and planning its schedule work); the process
    never crashes.  A child
    process, so a crash is reported instead of ending the test run."""
    import subprocess
    import sys
    from pathlib import Path

    dp, sp, _ = design
    root = str(Path(__file__).resolve().parents[1])
    r = subprocess.run([sys.executable, "-c", _FUZZ_CHILD, root, str(dp), str(tmp_path), "7", "300"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    accepted, rejected = map(int, r.stdout.split()[-2:])
    assert accepted + rejected == 300 and rejected > 0
