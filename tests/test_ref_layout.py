"""The device netlist layout that drives the reference's own kernels in the
GPU harness (oracle/ref_layout.h, restated from copy_netlist_to_gpu /
copyMicroPartToNetlist, src/SimEval.cu:69-148,1114-1343) against the
reference's own host code: the reference's src/SimEval.cu, Serializer.cpp and
SimInit.cpp, built from its tree (oracle/Makefile) and run against a
test-double CUDA runtime (oracle/fake_cudart.cpp), write their layout into
host memory; both layouts are printed in one canonical form
(oracle/layout_canon.h: every buffer's size and digest, every scalar field,
no addresses) and must be equal.  Every committed fixture design (the ones
the reference kernel ran to make tests/golden/refgpu_golden.json) and the
1M- and mixed 4M-LUT benchmark designs.  Skipped without the reference
checkout (the reference-side tool is not built then)."""
import subprocess
from pathlib import Path

import pytest

from oracle import pyoracle
from toucangpurt_gb300 import sim, workloads

HERE = Path(__file__).resolve().parent
DUMP = pyoracle.HERE / "_build" / "layout_dump"
REF = pyoracle.HERE / "_ref" / "ref_layout"
FIXTURES = sorted(p.name for p in (HERE / "golden").glob("*.bin"))


def _layouts(design: Path):
    a = subprocess.run([str(DUMP), str(design)], capture_output=True, text=True, timeout=600)
    b = subprocess.run([str(REF), str(design)], capture_output=True, text=True, timeout=600)
    assert a.returncode == 0, a.stderr
    assert b.returncode == 0, b.stderr
    return a.stdout, b.stdout


@pytest.fixture(scope="module")
def tools(built):
    pyoracle.build()
    if not REF.exists():
        pytest.skip("reference checkout not available: the reference-side layout tool is not built")
    assert DUMP.exists()


@pytest.mark.parametrize("name", FIXTURES)
def test_fixture_design_layout_equals_reference(tools, name):
    ours, ref = _layouts(HERE / "golden" / name)
    assert "partitions ok" in ref
    assert ours == ref


@pytest.mark.parametrize("workload", ["scale", "learned"])
def test_benchmark_design_layout_equals_reference(tools, tmp_path, workload):
    dp, sp = tmp_path / "d.bin", tmp_path / "s.bin"
    sim.generate(dp, sp, **workloads.design_config(workload))
    ours, ref = _layouts(dp)
    assert ours.count("\npart ") > 100
    assert ours == ref
