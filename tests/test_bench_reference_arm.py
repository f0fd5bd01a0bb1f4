"""The reference arm of bench.py runs on the host alone (the CPU evaluation of
the same synthetic design): its JSON line carries the fields the benchmark
contract asks for, and its timing counts cycles only (a run of 1 + k cycles
less a run of 1 cycle)."""
import json
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_line(built):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "small",
                        "--steps", "1", "--warmup", "1", "--cpu-sample-cycles", "50"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["unit"] == "stimulus-cycles/s" and line["higher_is_better"] is True
    assert line["value"] > 0 and line["value"] == line["e2e"]["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] == 1  # one stream, one partition per region
    assert "less a run of 1 cycle" in cb["sample"]


def test_cycles_time_excludes_setup(small_design):
    """The differenced timing is positive and ignores the final digests."""
    import bench
    from oracle import pyoracle
    from toucangpurt_gb300 import sim

    dp, sp, info = small_design
    od = pyoracle.OracleDesign(dp, sp)
    stim = sim.StimulusSpec(3, info["pi_ids"], info["pi_bits"])
    assert bench.cpu_cycles_time(od, stim, 2, 20, 1) > 0
    full = od.run(np.full(2, 20, np.uint32), stim, threads=1)
    lean = od.run(np.full(2, 20, np.uint32), stim, threads=1, final_digests=False)
    np.testing.assert_array_equal(lean["rolling_digest"], full["rolling_digest"])
    assert not lean["final_mem_digest"].any() and full["final_mem_digest"].any()
