"""Golden digests of the reference's own GPU kernel on the benchmarked
configurations at full size.

Runs on a GB300 (needs oracle/_ref/ref_simeval.cubin, compiled by
oracle/Makefile from the reference's src/SimEval.cu, and the driver-API
harness oracle/_build/refgpu):

    python tests/golden/make_refgpu_fullsize.py <outdir>

For each benchmarked workload of toucangpurt_gb300.workloads (the seeded
1M-LUT, mixed 4M-LUT and 16M-LUT netlists) the design is regenerated from its
seed (the files are large and are not committed), run for one stream through
the reference's race-free eval() path (evalSingleCycle, one cooperative
launch per cycle, inputs written between cycles as
src/ToucanSim.cu:206-230 drives it) with the workload's primary-input
statistics, and the per-cycle register digests, final register, memory and
rolling digests are written to <outdir>/refgpu_fullsize.json (committed as
tests/golden/refgpu_fullsize.json, checked by tests/test_fullsize_golden.py).
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

# (workload, stimulus seed, cycles)
RUNS = [("scale", 2002, 24), ("learned", 4004, 24), ("largest", 5005, 24)]


def main(outdir: str) -> None:
    from toucangpurt_gb300 import build, sim, workloads

    build.build()
    build.build_oracle()
    exe = ROOT / "oracle" / "_build" / "refgpu"
    cubin = ROOT / "oracle" / "_ref" / "ref_simeval.cubin"
    out = Path(outdir)
    out.mkdir(parents=True, exist_ok=True)
    fixtures = []
    for name, seed, cycles in RUNS:
        dp, sp = out / f"{name}.bin", out / f"{name}.sym"
        info = sim.generate(dp, sp, **workloads.design_config(name))
        tog = workloads.toggles(name, info["pi_bits"])
        tog = tog if tog is not None else [0] * len(info["pi_ids"])
        stim = out / "stim.txt"
        stim.write_text(f"{seed} {len(info['pi_ids'])}\n" +
                        "".join(f"{int(r)} {int(b)} {int(t)}\n" for r, b, t in zip(info["pi_ids"], info["pi_bits"], tog)))
        res = out / "tmp.jsonl"
        subprocess.run([str(exe), str(cubin), str(dp), str(sp), "0", "eval", str(cycles), "1", str(stim), str(res)],
                       check=True, timeout=1800)
        rows = [json.loads(l) for l in res.read_text().splitlines()]
        fixtures.append({"case": name, "design_seed": workloads.DESIGN_SEEDS[name], "stim_seed": seed,
                         "cycles": cycles, "lut_ops": info["lut_ops"], "results": rows})
        print(name, "ok", rows[0]["kernel_ms"], "ms", flush=True)
        dp.unlink()
        sp.unlink()
        res.unlink()
        stim.unlink()
    (out / "refgpu_fullsize.json").write_text(json.dumps(fixtures, indent=1) + "\n")


if __name__ == "__main__":
    main(sys.argv[1])
