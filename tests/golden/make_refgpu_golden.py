"""Golden fixtures from the reference's own GPU kernel.

Runs on a GB300 (needs oracle/_ref/ref_simeval.cubin, compiled by
oracle/Makefile from the reference's src/SimEval.cu, and the driver-API
harness oracle/_build/refgpu):

    python tests/golden/make_refgpu_golden.py <outdir>

For every case it writes the design/symbol files it ran (generated by the
seeded generator, or hand-built known-answer designs) and one JSON file with
the reference kernel's results: per-cycle register digests, rolling digest,
final register/memory digests and, for small designs, the full final pools.
The files are committed under tests/golden/ and checked by test_golden.py.
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

# name -> generator fields
GEN_CASES = {
    "small": dict(seed=101, n_lut=4096, levels=16, operands=2, ff_bits=512, pi_bits=32, n_mems=1, mem_depth=1024,
                  mem_width=32, mem_read_ports=1, mem_write_ports=1, luts_per_part=2048),
    "deep": dict(seed=11, n_lut=6000, levels=16, operands=2, ff_bits=512, pi_bits=32, n_mems=1, mem_depth=1024,
                 mem_width=32, mem_read_ports=1, mem_write_ports=1, luts_per_part=2048, cone_depth=4, mpart_width=16),
    "wide3op": dict(seed=12, n_lut=20000, levels=12, operands=3, palette_pct=40, ff_bits=2048, pi_bits=64,
                    n_vec_ops=24, vec_nibbles=8, n_mems=3, mem_depth=4096, mem_width=32, mem_read_ports=2,
                    mem_write_ports=2, mem_multi_writer=1, luts_per_part=2500, cone_depth=2),
    "vec16": dict(seed=13, n_lut=8000, levels=8, operands=3, ff_bits=4096, pi_bits=64, n_vec_ops=40, vec_nibbles=16,
                  n_mems=2, mem_depth=256, mem_width=64, mem_read_ports=1, mem_write_ports=1, luts_per_part=2000),
    "mixed": dict(seed=14, n_lut=40000, levels=64, operands=3, palette_pct=40, ff_bits=8192, pi_bits=64, n_mems=16,
                  mem_depth=1024, mem_width=64, mem_read_ports=2, mem_write_ports=1, luts_per_part=4000, mixed=1),
    "stop": dict(seed=15, n_lut=4096, levels=16, operands=2, ff_bits=512, pi_bits=32, n_mems=1, mem_depth=1024,
                 mem_width=32, mem_read_ports=1, mem_write_ports=1, luts_per_part=2048, with_stop=1),
    # more partitions per region than SMs: free running selects the _Large kernel
    "many_parts": dict(seed=16, n_lut=80000, levels=8, operands=2, ff_bits=8192, pi_bits=32, n_mems=0,
                       luts_per_part=200),
}

# (case, mode, randomize, cycles, streams, stim_seed, toggle16)
RUNS = [
    ("small", "eval", 0, 200, 3, 2024, 0),
    ("small", "free", 1, 1000, 1, 0, 0),
    ("deep", "eval", 0, 100, 2, 7, 0),
    ("wide3op", "eval", 0, 60, 2, 9, 0),
    ("wide3op", "free", 1, 300, 1, 0, 0),
    ("vec16", "eval", 1, 60, 2, 13, 0),
    ("mixed", "eval", 0, 40, 1, 14, 0),
    ("stop", "eval", 0, 40, 2, 3, 0),
    ("small", "eval", 0, 120, 2, 31, 3277),
    ("many_parts", "eval", 1, 30, 1, 5, 0),
    ("many_parts", "free", 1, 30, 1, 0, 0),
]


def run_harness(out: Path, design, symbols, randomize, mode, cycles, streams, stim_file) -> list[dict]:
    exe = ROOT / "oracle" / "_build" / "refgpu"
    cubin = ROOT / "oracle" / "_ref" / "ref_simeval.cubin"
    res = out / "tmp.jsonl"
    cmd = [str(exe), str(cubin), str(design), str(symbols) if symbols else "-", str(randomize), mode, str(cycles),
           str(streams), str(stim_file) if stim_file else "-", str(res)]
    subprocess.run(cmd, check=True, timeout=600)
    return [json.loads(l) for l in res.read_text().splitlines()]


def main(outdir: str) -> None:
    from tests import test_kat
    from toucangpurt_gb300 import build, sim

    build.build()
    build.build_oracle()
    out = Path(outdir)
    out.mkdir(parents=True, exist_ok=True)
    fixtures = {"generated": [], "kat": []}
    infos = {}
    for name, cfg in GEN_CASES.items():
        info = sim.generate(out / f"{name}.bin", out / f"{name}.sym", **cfg)
        infos[name] = info
    for name, mode, rnd, cycles, streams, seed, tog in RUNS:
        info = infos[name]
        stim = None
        if mode == "eval":
            stim = out / "stim.txt"
            lines = [f"{seed} {len(info['pi_ids'])}"]
            lines += [f"{int(r)} {int(b)} {tog}" for r, b in zip(info["pi_ids"], info["pi_bits"])]
            stim.write_text("\n".join(lines) + "\n")
        rows = run_harness(out, out / f"{name}.bin", out / f"{name}.sym", rnd, mode, cycles, streams, stim)
        fixtures["generated"].append({"case": name, "mode": mode, "randomize": rnd, "cycles": cycles, "streams": streams,
                                      "stim_seed": seed, "toggle": tog, "results": rows})
        print(name, mode, "ok", flush=True)
    for name in list(test_kat.CASES) + ["mem_write", "reg_copy_rounding", "stop_print"]:
        dp = out / f"kat_{name}.bin"
        test_kat.kat_design_with_inputs(name).write(dp)
        rows = run_harness(out, dp, None, 0, "eval", 3, 1, None)
        fixtures["kat"].append({"case": name, "results": rows})
        print("kat", name, "ok", flush=True)
    (out / "tmp.jsonl").unlink(missing_ok=True)
    (out / "stim.txt").unlink(missing_ok=True)
    (out / "refgpu_golden.json").write_text(json.dumps(fixtures, indent=1) + "\n")


if __name__ == "__main__":
    main(sys.argv[1])
