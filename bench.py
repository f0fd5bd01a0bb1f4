#!/usr/bin/env python3
"""Throughput benchmark of the GB300 Toucan netlist simulator.

Workload (default, N=1): the largest synthetic configuration that fits one
GPU -- a seeded 16M-LUT (3-operand) levelized netlist in 96 levels with 2M
flip-flops, 8K 64-bit vector ops and 256 memories of 256K x 32 (2R/2W), run
with 64 independent stimulus streams (1,024 primary-input bits each).  One
step = every stream advanced by --cycles-per-step cycles.

  value  : stimulus-cycles/s over the timed steps, device time (CUDA events on
           the library's stream), inputs resident in HBM.
  e2e    : the same through the C ABI with host buffers: host stimulus table
           uploaded and result digests read back inside the timed region.
  --impl reference : the CPU evaluation of the same design on the host cores
           (the reference has no CPU evaluator of its own: the oracle port is
           the reference arm).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "stimulus-cycles/s & LUT-evals/s: batched+learned vs plain, same GB300, bit-exact"


def args_parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference", "reference-gpu"])
    p.add_argument("--workload", default="largest")
    p.add_argument("--cycles-per-step", type=int, default=0)
    p.add_argument("--streams", type=int, default=0)
    p.add_argument("--groups", type=int, default=0, help="8-stream groups per item (0: the library's default)")
    p.add_argument("--warps", type=int, default=0, help="warps per block (0: the design's typical exec-level width)")
    p.add_argument("--schedule", default="auto", choices=["auto", "greedy", "learned"],
                   help="auto: the learned cost model for batched runs (more than one stream), greedy gate count "
                        "for the plain single-stream form")
    p.add_argument("--no-stage", action="store_true", help="read exec levels from global memory (same as --levels global)")
    p.add_argument("--levels", default="auto", choices=["auto", "resident", "global", "staged"],
                   help="where blocks read exec levels: resident in shared memory for the launch, staged per level, "
                        "or global memory (auto: resident when every block still fits on the GPU, else staged)")
    p.add_argument("--value-pool", default="compact", choices=["compact", "design"],
                   help="value-pool slots renumbered by live range (default) or as numbered in the design file")
    p.add_argument("--autotune", action="store_true", help="time the launch configurations first and keep the fastest")
    p.add_argument("--mode", default="auto", choices=["auto", "persistent", "graph"],
                   help="cycle loop as one persistent launch or as replayed CUDA-graph chunks (one launch per region); "
                        "auto: persistent when the exec levels stay resident in shared memory (short, latency-bound "
                        "levels: one launch keeps them for the whole run), else graph")
    p.add_argument("--slots", type=int, default=0, help="resident slots for queued streams of uneven length")
    p.add_argument("--no-cpu-baseline", action="store_true", help="skip the CPU baseline and the oracle parity check")
    p.add_argument("--no-baselines", action="store_true",
                   help="skip the plain single-stream form and the reference kernel run after the timed region")
    p.add_argument("--ref-cycles", type=int, default=20, help="cycles of the reference kernel's eval() run")
    p.add_argument("--cpu-sample-cycles", type=int, default=5)
    p.add_argument("--out", default="")
    p.add_argument("--set", action="append", default=[], metavar="OPTION=VALUE",
                   help="further tgs_options field of the simulator (e.g. fast_luts=1 for table lookups only)")
    p.add_argument("--override", action="append", default=[],
                   help="generator field override key=value (e.g. a smaller memory depth for profiling)")
    return p.parse_args()


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("gloo")
    return rank, ws


def local_gpu(ws: int) -> int:
    """This rank's GPU: LOCAL_RANK, wrapped onto the GPUs the node has (ranks
    are independent replicas, so more ranks than GPUs share them)."""
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    if ws == 1:
        return lr
    import torch

    return lr % max(1, torch.cuda.device_count())


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist

        dist.barrier()


def allreduce_max(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(x: float, ws: int) -> float:
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


class Clocks:
    """nvidia-smi samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.f.name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def profiled(key: str):
    """A figure of the committed ncu summary of the region kernel (small case
    of the same kernel): traffic_bytes_per_launch (dram__bytes_read.sum +
    dram__bytes_write.sum), smem_wavefronts_per_sm_cycle and
    smem_useful_wavefronts_per_sm_cycle (shared-memory wavefronts, without
    bank-conflict replays, per SM and cycle), or None."""
    import re

    try:
        t = (ROOT / "profiles" / "regionkernel_largest_64streams.md").read_text()
        return float(re.search(key + r": ([0-9.]+)", t).group(1))
    except Exception:
        return None


def measured_peak():
    try:
        d = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def make_design(workload: str, workdir: Path, rank: int, overrides=()):
    from toucangpurt_gb300 import sim, workloads

    ov = {}
    for kv in overrides:
        k, v = kv.split("=", 1)
        ov[k] = float(v) if "." in v else int(v)
    dp, sp = workdir / f"{workload}.bin", workdir / f"{workload}.sym"
    info = sim.generate(dp, sp, **workloads.design_config(workload, **ov))
    return dp, sp, info


def algorithmic_bytes(st: dict, streams: int, cycles: int) -> float:
    """Algorithmic bytes of `cycles` cycles of `streams` streams: instruction
    words (4 B per op slot) read once per cycle, plus 0.5 B per state nibble
    read or written per stream (registers, exchange, memories)."""
    instr = 4.0 * st["op_slots"]
    state = 0.5 * (st["l0_reg_reads"] + st["reg_copy_slots"] + st["l0_exg_reads"] + st["exg_copy_slots"]
                   + st["mem_read_ops"] + st["mem_write_ops"])
    return cycles * (instr + streams * state)


def cpu_threads(info, streams) -> int:
    """Host threads the oracle can use: streams run in parallel; a single
    stream runs the partitions of a region in parallel (more threads than
    partitions would only wait at the region barriers)."""
    n = os.cpu_count() or 1
    width = streams if streams > 1 else max(1, int(info.get("partitions", 2)) // 2)
    return max(1, min(n, width))


def cpu_cycles_time(od, stim, streams, cycles, threads):
    """Seconds the oracle spends on `cycles` cycles of `streams` streams:
    a run of 1 + cycles cycles minus a run of 1 cycle, so the per-run work
    the GPU timing leaves out too (state set-up, per-stream pool copies) is
    excluded; final digests are skipped in both."""
    one = np.full(streams, 1, np.uint32)
    more = np.full(streams, 1 + cycles, np.uint32)
    t0 = time.perf_counter()
    od.run(one, stim, threads=threads, final_digests=False)
    t1 = time.perf_counter()
    od.run(more, stim, threads=threads, final_digests=False)
    t2 = time.perf_counter()
    return max((t2 - t1) - (t1 - t0), 1e-9)


def cpu_sample(od, stim, streams, cycles, threads, min_s=0.5):
    """(seconds, cycles) of a CPU sample of at least `cycles` cycles, grown
    until it takes `min_s` or more: a small design's few cycles take
    microseconds, below what the difference of two runs resolves."""
    while True:
        dt = cpu_cycles_time(od, stim, streams, cycles, threads)
        if dt >= min_s or cycles >= 1 << 20:
            return dt, cycles
        cycles = min(1 << 20, cycles * max(2, min(64, int(1.5 * min_s / max(dt, 1e-5)) + 1)))


def run_reference(a, rank, ws):
    """Reference arm: CPU evaluation of the workload on all host threads."""
    if rank != 0:
        return
    from oracle import pyoracle
    from toucangpurt_gb300 import build, workloads

    build.build()
    pyoracle.build()
    wd = Path(tempfile.mkdtemp(prefix="tgs_ref_"))
    dp, sp, info = make_design(a.workload, wd, 0, a.override)
    streams = a.streams or workloads.RUNS[a.workload]["streams"]
    cyc = a.cpu_sample_cycles
    threads = cpu_threads(info, streams)
    from oracle import pyoracle as po
    from toucangpurt_gb300 import sim

    od = po.OracleDesign(dp, sp)
    stim = sim.StimulusSpec(1234, info["pi_ids"], info["pi_bits"], workloads.toggles(a.workload, info["pi_bits"]))
    _, cyc = cpu_sample(od, stim, streams, cyc, threads)
    for _ in range(a.warmup - 1):
        cpu_cycles_time(od, stim, streams, cyc, threads)
    dt = sum(cpu_cycles_time(od, stim, streams, cyc, threads) for _ in range(a.steps))
    v = streams * cyc * a.steps / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "stimulus-cycles/s", "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1000 * dt / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "u8 nibbles", "data": "synthetic (seeded generator)",
        "config": {"workload": f"{a.workload}: {info['lut_ops']} LUT ops, {streams} streams, {cyc} cycle(s) per step",
                   "lut_ops": info["lut_ops"]},
        "lut_evals_per_s": v * info["lut_ops"],
        "cpu_baseline": {"value": v, "unit": "stimulus-cycles/s", "cores": threads, "kind": "port",
                         "sample": f"{streams} streams x {cyc} cycle(s) per step, {a.steps} steps (a run of "
                                   f"1 + {cyc} cycles less a run of 1 cycle: set-up and final digests excluded)"},
        "e2e": {"value": v, "unit": "stimulus-cycles/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_reference_gpu(a, rank, ws):
    """The reference's own GPU kernel (src/SimEval.cu built unmodified into
    oracle/_ref/ref_simeval.cubin, driven by oracle/refgpu_harness.cpp) on the
    same design: one stream (the reference cannot batch), free running
    (eval_free_running) and one cooperative launch per cycle with host-side
    stimulus (eval() + setRegister)."""
    if rank != 0:
        return
    from oracle import pyoracle
    from toucangpurt_gb300 import build

    build.build()
    pyoracle.build()
    exe, cubin = pyoracle.HERE / "_build" / "refgpu", pyoracle.REF_CUBIN
    if not exe.exists() or not cubin.exists():
        print(json.dumps({"impl": "reference-gpu", "unavailable": "reference cubin not built (needs the reference checkout)"}))
        return
    wd = Path(tempfile.mkdtemp(prefix="tgs_refgpu_"))
    dp, sp, info = make_design(a.workload, wd, 0, a.override)
    stim = wd / "stim.txt"
    stim.write_text(f"1234 {len(info['pi_ids'])}\n" + "".join(f"{int(r)} {int(b)} 0\n" for r, b in zip(info["pi_ids"], info["pi_bits"])))
    res = {}
    for mode, cycles in (("free", a.cycles_per_step or 20), ("eval", max(1, (a.cycles_per_step or 20) // 4))):
        out = wd / f"{mode}.jsonl"
        subprocess.run([str(exe), str(cubin), str(dp), str(sp), "0", mode, str(cycles), "1",
                        str(stim) if mode == "eval" else "-", str(out)], check=True, timeout=1800)
        r = json.loads(out.read_text().splitlines()[0])
        res[mode] = {"cycles": cycles, "kernel_ms": r["kernel_ms"], "stimulus_cycles_per_s": cycles / (r["kernel_ms"] / 1e3),
                     "large_kernel": r["large_kernel"], "grid": r["grid_multi"] if mode == "free" else r["grid_single"],
                     "threads": r["threads"]}
    line = {"impl": "reference-gpu", "metric": METRIC, "unit": "stimulus-cycles/s",
            "value": res["free"]["stimulus_cycles_per_s"], "lut_evals_per_s": res["free"]["stimulus_cycles_per_s"] * info["lut_ops"],
            "config": {"workload": f"{a.workload}: {info['lut_ops']} LUT ops, 1 stream"}, "modes": res}
    print(json.dumps(line), flush=True)


def levels_option(a) -> int:
    """tgs_options.resident_netlist for --levels / --no-stage."""
    return 2 if a.no_stage else {"auto": 0, "resident": 1, "global": 2, "staged": 3}[a.levels]


def exec_levels(st) -> str:
    return "resident" if st.get("resident_words") else "staged" if st.get("stage_words") else "global"


def make_simulator(a, dp, sp, streams, gpu):
    """The simulator configured as the benchmark runs the workload
    (workloads.bench_simulator: mode choice, learned schedule trained before
    the timed region), then autotuned when asked.  Returns (sim, notes)."""
    from toucangpurt_gb300 import workloads

    s, notes = workloads.bench_simulator(a.workload, dp, sp, streams=streams, gpu=gpu, schedule=a.schedule,
                                         mode=a.mode, groups=a.groups, warps=a.warps, levels=levels_option(a),
                                         value_pool=0 if a.value_pool == "compact" else 1,
                                         **{k: int(v) for k, v in (kv.split("=", 1) for kv in a.set)})
    if a.set:
        notes["options"] = list(a.set)
    if a.autotune:
        best, trials = s.autotune(cycles=8, warmup=2)
        notes["autotuned"] = {k: best[k] for k in ("groups_per_item", "warps_per_block", "blocks_per_sm", "mode", "staged",
                                                   "mpart_lanes", "levels_per_barrier")}
        notes["autotune_trials"] = len(trials)
    return s, notes


def run_gb300_queued(a, rank, ws, dp, sp, info, streams, schedule, gpu):
    """Streams of log-uniform length queued, longest first, onto resident
    slots (retired and admitted in place inside one launch or one sequence of
    graph replays).  One step = the whole job."""
    from toucangpurt_gb300 import sim, workloads

    s, notes = make_simulator(a, dp, sp, a.slots or 8, gpu)
    cyc = workloads.stream_lengths(a.workload, streams, seed=7 + rank)
    stim = sim.StimulusSpec(1000 + rank, info["pi_ids"], info["pi_bits"], workloads.toggles(a.workload, info["pi_bits"]))
    for _ in range(a.warmup):
        s.batch_run(cyc, stim, rolling=False, slots=a.slots)
    barrier(ws)
    clk = Clocks(gpu)
    dev_ms, t0 = 0.0, time.perf_counter()
    launches = 0
    for _ in range(a.steps):
        out = s.batch_run(cyc, stim, rolling=False, slots=a.slots)
        dev_ms += out.device_ms
        launches += out.launches
    wall = time.perf_counter() - t0
    clocks = clk.stop()
    st = s.design_stats()
    total = allreduce_sum(float(cyc.sum()) * a.steps, ws)
    dev_s = allreduce_max(dev_ms / 1000.0, ws)
    wall_s = allreduce_max(wall, ws)
    if rank == 0:
        line = {
            "metric": METRIC, "value": total / dev_s, "unit": "stimulus-cycles/s", "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1000 * dev_s / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8 nibbles (8 streams per u32)", "data": "synthetic (seeded generator)",
            "config": {"workload": f"{a.workload}: {st['lut_ops']} LUT ops, {streams} streams of log-uniform length "
                                   f"(mean {cyc.mean():.0f}), {s.options()['n_streams']} slots, longest first",
                       "stream_cycles": int(cyc.sum()), "schedule": a.schedule, "exec_levels": exec_levels(st),
                       "mode": ["persistent", "graph"][s.options()["mode"]],
                       "blocks": st["blocks"],
                       "threads_per_block": st["threads"],
                       "groups_per_item": st["groups_per_item"], **notes},
            "lut_evals_per_s": total / dev_s * st["lut_ops"],
            "e2e": {"value": total / wall_s, "unit": "stimulus-cycles/s", "h2d_bytes_per_step": int(cyc.nbytes),
                    "d2h_bytes_per_step": int(streams * 8 * 3),
                    "path": "tgs_batch_run per step: stream lengths uploaded, each queued stream's inputs derived "
                            "from its seed on the device (a host table of every stream's inputs would be "
                            f"{int(cyc.sum()) * len(info['pi_ids']) / 1e9:.1f} GB per step), final register, "
                            "memory and rolling digests read back"},
            "gpu_launches": launches, "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    s.cleanup()


def run_e2e(a, s, info, stim, streams, cps):
    """End-to-end steps through the public API: every step uploads that
    step's input table from pinned host memory (tgs_stimulus.table), runs the
    design on from the previous step's state (TGS_BATCH_CONTINUE) and reads
    the per-stream rolling digests and stop cycles back.  The tables hold the
    same values the device derives from the seed (toggles included); they are
    written before the timed region.  Returns (seconds, h2d bytes per step,
    d2h bytes per step)."""
    from toucangpurt_gb300 import sim

    n_in = len(info["pi_ids"])
    steps = a.steps + 1  # one untimed step from the initial state
    bufs = [sim.PinnedBuffer((cps, n_in, streams)) for _ in range(steps)]
    prev = np.repeat(s.reg_pool(0)[info["pi_ids"]][:, None], streams, axis=1)
    for k in range(steps):
        sim.stimulus_table(stim, streams, k * cps, cps, out=bufs[k].array, prev=prev)
        prev = bufs[k].array[-1].copy()
    cyc = np.full(streams, cps, np.uint32)

    def step(k):
        t = sim.StimulusSpec(stim.base_seed, info["pi_ids"], info["pi_bits"], table=bufs[k].array)
        return s.batch_run(cyc, t, continue_=k > 0, final_digests=False)

    step(0)
    t0 = time.perf_counter()
    for k in range(1, steps):
        out = step(k)
    dt = time.perf_counter() - t0
    _ = out.rolling_digest.sum()
    for b in bufs:
        b.free()
    return dt, int(cps * n_in * streams), int(streams * (8 + 4))


def parity_check(od, s, stim, timed, streams, cps, cycles, threads):
    """The oracle against this library on the benchmark's own inputs: the
    per-cycle register digests of every stream over the first `cycles`
    cycles of the run's first step, and the final register, memory and rolling
    digests of a separate `cycles`-cycle run (memories included)."""
    c = max(1, min(cycles, cps))
    ref = od.run(np.full(streams, c, np.uint32), stim, threads=threads, cycle_digests=True)
    short = s.batch_run(np.full(streams, c, np.uint32), stim)
    bad = []
    if not np.array_equal(timed.cycle_digest[:, :c], ref["cycle_digest"]):
        bad.append("per-cycle register digests")
    for k in ("final_reg_digest", "final_mem_digest", "rolling_digest", "stop_cycle"):
        if not np.array_equal(getattr(short, k), ref[k]):
            bad.append(k)
    return {"result": "bit-exact" if not bad else "MISMATCH: " + ", ".join(bad), "against": "CPU oracle",
            "checked": f"{streams} streams x {c} cycles: per-cycle register digests of the run's first step; final register, "
                       f"memory and rolling digests and stop cycles of a {c}-cycle run"}


def plain_form(a, dp, sp, info, gpu, cps, stim):
    """The plain form on the same design: one stream, gate-count schedule,
    the same cycles per step; device time per step (CUDA events)."""
    from toucangpurt_gb300 import workloads

    s, _ = workloads.bench_simulator(a.workload, dp, sp, streams=1, gpu=gpu, schedule="greedy", mode=a.mode,
                                     **{k: int(v) for k, v in (kv.split("=", 1) for kv in a.set)})
    cyc = np.full(1, cps, np.uint32)
    for _ in range(a.warmup):
        s.batch_run(cyc, stim)
    ms = sum(s.batch_run(cyc, stim).device_ms for _ in range(a.steps))
    opts = s.options()
    s.cleanup()
    return {"value": cps * a.steps / (ms / 1000.0), "unit": "stimulus-cycles/s", "streams": 1, "schedule": "greedy",
            "mode": ["persistent", "graph"][opts["mode"]]}


def reference_kernel(dp, sp, info, stim, timed, cycles):
    """The reference's own GPU kernel on the same design: its race-free
    eval() path (evalSingleCycle, one cooperative launch per cycle with the
    inputs written between cycles, src/ToucanSim.cu:206-230), one stream,
    kernel time from CUDA events; its per-cycle register digests are
    compared with stream 0 of a timed step of this library."""
    from oracle import pyoracle

    exe, cubin = pyoracle.HERE / "_build" / "refgpu", pyoracle.REF_CUBIN
    if not exe.exists() or not cubin.exists():
        return {"unavailable": "reference cubin not built here (built from the reference checkout by oracle/Makefile)"}
    wd = Path(tempfile.mkdtemp(prefix="tgs_refk_"))
    tog = stim.toggle if stim.toggle is not None else np.zeros(len(stim.reg), np.uint16)
    (wd / "stim.txt").write_text(f"{stim.base_seed} {len(stim.reg)}\n" + "".join(
        f"{int(r)} {int(b)} {int(g)}\n" for r, b, g in zip(stim.reg, stim.bits, tog)))
    out = wd / "eval.jsonl"
    t0 = time.perf_counter()
    subprocess.run([str(exe), str(cubin), str(dp), str(sp), "0", "eval", str(cycles), "1", str(wd / "stim.txt"),
                    str(out)], check=True, timeout=1800, stdout=subprocess.DEVNULL)
    r = json.loads(out.read_text().splitlines()[0])
    digs = np.array([int(x, 16) for x in r["cycle_digests"]], np.uint64)
    same = bool(np.array_equal(digs, timed.cycle_digest[0, :cycles]))
    return {"value": cycles / (r["kernel_ms"] / 1e3), "unit": "stimulus-cycles/s", "path": "eval() (evalSingleCycle)",
            "streams": 1, "cycles": cycles, "threads": r["threads"], "grid": r["grid_single"],
            "parity": "bit-exact (stream 0, per-cycle register digests)" if same else "MISMATCH",
            "wall_s": round(time.perf_counter() - t0, 1)}


def run_gb300(a, rank, ws):
    from toucangpurt_gb300 import build, sim, workloads

    build.build()
    gpu = local_gpu(ws)
    wd = Path(tempfile.mkdtemp(prefix="tgs_bench_"))
    dp, sp, info = make_design(a.workload, wd, rank, a.override)
    streams = a.streams or workloads.RUNS[a.workload]["streams"]
    if a.schedule == "auto":
        a.schedule = "learned" if streams > 1 else "greedy"
    cps = a.cycles_per_step or (200 if a.workload in ("largest", "learned") else 2000)
    schedule = 1 if a.schedule == "learned" else 0
    if isinstance(workloads.RUNS[a.workload]["cycles"], tuple):
        return run_gb300_queued(a, rank, ws, dp, sp, info, streams, schedule, gpu)
    s, notes = make_simulator(a, dp, sp, streams, gpu)
    st = s.design_stats()
    toggle = workloads.toggles(a.workload, info["pi_bits"])
    stim = sim.StimulusSpec(1000 + rank, info["pi_ids"], info["pi_bits"], toggle)
    cyc = np.full(streams, cps, np.uint32)
    # step 0 starts from the initial state (the oracle checks it); every later
    # step, warm-up and timed, continues the run from the previous one, so the
    # timed steps cover cycles W*cps .. (W+K)*cps of one long run
    first = s.batch_run(cyc, stim, cycle_digests=True)
    for _ in range(a.warmup - 1):
        s.batch_run(cyc, stim, cycle_digests=True, continue_=True)
    barrier(ws)
    clk = Clocks(gpu)
    dev_ms = 0.0
    launches = 0
    for _ in range(a.steps):
        out = s.batch_run(cyc, stim, cycle_digests=True, continue_=True)
        dev_ms += out.device_ms
        launches += out.launches
    clocks = clk.stop()
    barrier(ws)
    # the continued steps against one uninterrupted run of the same length
    before = max(1, a.warmup)  # steps run before the timed ones
    whole = s.batch_run(np.full(streams, cps * (before + a.steps), np.uint32), stim, cycle_digests=True)
    continued = bool(np.array_equal(whole.cycle_digest[:, -cps:], out.cycle_digest))
    del whole
    e2e_s, h2d, d2h = run_e2e(a, s, info, stim, streams, cps)
    barrier(ws)
    dev_s = allreduce_max(dev_ms / 1000.0, ws)
    wall_s = allreduce_max(e2e_s, ws)
    total_sc = allreduce_sum(float(streams * cps * a.steps), ws)
    value = total_sc / dev_s
    e2e = total_sc / wall_s
    peak, peak_kind = measured_peak()
    # the dominant kernel: one regionKernel launch per region and cycle (graph
    # form) or one cycleKernel launch per step (persistent form); the device
    # time of a step is those launches (advance and stimulus launches are
    # ~0.01 % of it, profiles/)
    graph = s.options()["mode"] == 1
    launches_step = 2 * cps if graph else 1
    bytes_launch = algorithmic_bytes(st, streams, cps) / launches_step
    launch_s = dev_ms / 1000.0 / a.steps / launches_step
    achieved = bytes_launch / launch_s / 1e9
    prof = a.workload == "largest" and streams == 64
    traffic = int(profiled("traffic_bytes_per_launch")) if prof and profiled("traffic_bytes_per_launch") else None
    cpu = parity = plain = refk = None
    if rank == 0 and ws == 1 and not a.no_cpu_baseline:
        from oracle import pyoracle

        nth = cpu_threads(info, streams)
        od = pyoracle.OracleDesign(dp, sp)
        cdt, ccyc = cpu_sample(od, stim, streams, a.cpu_sample_cycles, nth)
        cpu = {"value": streams * ccyc / cdt, "unit": "stimulus-cycles/s", "cores": nth, "kind": "port",
               "sample": f"{streams} streams x {ccyc} cycle(s) of the same design, {cdt:.1f} s "
                         f"(a run of 1 + {ccyc} cycles less a run of 1 cycle)"}
        parity = parity_check(od, s, stim, first, streams, cps, a.cpu_sample_cycles, nth)
        parity["continued_steps"] = ("equal to one uninterrupted run" if continued else "MISMATCH against one "
                                     "uninterrupted run") + f" (per-cycle register digests, cycles " \
                                    f"{before * cps}..{(before + a.steps) * cps - 1})"
        del od
    sched_gain = None
    if rank == 0 and ws == 1 and not a.no_baselines and a.schedule == "learned":
        # the same steps with the gate-count schedule (the learned model's fallback)
        s.set_options(schedule=0)
        s.batch_run(cyc, stim)
        for _ in range(a.warmup - 1):
            s.batch_run(cyc, stim, continue_=True)
        greedy_ms = sum(s.batch_run(cyc, stim, continue_=True).device_ms for _ in range(a.steps))
        s.set_options(schedule=1)
        sched_gain = {"greedy_value": streams * cps * a.steps / (greedy_ms / 1000.0), "unit": "stimulus-cycles/s",
                      "learned_over_greedy": greedy_ms / dev_ms,
                      "train_s": notes.get("cost_model", {}).get("train_s"),
                      "samples": notes.get("cost_model", {}).get("samples")}
    if rank == 0 and ws == 1 and not a.no_baselines:
        if streams > 1:
            plain = plain_form(a, dp, sp, info, gpu, cps, stim)
            plain["batched_over_plain"] = value / plain["value"]
        refk = reference_kernel(dp, sp, info, stim, first, min(cps, a.ref_cycles))
        if "value" in refk:
            refk["batched_over_reference_kernel"] = value / refk["value"]
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "stimulus-cycles/s", "n_gpus": ws, "steps": a.steps,
            "warmup": a.warmup, "ms_per_step": 1000 * dev_s / a.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8 nibbles (8 streams per u32)", "data": "synthetic (seeded generator)",
            "config": {"workload": f"{a.workload}: {st['lut_ops']} LUT ops, {streams} streams, {cps} cycles per step",
                       "streams": streams, "cycles_per_step": cps, "lut_ops": st["lut_ops"],
                       "partitions": st["partitions"], "groups_per_item": st["groups_per_item"],
                       "mode": ["persistent", "graph"][s.options()["mode"]], "value_pool": a.value_pool,
                       "smem_per_block": st.get("smem_per_block"), "exec_levels": exec_levels(st), **notes,
                       "threads_per_block": st["threads"], "blocks": st["blocks"],
                       "l2": "working set (memories) larger than L2"},
            "lut_evals_per_s": value * st["lut_ops"],
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_source": peak_kind,
                         "kernel": f"{'regionKernel' if graph else 'cycleKernel'}<{st['streams_per_word']},"
                                   f"{st['groups_per_item']}>",
                         "algorithmic_bytes_per_launch": bytes_launch, "launch_us": launch_s * 1e6,
                         "note": "bound on chip by instruction issue and shared-memory table lookups (profiles/): HBM "
                                 "is not the limit",
                         "smem": {"wavefronts_per_sm_cycle": profiled("smem_wavefronts_per_sm_cycle") if prof else None,
                                  "useful_wavefronts_per_sm_cycle":
                                      profiled("smem_useful_wavefronts_per_sm_cycle") if prof else None,
                                  "peak": 1.0, "source": "ncu capture of the same kernel (profiles/)"}},
            "e2e": {"value": e2e, "unit": "stimulus-cycles/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h,
                    "path": "tgs_batch_run per step: host stimulus table (pinned) uploaded, continued run, "
                            "rolling digests and stop cycles read back"},
            "gpu_launches": launches,
            "clocks": clocks,
        }
        if parity:
            line["parity"] = parity
        if sched_gain:
            line["learned_schedule"] = sched_gain
        if plain:
            line["plain"] = plain
        if refk:
            line["reference_kernel"] = refk
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)
        if a.out:
            Path(a.out).write_text(json.dumps(line) + "\n")
    s.cleanup()


def main():
    a = args_parse()
    rank, ws = dist_init()
    if a.impl == "reference":
        run_reference(a, rank, ws)
    elif a.impl == "reference-gpu":
        run_reference_gpu(a, rank, ws)
    else:
        run_gb300(a, rank, ws)


if __name__ == "__main__":
    main()
