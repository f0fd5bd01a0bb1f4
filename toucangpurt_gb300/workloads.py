"""Seeded synthetic workloads standing in for the five benchmark
configurations of the Toucan hot path (the reference ships no design files).

Mapping of a configuration onto the reference's nibble value model: one
configuration LUT is one table-lookup op (lutIndex != 0); a 4-input LUT is a
2-operand op (op0 = 0, a 256-entry table window), a 6-input LUT a 3-operand
op (4,096-entry window); flip-flop and primary-input bits are packed four per
register nibble; a w-bit memory is ceil(w / 4) nibble memories sharing the
address.  Stimulus streams follow tgs_stimulus (seeded splitmix64 bits).
"""
from __future__ import annotations

import numpy as np

DESIGN_SEEDS = {"small": 101, "scale": 202, "batch": 101, "learned": 404, "largest": 505}

# generator fields per workload
DESIGNS = {
    # 4,096 4-input LUTs in 16 levels, 512 FFs, 32 PIs, one 1,024 x 32 memory 1R/1W
    "small": dict(n_lut=4096, levels=16, operands=2, ff_bits=512, pi_bits=32, n_mems=1, mem_depth=1024,
                  mem_width=32, mem_read_ports=1, mem_write_ports=1, luts_per_part=2048, mpart_width=32, cone_depth=1),
    # 1M 6-input LUTs, 48 levels, 40% AND/OR/XOR/MUX, power-law fan-out 2.2 (max 4,096), 64K FFs,
    # 512 32-bit vector ops, 16 memories 64K x 32 with 2R/1W, 256 PIs
    "scale": dict(n_lut=1 << 20, levels=48, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=4096,
                  ff_bits=64 * 1024, pi_bits=256, n_vec_ops=512, vec_nibbles=8, n_mems=16, mem_depth=64 * 1024,
                  mem_width=32, mem_read_ports=2, mem_write_ports=1, luts_per_part=4096, mpart_width=32, cone_depth=1),
    # the small design, run with many streams
    "batch": dict(n_lut=4096, levels=16, operands=2, ff_bits=512, pi_bits=32, reset_inputs=1, n_mems=1,
                  mem_depth=1024, mem_width=32, mem_read_ports=1, mem_write_ports=1, luts_per_part=2048,
                  mpart_width=32, cone_depth=1),
    # 4M LUTs of mixed regions (datapath / deep control / memory / high fan-out), 512K FFs,
    # 1,024 memories 4K x 64 with 1-4 ports
    "learned": dict(n_lut=4 << 20, levels=128, operands=3, palette_pct=40, fanout_alpha=2.2, max_fanout=65536,
                    ff_bits=512 * 1024, pi_bits=256, n_mems=1024, mem_depth=4096, mem_width=64, mem_read_ports=2,
                    mem_write_ports=1, luts_per_part=8192, mpart_width=32, cone_depth=1, mixed=1),
    # 16M 6-input LUTs, 96 levels, power-law 2.0, 2M FFs, 8K 64-bit vector ops,
    # 256 memories 256K x 32 with 2R/2W (multi-writer), 1,024 PIs
    "largest": dict(n_lut=16 << 20, levels=96, operands=3, palette_pct=40, fanout_alpha=2.0, max_fanout=4096,
                    ff_bits=2 << 20, pi_bits=1024, n_vec_ops=8192, vec_nibbles=16, n_mems=256,
                    mem_depth=256 * 1024, mem_width=32, mem_read_ports=2, mem_write_ports=2, mem_multi_writer=1,
                    luts_per_part=8192, mpart_width=32, cone_depth=1),
}

# stream counts and cycles per workload
RUNS = {
    "small": dict(streams=1, cycles=1000, toggle=0.0),
    "scale": dict(streams=1, cycles=100_000, toggle=0.0),
    "batch": dict(streams=4096, cycles=(1000, 100_000), toggle=0.05),  # log-uniform lengths, reset toggles 5%
    "learned": dict(streams=256, cycles=20_000, toggle=0.0),
    "largest": dict(streams=64, cycles=10_000, toggle=0.10),
}


def design_config(name: str, **override) -> dict:
    cfg = dict(DESIGNS[name])
    cfg["seed"] = DESIGN_SEEDS[name]
    cfg.update(override)
    return cfg


def stream_lengths(name: str, n: int | None = None, seed: int = 7) -> np.ndarray:
    r = RUNS[name]
    n = n or r["streams"]
    c = r["cycles"]
    if isinstance(c, tuple):
        rng = np.random.default_rng(seed)
        lo, hi = np.log(c[0]), np.log(c[1])
        return np.exp(rng.uniform(lo, hi, n)).astype(np.uint32)
    return np.full(n, c, np.uint32)


def toggles(name: str, bits: np.ndarray) -> np.ndarray | None:
    """Per-input toggle thresholds: 1-bit reset lines toggle with the
    workload's probability, the other inputs are fresh uniform bits; for the
    largest workload every input toggles at its rate."""
    p = RUNS[name]["toggle"]
    if p == 0:
        return None
    t = np.zeros(bits.size, np.uint16)
    if name == "largest":
        t[:] = int(round(p * 65536))
    else:
        t[bits == 1] = int(round(p * 65536))
    return t


def bench_simulator(name: str, design, symbols, *, streams: int | None = None, gpu: int = 0, schedule: str = "auto",
                    mode: str = "auto", groups: int = 0, warps: int = 0, levels: int = 0, value_pool: int = 0,
                    profile_cycles: int = 20, epochs: int = 40, seed: int = 5, samples: int = 200_000, **options):
    """A simulator loaded and configured the way the benchmark runs a
    workload: `streams` resident streams (default: the workload's count),
    the CUDA-graph form unless the exec levels stay resident in shared
    memory (then one persistent launch), and for more than one stream the
    learned schedule (every micro-partition profiled for `profile_cycles`
    cycles, repeated until about `samples` (features, clock64 cycles) samples
    are collected, the cost model trained on them).  Further tgs_options
    fields may be given by name.  Returns (simulator, notes) where notes
    holds the cost model's validation figures."""
    import time

    from . import capi, sim

    streams = streams or RUNS[name]["streams"]
    if schedule == "auto":
        schedule = "learned" if streams > 1 else "greedy"
    # the named arguments are defaults that an explicit tgs_options field overrides
    base = dict(n_streams=streams, groups_per_item=groups, warps_per_block=warps, resident_netlist=levels,
                mode=capi.MODE_PERSISTENT if mode == "persistent" else capi.MODE_GRAPH, value_pool=value_pool)
    s = sim.Simulator(**{**base, **options})
    s.init(gpu, design, symbols, False, False)
    notes = {"schedule": schedule}
    if mode == "auto" and s.design_stats().get("resident_words"):
        s.set_options(mode=capi.MODE_PERSISTENT)  # resident levels are loaded once per run
    if schedule == "learned":
        t0 = time.perf_counter()
        feats = s.mpart_features()
        passes = max(1, min(8, -(-samples // max(1, len(feats)))))
        X = np.concatenate([feats] * passes)
        y = np.concatenate([s.profile_mparts(profile_cycles) for _ in range(passes)])
        rep = s.train_cost_model(X, y, epochs=max(1, epochs // passes), seed=seed)
        s.set_options(schedule=capi.SCHED_LEARNED)
        notes["cost_model"] = {k: round(float(v), 4) for k, v in rep.items() if k in ("val_mse", "val_corr", "gate_corr")}
        notes["cost_model"]["train_s"] = round(time.perf_counter() - t0, 2)
        notes["cost_model"]["samples"] = int(len(y))
    return s, notes
