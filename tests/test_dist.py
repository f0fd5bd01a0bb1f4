"""Multi-GPU form is replicas only: each rank simulates its own streams, no
data-path collective; the bench takes the max time and the summed units over
ranks.  Covered here with world_size 2 on gloo (CPU), ranks running the
oracle on disjoint stream seeds."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, design, symbols, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws))
    import sys
    from pathlib import Path

    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import bench
    from oracle import pyoracle
    from toucangpurt_gb300 import sim

    r, w = bench.dist_init()
    assert (r, w) == (rank, ws)
    info = sim.generate(design + f".{rank}", symbols + f".{rank}", **__import__("toucangpurt_gb300.workloads", fromlist=["x"]).design_config("small"))
    od = pyoracle.OracleDesign(design + f".{rank}", symbols + f".{rank}")
    stim = sim.StimulusSpec(1000 + rank, info["pi_ids"], info["pi_bits"])
    out = od.run(np.full(4, 20, np.uint32), stim, threads=1)
    units = bench.allreduce_sum(4 * 20.0, ws)
    tmax = bench.allreduce_max(float(rank + 1), ws)
    bench.barrier(ws)
    q.put((rank, units, tmax, int(out["final_reg_digest"][0])))
    import torch.distributed as dist

    dist.destroy_process_group()


def test_two_rank_replicas(tmp_path, built):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, str(tmp_path / "d.bin"), str(tmp_path / "s.bin"), q))
             for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    assert [r[1] for r in res] == [160.0, 160.0]   # units summed over ranks
    assert [r[2] for r in res] == [2.0, 2.0]       # max over ranks
    assert res[0][3] != res[1][3]                  # ranks ran distinct stimulus


@pytest.mark.gpu
def test_bench_two_replicas(tmp_path):
    """bench.py under torchrun with two ranks: each rank runs its own replica
    of the 4K-LUT design (here both on the one GPU; ranks never wait on each
    other's kernels, only on gloo barriers between steps), and rank 0 prints
    one line whose value is the units of both ranks over the slower rank's
    time."""
    import json
    import subprocess
    import sys
    from pathlib import Path

    pytest.importorskip("torch")
    root = Path(__file__).resolve().parents[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), str(root / "bench.py"), "--gpus", "2", "--workload", "small",
           "--steps", "3", "--warmup", "3", "--no-cpu-baseline", "--no-baselines"]
    r = subprocess.run(cmd, cwd=root, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-4000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = lines[0]
    assert line["n_gpus"] == 2 and line["scaling"] == "weak" and line["value"] > 0
    assert line["config"]["streams"] == 1
    # two replicas' units over the slower rank's device time
    assert abs(line["value"] - 2 * 2000 * 3 / (line["ms_per_step"] * 3 / 1000)) / line["value"] < 1e-6
