"""The N > 1 host path of bench.py on CPU with gloo, world size 2 (the
simulation itself does not shard: N GPUs run independent replicas, so the
only cross-rank steps are the barrier around the timed region and the
max-over-ranks time)."""
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _worker(rank, world, port, out):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(ROOT))
    import bench
    bench.barrier(world)
    t = bench.max_over_ranks(torch, 1.0 + rank, world, torch.device("cpu"))
    out.put((rank, t, bench.job_value(world, 1000, t)))
    bench.barrier(world)
    dist.destroy_process_group()


def test_max_over_ranks_and_job_value():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29000 + os.getpid() % 2000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.0, 2.0]           # the slowest rank's time on every rank
    assert [r[2] for r in res] == [1000.0, 1000.0]     # 2 replicas x 1000 units / 2.0 s


def test_reference_arm_under_torchrun():
    """bench.py --impl reference launched as 2 ranks: rank 0 prints one JSON
    line, the other rank exits 0 without output."""
    pytest.importorskip("torch")
    port = 31000 + os.getpid() % 2000
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), str(ROOT / "bench.py"), "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0", "--workload", "sphere32", "--cpu-particles", "2000",
           "--cpu-timesteps", "1"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    import json
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0 and d["cpu_baseline"]["kind"] == "port"
    cb = d["cpu_baseline"]
    assert cb["cores"] >= 1 and cb["cpu"] and cb["forward_s"] > 0 and cb["backward_s"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["value"] == d["value"]
    st = cb["single_thread"]
    assert st["cores"] == 1 and st["value"] > 0
    # the reference arm runs the CPU restatement only: none of this
    # repository's engine or kernels is mapped into its process
    assert d["native_libs"] == ["oracle/liboracle.so"], d["native_libs"]
