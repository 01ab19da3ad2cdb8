"""Multi-GPU form of the benchmark: independent replicas (no data-path
collective).  Two gloo ranks on the CPU exercise the barrier and the
max-over-ranks / sum-over-ranks reductions that bench.py uses."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    w, r, local, dist = bench.dist_setup()
    assert (w, r, local) == (world, rank, rank)
    bench.barrier(dist)
    ms = 1.0 + rank            # rank 1 is the slow one
    rays = 1000.0 * (rank + 1)
    q.put((rank, bench.reduce_max(dist, ms), bench.reduce_sum(dist, rays)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replica_reductions():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res == [(0, 2.0, 3000.0), (1, 2.0, 3000.0)]
    # whole-job throughput: rays of all ranks over the slowest rank's time
    assert 3000.0 / (2.0 * 1e3) == pytest.approx(1.5)


def test_count_rays_counts_primary_and_traced_shadow():
    import numpy as np
    import bench
    import oracle
    h = np.zeros(4, dtype=oracle.HIT_DTYPE)
    h["shadow_steps"] = [0, 3, 0, 1]
    assert bench.count_rays(h) == 6


def test_bench_gpus_2_launches_two_replicas():
    """bench.py --gpus 2, run directly, starts two replica processes itself;
    the reference arm (CPU) runs on rank 0 only and prints one line with
    n_gpus = 2, and both processes exit 0."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    assert lines[0]["impl"] == "reference" and lines[0]["n_gpus"] == 2 and lines[0]["value"] > 0


def test_bench_rejects_world_size_mismatch():
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, WORLD_SIZE="2", RANK="0", LOCAL_RANK="0")
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--gpus", "1"],
                       capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode != 0 and "WORLD_SIZE" in r.stderr
