"""Multi-GPU host logic on CPU: the path runs as independent replicas (one
simulation per GPU, no data-path collective); bench.py aggregates the units all
ranks processed over the slowest rank's time.  world_size 2 over gloo."""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    units, secs = 1000.0 * (rank + 1), 2.0 + rank
    t = torch.tensor([secs, float(units)], dtype=torch.float64)
    g = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(g, t)
    value, tmax = bench.aggregate_replicas([x[1].item() for x in g], [x[0].item() for x in g])
    q.put((rank, value, tmax))
    dist.destroy_process_group()


def test_replica_aggregation_over_gloo():
    import torch.multiprocessing as mp
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # units 1000 + 2000 over the slowest rank's 3 s, identical on both ranks
    for _, value, tmax in res:
        assert tmax == 3.0 and value == pytest.approx(1000.0)


def test_reference_arm_runs_on_rank0_only(tmp_path):
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1"], env=env, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0 and out.stdout.strip() == ""
