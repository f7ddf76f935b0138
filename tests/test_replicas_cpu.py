"""The multi-GPU path of bench.py is independent replicas (pixels, tiles and
scenes shard with no exchange step): whole-job throughput = all ranks' units
over the slowest rank's time.  Exercised with world_size 2 on the gloo backend
(CPU, no GPU needed)."""
import os
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parents[1]


def _rank(rank: int, ws: int, port: int, out):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    # rank 1 is the slow one: 2000 ms against 1000 ms on rank 0
    value, t_max = bench.replica_throughput(1000.0 * (rank + 1), 132.7e6, ws, device="cpu")
    out.put((rank, value, t_max))
    dist.destroy_process_group()


def test_replica_throughput_uses_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + (os.getpid() % 1000)
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, t_max in res:
        assert t_max == 2000.0
        assert abs(value - 2 * 132.7e6 / 2.0 / 1e6) < 1e-9


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    value, t_max = bench.replica_throughput(500.0, 1e6, 1)
    assert t_max == 500.0 and abs(value - 2.0) < 1e-12
