"""bench.py's N-GPU mode runs independent replicas (one per rank) and reports
all ranks' work over the slowest rank's time.  Checked with two gloo ranks on
the CPU (no GPU, no NCCL)."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, w, local = bench.dist_env()
    ms = 10.0 * (rank + 1)                         # rank 1 is the slow one
    q.put((r, w, local, bench.barrier_max(ms, w), bench.replica_value(1000.0, ms, w)))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_report_max_over_ranks():
    ctx = torch.multiprocessing.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r, (rank, world, local, mx, value) in enumerate(res):
        assert (rank, world, local) == (r, 2, r)
        assert mx == 20.0
        assert value == pytest.approx(2 * 1000.0 / 0.020)
