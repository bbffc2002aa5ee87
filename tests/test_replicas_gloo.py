"""Multi-process (world size 2) path of bench.py on CPU with the gloo backend:
every rank times its own replica; the job reports total work over the slowest
rank's time (one GPU per process, no data-path collective)."""
import os
import socket
import sys
from pathlib import Path

import pytest
import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_time = [0.5, 0.8][rank]  # rank 1 is the slowest replica
    t = bench.reduce_max(local_time, world)
    v = bench.replica_throughput(2.0e12, t, world)
    out.put((rank, t, v))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_report_total_work_over_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(2))
    for rank, t, v in got:
        assert t == pytest.approx(0.8)
        assert v == pytest.approx(2 * 2.0e12 / 0.8 / 1e12)


def test_single_rank_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.reduce_max(1.25, 1) == 1.25
    assert bench.replica_throughput(1e12, 0.5, 1) == pytest.approx(2.0)
