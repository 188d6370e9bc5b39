"""The bench's multi-GPU path is replicas only: each rank runs its own chains
and the whole-job rate is the units all ranks processed over the slowest
rank's time. Checked on CPU with two gloo ranks."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    # rank r took (r + 1) * 100 ms for 640 proposals
    rate, ms = bench.job_rate(640, 100.0 * (rank + 1), ws, None)
    q.put((rank, rate, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rate_uses_slowest_rank():
    ws = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(ws)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, ms in res:
        assert ms == pytest.approx(200.0)
        assert rate == pytest.approx(640 * 2 / 0.2)


def test_single_rank_rate():
    import bench
    rate, ms = bench.job_rate(640, 100.0, 1)
    assert ms == 100.0 and rate == pytest.approx(6400.0)
