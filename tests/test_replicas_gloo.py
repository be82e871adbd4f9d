"""CPU, world size 2 over gloo: the multi-GPU bench path runs independent
replicas (the step has no data exchange); the job throughput counts every
rank's points and is timed by the slowest rank."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local_ms = 100.0 if rank == 0 else 250.0
    value, ms = bench.replica_throughput(dist, world, 1000, 10, local_ms)
    q.put((rank, value, ms))
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, value, ms in res:
        assert ms == 250.0
        assert abs(value - 2 * 1000 * 10 / 0.25) < 1e-9
