"""bench.py's multi-GPU form is N independent replicas (the exact MIC(0)
preconditioner does not partition across GPUs, so there is no data-path
collective); the only cross-rank step is the max of the ranks' times.  Checked
with two gloo ranks on the CPU."""
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
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    local = 2.0 if rank == 0 else 3.5
    q.put((rank, bench.reduce_max(local, world, "cpu"), bench.job_rate(10, local, world, "cpu")))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, tmax, rate in out:
        assert tmax == 3.5
        assert abs(rate - 2 * 10 / 3.5) < 1e-12
