"""The bench's multi-process plumbing on the CPU (gloo, world size 2): the
barrier and the max over ranks that the timed region and every reported value
go through under torchrun (one GPU per rank; here no GPU is touched)."""
import multiprocessing as mp
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    d = bench.Dist()
    d.barrier()
    q.put((rank, d.max(10.0 + 3 * rank), d.world, d.rank))
    d.barrier()
    d.dist.destroy_process_group()


def test_max_over_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    got = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 13.0, 2, 0), (1, 13.0, 2, 1)]


def test_single_process_needs_no_process_group():
    import bench
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        os.environ.pop(k, None)
    d = bench.Dist()
    d.barrier()
    assert d.pg is None and d.max(2.5) == 2.5
