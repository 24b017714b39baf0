"""The multi-GPU launch of bench.py on the host: two ranks over gloo (torchrun's environment,
127.0.0.1) agree on the maximum of their times and pass the barrier; one rank runs alone without
a process group."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench

    r = bench.Ranks("gloo")
    r.barrier()
    out.put((rank, r.world, r.max(1.5 + rank)))
    r.barrier()
    r.dist.destroy_process_group()


def test_two_ranks_take_the_maximum_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert got == [(0, 2, 2.5), (1, 2, 2.5)]


def test_single_rank_has_no_process_group(monkeypatch):
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    import bench

    r = bench.Ranks()
    assert r.world == 1 and r.dist is None
    r.barrier()
    assert r.max(3.25) == 3.25
