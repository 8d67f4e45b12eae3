"""Multi-rank host logic on CPU with gloo (world size 2): disjoint frame
numbers per rank and the max-time / sum-rays reduction bench.py reports."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from mambatracer_gb300.dist import frame_number, reduce_max_sum  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    frames = [frame_number(s, rank, world) for s in range(5)]
    sec, rays = reduce_max_sum(1.0 + rank, 100 * (rank + 1))
    dist.barrier()
    q.put((rank, frames, sec, rays))
    dist.destroy_process_group()


def test_two_ranks_gloo():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(world)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    all_frames = sorted(f for _, fr, _, _ in res for f in fr)
    assert all_frames == [float(i) for i in range(1, 11)]  # disjoint, covering 1..N*K
    for _, _, sec, rays in res:
        assert sec == 2.0 and rays == 300


def test_single_process_identity():
    assert reduce_max_sum(3.5, 7) == (3.5, 7)
    assert frame_number(0, 0, 1) == 1.0 and frame_number(4, 0, 1) == 5.0
