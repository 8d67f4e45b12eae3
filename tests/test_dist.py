"""Multi-rank host logic on CPU with gloo (world size 2): disjoint frame
numbers per rank, the max-time / sum-rays reduction bench.py reports, the split
job's film (each rank renders its own frame numbers of one job; their films
summed are the one-rank progressive film over the same frames), and the served
requests' assignment to replicas."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from mambatracer_gb300.dist import assign_requests, frame_number, reduce_max_sum  # noqa: E402


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


W, H, DEPTH, STEPS = 24, 16, 4, 3


def _frame(orc, sc, nodes, bounds, fc):
    """One benchmark-semantics frame of the box room by the CPU oracle (the split
    job's contract holds for any renderer keyed on the frame number)."""
    import numpy as np

    from oracle.oracle import ptr
    acc = np.zeros((W * H, 4), np.float32)
    c = np.zeros(DEPTH, np.int32)
    z = np.zeros(4, np.float32)
    orc.lib.or_render_frame(ptr(sc.camera), W, H, DEPTH, 1, 0, None, float(fc), ptr(sc.points), ptr(sc.uvs),
                            ptr(sc.normals), ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds),
                            ptr(z), ptr(z), ptr(z), 1, 1, 0, 0, ptr(acc), ptr(c), None)
    return acc


def _film_worker(rank, world, port, q):
    import numpy as np

    from mambatracer_gb300 import scenes
    from oracle.oracle import Oracle, bvh_build
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    orc = Oracle()
    sc = scenes.box_room(W, H)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    frames = {}
    total = np.zeros((W * H, 4), np.float64)
    for step in range(STEPS):
        fc = frame_number(step, rank, world)
        frames[fc] = _frame(orc, sc, nodes, bounds, fc)
        total += frames[fc]
    t = torch.from_numpy(total)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    gathered = [None] * world
    dist.all_gather_object(gathered, frames)
    if rank == 0:
        q.put((t.numpy(), gathered))
    dist.barrier()
    dist.destroy_process_group()


def test_split_job_films_sum_to_the_one_rank_film():
    import numpy as np

    from mambatracer_gb300 import scenes
    from oracle.oracle import Oracle, bvh_build
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_film_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    total, gathered = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # one rank, the same frame numbers 1 .. world * STEPS
    orc = Oracle()
    sc = scenes.box_room(W, H)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    one = {float(fc): _frame(orc, sc, nodes, bounds, fc) for fc in range(1, world * STEPS + 1)}
    split = {fc: f for d in gathered for fc, f in d.items()}
    assert sorted(split) == sorted(one)
    for fc in one:  # every frame bit for bit
        assert split[fc].tobytes() == one[fc].tobytes()
    ref = sum(one[fc].astype(np.float64) for fc in sorted(one))
    assert ref[:, :3].sum() > 0
    np.testing.assert_allclose(total, ref, rtol=1e-12, atol=0)  # the sum, up to its order


def test_requests_go_to_the_least_loaded_replica():
    costs = [100, 50, 50, 10, 200, 5]
    r = assign_requests(costs, 2)
    assert r == [0, 1, 1, 0, 1, 0]
    loads = [sum(c for c, k in zip(costs, r) if k == w) for w in range(2)]
    assert abs(loads[0] - loads[1]) <= max(costs)
    assert assign_requests(costs, 1) == [0] * len(costs)
