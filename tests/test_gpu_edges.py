"""Edge cases of the GPU frame and query paths against the oracle: frame sizes
that fill no tile or block evenly (37 x 29, 1 x 1), a frame whose camera rays
all miss (empty queues from the first bounce on), a one-triangle scene, and
queries over no rays."""
import numpy as np
import pytest

from mambatracer_gb300 import api, layout, scenes
from tests.helpers import bvh_build, oracle_frames, rel_rmse

pytestmark = pytest.mark.gpu


def _seeds(depth, seed):
    return np.random.default_rng(seed).integers(2 ** 29, 2 ** 30, size=2 * (1 + 2 * depth)).astype(np.int32)


@pytest.mark.parametrize("W,H", [(37, 29), (1, 1), (257, 3)])
def test_ragged_frame_sizes(ctx, orc, W, H):
    sc = scenes.box_room(W, H)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    depth = 5
    J = api.Job(ctx, S, W, H, max_depth=depth, mode=0, film_kahan=0)
    J.set_camera(sc.camera)
    seeds = _seeds(depth, W * 7 + H)
    J.render(seeds, 1.0)
    rays, counts = J.stats()
    acc, oc, orays = oracle_frames(orc, sc, nodes, bounds, W, H, depth, 0, 0, [seeds])
    assert np.array_equal(counts, oc[0]) and np.array_equal(rays, orays)
    assert rel_rmse(J.film(), acc) < 1e-5 or np.array_equal(J.film(), acc)
    # benchmark semantics, frames in flight, at the same size
    J2 = api.Job(ctx, S, W, H, max_depth=depth, mode=1, rr_depth=2, film_kahan=1, inflight=3)
    J2.set_camera(sc.camera)
    for f in range(3):
        J2.render(None, float(f + 1))
    film = J2.film()
    assert film.shape == (W * H, 4) and np.isfinite(film).all()
    J2.close()
    J.close()
    S.close()


def test_all_camera_rays_miss(ctx, orc):
    """The camera looks away from the room and there is no environment: every
    queue after the camera rays is empty and the film stays zero."""
    sc = scenes.box_room(32, 24)
    sc.camera = layout.make_camera((0.5, 0.5, 3.0), (0.5, 0.5, 10.0), (0.0, 1.0, 0.0), 30.0, 32, 24)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    for mode in (0, 1):
        J = api.Job(ctx, S, 32, 24, max_depth=4, mode=mode, film_kahan=0)
        J.set_camera(sc.camera)
        J.render(_seeds(4, 3) if mode == 0 else None, 1.0)
        rays, counts = J.stats()
        assert not counts.any() and rays[0] == 32 * 24 and rays[1] == 0 and rays[2] == 0
        assert not J.film().any()
        J.close()
    S.close()


def test_one_triangle_scene(ctx, orc):
    room = scenes.box_room(16, 16)
    sc = scenes.Scene(points=room.points, faces=room.faces[:1].copy(), materials=room.materials,
                      camera=room.camera)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    S = api.Scene(ctx, sc)
    S.build_bvh_device(want_arrays=False)
    env = scenes.sky_env(64, 32)
    S.set_env(env, 64, 32)
    J = api.Job(ctx, S, 16, 16, max_depth=3, mode=1, rr_depth=2, film_kahan=1)
    J.set_camera(sc.camera)
    J.render(None, 1.0)
    assert np.isfinite(J.film()).all() and J.film()[:, :3].sum() > 0
    J.close()
    S.close()


def test_queries_over_no_rays(ctx, orc):
    sc = scenes.box_room(8, 8)
    S = api.Scene(ctx, sc)
    S.build_bvh_device(want_arrays=False)
    empty = np.zeros(0, layout.RAY)
    t, p = S.trace_closest(empty)
    assert t.shape == (0,) and p.shape == (0,)
    assert S.trace_any(empty).shape == (0,)
    S.close()
