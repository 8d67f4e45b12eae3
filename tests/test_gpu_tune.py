"""Launch shapes change the speed, never the film: benchmark-semantics frames rendered
under different tunings (traversal and shading builds, shared traversal grids, refill
steps) are bit-identical, including a job whose graphs are captured again after a
change between frames, and a merged batch."""
import numpy as np
import pytest

from mambatracer_gb300 import api, scenes
from tests.helpers import bvh_build

pytestmark = pytest.mark.gpu

OTHER = {"closest_minb": 8, "shadow_minb": 16, "closest_grid": 3, "shadow_grid": 6, "shade_minb": 3,
         "refill_steps": 16, "shadow_stream": 0}


@pytest.fixture
def soup_scene(ctx, orc):
    sc = scenes.soup(20000, seed=8, extent=0.8, width=96, height=64)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    S.set_env(scenes.sky_env(256, 128), 256, 128)
    yield sc, S
    S.close()


def _film(ctx, S, cam, frames, inflight, switch_at=None):
    J = api.Job(ctx, S, 96, 64, max_depth=6, mode=1, rr_depth=3, film_kahan=1, use_graph=1, inflight=inflight)
    J.set_camera(cam)
    for f in range(frames):
        if f == switch_at:
            api.set_tuning(OTHER)
        J.render(None, float(f + 1))
    film = J.film()
    J.close()
    return film


def test_films_do_not_depend_on_the_tuning(ctx, soup_scene):
    sc, S = soup_scene
    before = api.get_tuning()
    try:
        ref = _film(ctx, S, sc.camera, 4, 3)
        switched = _film(ctx, S, sc.camera, 4, 3, switch_at=2)  # graphs captured again mid-job
        assert switched.tobytes() == ref.tobytes()
        other = _film(ctx, S, sc.camera, 4, 3)  # OTHER throughout
        assert other.tobytes() == ref.tobytes()
        for prec in (1, 0):
            S.set_precision(prec)
            frames = [(sc.camera, 96, 64, 2, 1.0), (sc.camera, 40, 30, 3, 9.0)]
            api.set_tuning(before)
            a, ra = api.batch_render(ctx, S, frames, max_depth=6, rr_depth=3)
            api.set_tuning(OTHER)
            b, rb = api.batch_render(ctx, S, frames, max_depth=6, rr_depth=3)
            assert all(x.tobytes() == y.tobytes() for x, y in zip(a, b)) and np.array_equal(ra, rb)
    finally:
        api.set_tuning(before)
