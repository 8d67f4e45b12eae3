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


_SINGLE_LAUNCH = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
from mambatracer_gb300 import api, scenes
from oracle.oracle import Oracle, bvh_build
sc = scenes.soup(20000, seed=8, extent=0.8, width=96, height=64)
nodes, bounds, _, _ = bvh_build(Oracle(), sc)
ctx = api.Context(0)
S = api.Scene(ctx, sc)
S.import_bvh(nodes, bounds)
S.set_env(scenes.sky_env(256, 128), 256, 128)
S.grid_config(160, 160, 16, 32, {grid})
J = api.Job(ctx, S, 96, 64, max_depth=6, mode=1, rr_depth=3, film_kahan=1, use_graph=1, inflight=2,
            grid_updates=0)
J.set_camera(sc.camera)
for f in range(4):
    J.render(None, float(f + 1))
np.save({out!r}, J.film())
rays = J.total_rays()
np.save({out!r} + ".rays.npy", rays)
np.save({out!r} + ".launches.npy", np.array([J.launches()]))
J.close(); S.close(); ctx.close()
"""


@pytest.mark.parametrize("grid", [0, 2])
def test_two_launch_shading_equals_one_launch(ctx, soup_scene, tmp_path, grid):
    """Benchmark-semantics shading runs in two launches (hit phase, then the
    paths that go on); MT_SHADE_SPLIT=0 (read once per process) runs the single
    kernel. Films and ray counts are bit-identical either way. The light grid
    stays at its initial function: its updates sum environment hits with float
    atomics, whose order no two runs share."""
    import os
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    films = []
    for split in ("1", "0"):
        out = str(tmp_path / f"film{split}.npy")
        env = dict(os.environ, MT_SHADE_SPLIT=split)
        subprocess.run([sys.executable, "-c", _SINGLE_LAUNCH.format(root=root, out=out, grid=grid)], env=env,
                       check=True, timeout=600)
        films.append((np.load(out), np.load(out + ".rays.npy"), int(np.load(out + ".launches.npy")[0])))
    # launches (mt_job_launches): 4 frames x (raygen + 6 bounces x (closest hits,
    # shading in 2 or 1 launches, shadow rays) + ray totals) + 4 film merges
    assert films[0][2] == 4 * (2 + 6 * 4) + 4 and films[1][2] == 4 * (2 + 6 * 3) + 4
    assert films[0][0].tobytes() == films[1][0].tobytes()
    assert np.array_equal(films[0][1], films[1][1])
    assert films[0][0][:, :3].sum() > 0
