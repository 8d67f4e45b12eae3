"""Merged batches (mt_batch_render): frames of uneven size, cameras and spp
through one set of wavefront queues. Each frame's film equals the frame
rendered alone by a job with the same settings, bit for bit, and the batch's
ray counts are the sum of the frames' (benchmark semantics, full-map
environment sampling)."""
import numpy as np
import pytest

from mambatracer_gb300 import api, layout, scenes
from mambatracer_gb300._lib import MTError

pytestmark = pytest.mark.gpu

DEPTH, RR = 6, 3


def sphere_camera(rng, w, h, radius):
    d = rng.normal(size=3)
    d /= np.linalg.norm(d)
    return layout.make_camera(tuple(radius * d), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 45.0, w, h)


@pytest.mark.parametrize("which", ["soup_env", "room", "tex_room"])
def test_batch_frames_equal_frames_alone(ctx, which):
    rng = np.random.default_rng(21)
    if which == "soup_env":
        sc = scenes.soup(20000, seed=8, extent=0.8)
    elif which == "room":
        sc = scenes.box_room(64, 64)
    else:
        sc = scenes.textured_room(64, 64)
    S = api.Scene(ctx, sc)
    S.build_bvh_device(want_arrays=False)
    if which == "soup_env":
        S.set_env(scenes.sky_env(256, 128), 256, 128)
    frames = []
    for k in range(9):
        w, h = int(rng.integers(16, 160)), int(rng.integers(8, 120))
        cam = sphere_camera(rng, w, h, 3.0) if which == "soup_env" else sc.camera.copy()
        frames.append((cam, w, h, int(rng.choice([1, 2, 3])), float(1 + 7 * k)))
    films, rays = api.batch_render(ctx, S, frames, max_depth=DEPTH, rr_depth=RR, film_kahan=1)
    total = np.zeros(3, np.int64)
    for (cam, w, h, spp, fc), film in zip(frames, films):
        J = api.Job(ctx, S, w, h, max_depth=DEPTH, mode=1, rr_depth=RR, film_kahan=1, spp=spp)
        J.set_camera(cam)
        J.render(None, fc)
        assert film.tobytes() == J.film().tobytes(), (w, h, spp)
        total += J.total_rays()
        J.close()
    assert np.array_equal(rays, total)
    S.close()


def test_batch_arguments_checked(ctx):
    sc = scenes.box_room(8, 8)
    S = api.Scene(ctx, sc)
    with pytest.raises(MTError, match="BVH"):
        api.batch_render(ctx, S, [(sc.camera, 8, 8, 1, 1.0)])
    S.build_bvh_device(want_arrays=False)
    with pytest.raises(MTError, match="frame 0"):
        api.batch_render(ctx, S, [(sc.camera, 0, 8, 1, 1.0)])
    with pytest.raises(MTError, match="max_depth"):
        api.batch_render(ctx, S, [(sc.camera, 8, 8, 1, 1.0)], max_depth=0)
    S.close()
