"""Served mode: concurrent requests through mt_job_submit / poll / cancel / wait.

A served request runs the same passes as a render job with the same camera, size,
spp and frame numbers (benchmark semantics), so its film must equal that job's film
bit for bit, whatever other requests share the GPU with it.
"""
import numpy as np
import pytest

from mambatracer_gb300 import api, layout, scenes
from mambatracer_gb300._lib import MTError
from tests.helpers import bvh_build

pytestmark = pytest.mark.gpu

DEPTH, RR = 6, 3


def sphere_camera(rng, width, height, radius, target=(0.0, 0.0, 0.0)):
    w = rng.normal(size=3)
    w /= np.linalg.norm(w)
    pos = np.asarray(target) + radius * w
    return layout.make_camera(tuple(pos), target, (0.0, 1.0, 0.0), 45.0, width, height)


@pytest.fixture(scope="module")
def served_scenes(ctx, orc):
    out = {}
    env = scenes.sky_env(256, 128)
    for name, sc in (("room", scenes.box_room(64, 64)), ("soup", scenes.soup(20000, seed=8, extent=0.8)),
                     ("stadium", scenes.stadium(quads=80, level=4))):
        nodes, bounds, _, _ = bvh_build(orc, sc)
        S = api.Scene(ctx, sc)
        S.import_bvh(nodes, bounds)
        if name != "room":
            S.set_env(env, 256, 128)
        out[name] = (sc, S)
    yield out
    for sc, S in out.values():
        S.close()


@pytest.mark.parametrize("merged", [0, 1, 2])
def test_served_films_equal_plain_jobs(ctx, served_scenes, merged):
    """Lanes (a stream each) or merged queues on one or two streams (rounds of one pass
    per scene over the stream's running requests): every film equals the job rendered
    alone."""
    rng = np.random.default_rng(11)
    srv = api.Server(ctx, lanes=4, max_width=256, max_height=256, max_spp=8, max_depth=DEPTH, rr_depth=RR,
                     merged=merged)
    reqs = []
    for k in range(14):
        name = ("room", "soup", "stadium")[k % 3]
        sc, S = served_scenes[name]
        w, h = int(rng.integers(24, 200)), int(rng.integers(24, 160))
        spp = int(rng.choice([1, 2, 4]))
        cam = sc.camera.copy() if name == "room" else sphere_camera(rng, w, h, 3.0 if name == "soup" else 0.4)
        fc = float(1 + 10 * k)
        reqs.append((srv.submit(S, cam, w, h, spp, fc), S, cam, w, h, spp, fc))
    srv.drain()
    st = srv.stats()
    assert st["completed"] == len(reqs) and st["failed"] == 0 and st["queued"] == 0
    assert st["p50_ms"] > 0 and st["p50_ms"] <= st["p95_ms"] <= st["p99_ms"] <= st["max_ms"]
    total = np.zeros(3, np.int64)
    for rid, S, cam, w, h, spp, fc in reqs:
        state, lat = srv.poll(rid)
        assert state == api.Server.DONE and lat > 0
        J = api.Job(ctx, S, w, h, max_depth=DEPTH, mode=1, rr_depth=RR, film_kahan=1, spp=spp)
        J.set_camera(cam)
        J.render(None, fc)
        ref = J.film()
        total += J.total_rays()
        J.close()
        assert srv.film(rid).tobytes() == ref.tobytes(), (rid, w, h, spp)
    assert st["rays"] == total.tolist()
    srv.close()


@pytest.mark.parametrize("merged", [0, 1])
def test_cancel_poll_wait_and_busy_scene(ctx, served_scenes, merged):
    sc, S = served_scenes["soup"]
    rng = np.random.default_rng(12)
    srv = api.Server(ctx, lanes=1, max_width=512, max_height=512, max_spp=16, max_depth=DEPTH, rr_depth=RR,
                     merged=merged)
    big = srv.submit(S, sphere_camera(rng, 512, 512, 3.0), 512, 512, 16, 1.0)
    queued = [srv.submit(S, sphere_camera(rng, 64, 64, 3.0), 64, 64, 1, float(100 + i)) for i in range(3)]
    with pytest.raises(MTError, match="still"):
        srv.wait(queued[-1], timeout_ms=0.0)
    srv.cancel(queued[1])
    with pytest.raises(MTError, match="served requests"):
        S.close()  # the scene is in use
    srv.drain()
    assert srv.poll(big)[0] == api.Server.DONE
    assert srv.poll(queued[0])[0] == api.Server.DONE and srv.poll(queued[2])[0] == api.Server.DONE
    assert srv.poll(queued[1])[0] == api.Server.CANCELLED
    st = srv.stats()
    assert st["completed"] == 3 and st["cancelled"] == 1 and st["max_queue"] >= 3
    with pytest.raises(MTError):
        srv.submit(S, sc.camera, 1024, 1024, 1)  # larger than the server's largest frame
    srv.close()


def test_merged_cancel_running_request(ctx, served_scenes):
    """Merged mode stops a cancelled running request at the next round; the
    requests sharing its rounds, and those after it, still equal jobs alone."""
    _, S = served_scenes["soup"]
    rng = np.random.default_rng(13)
    srv = api.Server(ctx, lanes=3, max_width=384, max_height=384, max_spp=64, max_depth=DEPTH, rr_depth=RR,
                     merged=2)
    big = srv.submit(S, sphere_camera(rng, 384, 384, 3.0), 384, 384, 64, 1.0)
    reqs = []
    for k in range(5):
        w, h = int(rng.integers(16, 120)), int(rng.integers(16, 120))
        cam = sphere_camera(rng, w, h, 3.0)
        reqs.append((srv.submit(S, cam, w, h, 2, float(500 + k)), cam, w, h))
    srv.cancel(big)
    srv.drain()
    assert srv.poll(big)[0] == api.Server.CANCELLED
    st = srv.stats()
    assert st["completed"] == 5 and st["cancelled"] == 1 and st["failed"] == 0
    for k, (rid, cam, w, h) in enumerate(reqs):
        assert srv.poll(rid)[0] == api.Server.DONE
        J = api.Job(ctx, S, w, h, max_depth=DEPTH, mode=1, rr_depth=RR, film_kahan=1, spp=2)
        J.set_camera(cam)
        J.render(None, float(500 + k))
        assert srv.film(rid).tobytes() == J.film().tobytes()
        J.close()
    srv.close()


def test_merged_mixed_scenes_equal_jobs_alone(ctx):
    """One merged server over a textured scene, a scene with FP16 records and a scene
    with FP32 records: rounds hold one merged pass per scene, and every film equals the
    request rendered alone as a job."""
    rng = np.random.default_rng(14)
    tex = scenes.textured_room(64, 48)
    S_tex = api.Scene(ctx, tex)
    S_tex.build_bvh_device(want_arrays=False)
    soup = scenes.soup(20000, seed=9, extent=0.8)
    S16 = api.Scene(ctx, soup)
    S16.build_bvh_device(want_arrays=False)
    S16.set_env(scenes.sky_env(256, 128), 256, 128)
    S16.set_precision(1)
    S32 = api.Scene(ctx, soup)
    S32.build_bvh_device(want_arrays=False)
    S32.set_env(scenes.sky_env(256, 128), 256, 128)
    srv = api.Server(ctx, lanes=5, max_width=160, max_height=120, max_spp=4, max_depth=DEPTH, rr_depth=RR, merged=2)
    reqs = []
    for k in range(12):
        S, sc = ((S_tex, tex), (S16, soup), (S32, soup))[k % 3]
        w, h = int(rng.integers(16, 160)), int(rng.integers(16, 120))
        cam = tex.camera.copy() if S is S_tex else sphere_camera(rng, w, h, 3.0)
        spp, fc = int(rng.integers(1, 5)), float(3 + 7 * k)
        reqs.append((srv.submit(S, cam, w, h, spp, fc), S, cam, w, h, spp, fc))
    srv.drain()
    assert srv.stats()["completed"] == len(reqs)
    for rid, S, cam, w, h, spp, fc in reqs:
        J = api.Job(ctx, S, w, h, max_depth=DEPTH, mode=1, rr_depth=RR, film_kahan=1, spp=spp)
        J.set_camera(cam)
        J.render(None, fc)
        assert srv.film(rid).tobytes() == J.film().tobytes(), (rid, w, h, spp)
        J.close()
    srv.close()
    for S in (S_tex, S16, S32):
        S.close()
