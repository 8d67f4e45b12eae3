"""The GPU BVH build against the host build of CNormalBVH.build
(src/cl/scene/CNormalBVH.java:45-148): the reference-layout nodes equal
element for element, the bounds equal as values (a -0.0 / +0.0 tie may keep
either zero: the host keeps the first it meets, the GPU's integer-keyed
minimum keeps -0.0), and the traversal layout built on the GPU equals the one
imported from the host build, so rays hit the same triangles at the same
distances (0 ulp)."""
import numpy as np
import pytest

from mambatracer_gb300 import api, layout, scenes

pytestmark = pytest.mark.gpu


def _subset(sc, k):
    return scenes.Scene(points=sc.points, faces=sc.faces[:k].copy(), materials=sc.materials, camera=sc.camera)


def _stacked(k):
    """k copies of one triangle: every centroid bound is a point, so every split
    falls back to the middle index."""
    sc = scenes.box_room(8, 8)
    faces = np.repeat(sc.faces[:1], k)
    return scenes.Scene(points=sc.points, faces=faces, materials=sc.materials, camera=sc.camera)


CASES = {
    "one": lambda: _subset(scenes.box_room(8, 8), 1),
    "two": lambda: _subset(scenes.box_room(8, 8), 2),
    "three": lambda: _subset(scenes.box_room(8, 8), 3),
    "room": lambda: scenes.box_room(64, 48),
    "stacked": lambda: _stacked(1000),
    "soup": lambda: scenes.soup(20000, seed=3, extent=0.7, edge_sigma=0.01),
    "stadium": lambda: scenes.stadium(quads=60, level=4, width=64, height=48),
    "soup_large": lambda: scenes.soup(400000, seed=12, extent=0.9, edge_sigma=0.004),
}


def _layout_equal(a, b):
    ra, ta, roota = a
    rb, tb, rootb = b
    assert roota == rootb
    assert ra.shape == rb.shape and ta.shape == tb.shape
    assert np.array_equal(ra[:, :12], rb[:, :12])              # child boxes (values)
    assert ra[:, 12:].tobytes() == rb[:, 12:].tobytes()       # child refs, padding
    assert ta.tobytes() == tb.tobytes()                       # triangle slots


@pytest.mark.parametrize("which", list(CASES))
def test_device_build_equals_host(ctx, which):
    sc = CASES[which]()
    hn, hb, hd = api.bvh_build_host(sc)
    S = api.Scene(ctx, sc)
    dn, db = S.build_bvh_device()
    assert S.depth == hd
    assert np.array_equal(dn, hn)
    assert np.array_equal(db, hb)
    dev = S.layout()
    S.import_bvh(hn, hb)
    host = S.layout()
    _layout_equal(dev, host)
    S.close()


@pytest.mark.parametrize("which", ["room", "soup", "stadium"])
def test_device_build_traces_identically(ctx, which):
    sc = CASES[which]()
    o, d = scenes.random_rays(sc, 50000, seed=17, inside=True)
    rays = layout.make_rays(o, d)
    S = api.Scene(ctx, sc)
    S.build_bvh()
    t0, p0 = S.trace_closest(rays)
    a0 = S.trace_any(layout.make_rays(o, d, tmin=1e-4, tmax=0.3))
    S.build_bvh_device(want_arrays=False)
    t1, p1 = S.trace_closest(rays)
    a1 = S.trace_any(layout.make_rays(o, d, tmin=1e-4, tmax=0.3))
    assert (p0 >= 0).sum() > 1000
    assert np.array_equal(p0, p1)
    assert t0.tobytes() == t1.tobytes()
    assert np.array_equal(a0, a1)
    S.close()


def test_device_build_then_frame(ctx):
    """A job renders the same film after a device build as after the host build
    (the scene version change rebuilds the job's graphs)."""
    sc = scenes.box_room(64, 48)
    S = api.Scene(ctx, sc)
    S.build_bvh()
    J = api.Job(ctx, S, 64, 48, max_depth=4, mode=1, film_kahan=0)
    J.set_camera(sc.camera)
    seeds = np.arange(2 * (1 + 2 * 4), dtype=np.int32) + 1000
    J.render(seeds, 1.0)
    f0 = J.film()
    J.clear()
    S.build_bvh_device(want_arrays=False)
    J.render(seeds, 1.0)
    f1 = J.film()
    assert f0.tobytes() == f1.tobytes()
    J.close()
    S.close()
