"""Quantised traversal formats (mt_scene_set_bvh_precision):

1. FP16 records: child boxes rounded outward to half precision, 32 bytes per
   record. The traversal enters every node the FP32 records let it enter, so
   closest hits are the same triangles at the same distances (bit for bit) and
   any-hit answers are the same; the only freedom is which of two triangles hit
   at exactly the same distance is kept, when the changed visit order meets them
   the other way round.
2. The wide BVH: the same tree collapsed into nodes of up to eight children with
   8-bit child boxes rounded outward (96-byte nodes). Its boxes contain the FP32
   boxes, and its triangle test is the same FP32 Moller-Trumbore, so any-hit
   answers are the same and so is every closest hit, except where two triangles
   are hit within a few ulps of each other (coplanar surfaces: the box room's
   boxes stand on its floor): the reference's slab test on a flat triangle box
   then sometimes skips the nearer one, which the wide traversal tests. Those
   rays are counted, and the wide traversal's distance is never the larger.
3. 4-wide FP16 nodes: a record's grandchildren with the FP16 records' boxes (the
   intermediate level's boxes are not tested): the same hits, except among
   triangles hit at exactly or within a few ulps of the same distance, where
   either may be kept, and the one kept may change between runs (leaf tests
   wait for the warp).

Frames in benchmark semantics are compared with the FP32 records' frames."""
import numpy as np
import pytest

from mambatracer_gb300 import api, layout, scenes
from mambatracer_gb300._lib import MTError
from tests.helpers import rel_rmse

pytestmark = pytest.mark.gpu

CASES = {
    "room": lambda: scenes.box_room(64, 48),
    "soup": lambda: scenes.soup(200000, seed=8, extent=0.8, edge_sigma=0.01),
    "stadium": lambda: scenes.stadium(quads=300, level=6, width=64, height=48),
}


@pytest.mark.parametrize("prec", [1, 2, 3])
@pytest.mark.parametrize("which", list(CASES))
def test_quantised_formats_trace_the_same_hits(ctx, which, prec):
    sc = CASES[which]()
    S = api.Scene(ctx, sc)
    S.build_bvh_device(want_arrays=False)
    o, d = scenes.random_rays(sc, 200000, seed=19, inside=True)
    rays = layout.make_rays(o, d)
    srays = layout.make_rays(o, d, tmin=1e-4, tmax=0.25)
    t0, p0 = S.trace_closest(rays)
    a0 = S.trace_any(srays)
    S.set_precision(prec)
    t1, p1 = S.trace_closest(rays)
    a1 = S.trace_any(srays)
    assert (p0 >= 0).sum() > 10000
    assert np.array_equal(a0, a1)
    tdiff = t0.view(np.uint32) != t1.view(np.uint32)
    differ = p0 != p1
    if prec == 1 or which != "room":
        assert not tdiff.any()
        assert differ.sum() <= 1e-4 * len(p0), differ.sum()   # exact-distance ties only
    else:
        # coplanar triangles hit within a few ulps: the wide BVH keeps the nearer;
        # the 4-wide nodes keep either
        ulps = np.abs(t0.view(np.int32).astype(np.int64) - t1.view(np.int32).astype(np.int64))
        print(f"room, format {prec}: {differ.sum()} of {len(p0)} hit ids differ, {tdiff.sum()} distances "
              f"(at most {ulps.max()} ulps, {(t1[tdiff] > t0[tdiff]).sum()} farther)")
        assert ulps.max() <= 8
        assert prec == 3 or np.all(t1[tdiff] < t0[tdiff])
        assert differ.sum() <= 0.01 * len(p0)
        assert np.all(differ | ~tdiff)
    # a rebuild keeps the format; going back to FP32 gives the FP32 answers
    S.build_bvh_device(want_arrays=False)
    t2, p2 = S.trace_closest(rays)
    if prec == 3:
        # among coplanar triangles the one kept depends on when the warp tests
        # its waiting leaves, so it may change between runs (by a few ulps)
        ulps2 = np.abs(t2.view(np.int32).astype(np.int64) - t1.view(np.int32).astype(np.int64))
        assert ulps2.max() <= (8 if which == "room" else 0)
        assert (p2 != p1).sum() <= (0.01 if which == "room" else 1e-4) * len(p1)
    else:
        assert t2.tobytes() == t1.tobytes() and np.array_equal(p2, p1)
    # the traversal work: the FP32 records' triangle tests are the oracle's
    # (deferred leaves are always tested); the quantised formats test fewer or
    # more boxes but reach every triangle the FP32 records do
    _, _, c1 = S.trace_counts(rays[:20000])
    assert np.all(c1[:, 0] > 0)
    S.set_precision(0)
    t3, p3 = S.trace_closest(rays)
    assert t3.tobytes() == t0.tobytes() and np.array_equal(p3, p0)
    S.close()


def _same_or_nearer(t0, p0, t1, p1, prec):
    """Format 1: the same distances; the wide BVH (2): the same, or the nearer of
    coplanar triangles hit within a few ulps; the 4-wide nodes (3): either."""
    tdiff = t0.view(np.uint32) != t1.view(np.uint32)
    if prec == 1:
        assert not tdiff.any()
        return
    ulps = np.abs(t0.view(np.int32).astype(np.int64) - t1.view(np.int32).astype(np.int64))
    assert (ulps.max() if tdiff.any() else 0) <= 8
    assert prec == 3 or np.all(t1[tdiff] < t0[tdiff])
    assert np.all((p0 != p1) | ~tdiff)


@pytest.mark.parametrize("prec", [1, 2, 3])
def test_quantised_formats_axis_aligned_rays(ctx, prec):
    """Zero direction components (infinite 1/d, NaN slab terms: the traversal takes
    the reference's comparison chain, Util.cl:707-732) and origins on box planes:
    the quantised formats give the FP32 records' distances and any-hit answers."""
    sc = scenes.box_room(8, 8)
    S = api.Scene(ctx, sc)
    S.build_bvh_device(want_arrays=False)
    rng = np.random.default_rng(3)
    n = 20000
    o = rng.uniform(-0.2, 1.2, size=(n, 3)).astype(np.float32)
    o[: n // 4, 0] = 0.5
    o[n // 4: n // 2, 1] = 0.0
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    d[::3, 0] = 0.0
    d[1::3, 1] = 0.0
    d[2::5, 2] = 0.0
    d[::7] = np.array([0.0, 0.0, -1.0], np.float32)
    rays = layout.make_rays(o, d)
    srays = layout.make_rays(o, d, tmin=1e-4, tmax=0.3)
    t0, p0 = S.trace_closest(rays)
    a0 = S.trace_any(srays)
    S.set_precision(prec)
    t1, p1 = S.trace_closest(rays)
    assert np.array_equal(S.trace_any(srays), a0)
    assert (p0 >= 0).sum() > n // 4
    # the box room's coplanar triangles
    _same_or_nearer(t0, p0, t1, p1, prec)
    S.close()


@pytest.mark.parametrize("prec", [1, 2, 3])
@pytest.mark.parametrize("ntri", [1, 2, 3, 5])
def test_quantised_formats_tiny_trees(ctx, prec, ntri):
    """A root that is a leaf, and nodes with fewer than four (eight) children."""
    room = scenes.box_room(8, 8)
    sc = scenes.Scene(points=room.points.copy(), faces=room.faces[:ntri].copy(), materials=room.materials)
    S = api.Scene(ctx, sc)
    S.build_bvh_device(want_arrays=False)
    o, d = scenes.random_rays(room, 20000, seed=5, inside=True)
    rays = layout.make_rays(o, d)
    t0, p0 = S.trace_closest(rays)
    a0 = S.trace_any(rays)
    S.set_precision(prec)
    t1, p1 = S.trace_closest(rays)
    assert np.array_equal(S.trace_any(rays), a0)
    assert (p0 >= 0).sum() > 0
    _same_or_nearer(t0, p0, t1, p1, prec)
    assert np.array_equal(p0 >= 0, p1 >= 0)
    S.close()


def test_fp16_records_render(ctx):
    sc = scenes.soup(100000, seed=3, extent=0.8, edge_sigma=0.01)
    env = scenes.sky_env(512, 256)
    S = api.Scene(ctx, sc)
    S.build_bvh_device(want_arrays=False)
    S.set_env(env, 512, 256)
    films = []
    for prec in (0, 1, 2):
        S.set_precision(prec)
        J = api.Job(ctx, S, 96, 64, max_depth=8, mode=1, rr_depth=3, film_kahan=1)
        J.set_camera(sc.camera)
        for f in range(4):
            J.render(None, float(f + 1))
        films.append(J.film())
        J.close()
    assert rel_rmse(films[1], films[0]) < 1e-4
    assert rel_rmse(films[2], films[0]) < 1e-4
    S.close()


def test_precision_argument_checked(ctx):
    S = api.Scene(ctx, scenes.box_room(8, 8))
    with pytest.raises(MTError):
        S.set_precision(4)
    S.close()


def test_record_formats_against_fp64_oracle(ctx, orc):
    """Both record formats' films (benchmark semantics, Kahan film) against the FP64
    oracle at matched samples: relative RMSE within 1e-3 each, and the two films
    within 1e-4 of each other (the same hits, up to exact-distance ties)."""
    from tests.helpers import bvh_build, env_tables, oracle_frames
    sc = scenes.soup(20000, seed=4, extent=0.8, edge_sigma=0.02, width=64, height=48)
    env = scenes.sky_env(256, 128)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    lum, sat = env_tables(orc, env, 256, 128)
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    S.set_env_with_sat(env, lum, sat, 256, 128)
    depth, spp = 6, 4
    films = {}
    for prec in (0, 1, 2):
        S.set_precision(prec)
        J = api.Job(ctx, S, 64, 48, max_depth=depth, mode=1, rr_depth=3, film_kahan=1, spp=spp)
        J.set_camera(sc.camera)
        J.render(None, 1.0)
        films[prec] = J.film()
        J.close()
    acc64, _, _ = oracle_frames(orc, sc, nodes, bounds, 64, 48, depth, 1, 3, [None] * spp,
                                env=(env, 256, 128), fp64=True)
    e32, e16, e8 = rel_rmse(films[0], acc64), rel_rmse(films[1], acc64), rel_rmse(films[2], acc64)
    print(f"relative RMSE vs FP64 oracle: FP32 records {e32:.3e}, FP16 records {e16:.3e}, wide 8-bit {e8:.3e}")
    assert e32 < 1e-3 and e16 < 1e-3 and e8 < 1e-3
    assert rel_rmse(films[1], films[0]) < 1e-4
    assert rel_rmse(films[2], films[0]) < 1e-4
    S.close()
