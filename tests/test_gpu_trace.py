"""GPU traversal parity: closest hit and any hit through the C-ABI against the
oracle and the golden outputs of the reference kernels. Hit ids and hit
distances are compared bit for bit (0 ulp)."""
import numpy as np
import pytest

from mambatracer_gb300 import _lib, api, layout, scenes
from tests.helpers import bvh_build, oracle_any, oracle_trace, ptr

pytestmark = pytest.mark.gpu


def gpu_scene(ctx, orc, sc):
    nodes, bounds, depth, _ = bvh_build(orc, sc)
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    return S, nodes, bounds


def test_golden_rays(ctx, orc, ginputs, golden):
    sc = ginputs["soup"]
    S, nodes, bounds = gpu_scene(ctx, orc, sc)
    for key in ("rays_in", "rays_out"):
        t, p = S.trace_closest(ginputs[key])
        assert np.array_equal(p, golden[key + "_id"]), key
        assert t.tobytes() == golden[key + "_tmax"].tobytes(), key
    occ = S.trace_any(ginputs["rays_shadow"])
    assert np.array_equal(occ, golden["rays_shadow_occ"])
    S.close()


@pytest.mark.parametrize("inside", [True, False])
def test_dense_soup(ctx, orc, inside):
    sc = scenes.soup(200000, seed=41, extent=0.6, edge_sigma=0.01)
    S, nodes, bounds = gpu_scene(ctx, orc, sc)
    o, d = scenes.random_rays(sc, 100000, seed=42, inside=inside)
    rays = layout.make_rays(o, d)
    t, p = S.trace_closest(rays)
    to, po = oracle_trace(orc, sc, nodes, bounds, rays)
    assert (po >= 0).sum() > (20000 if inside else 3000)
    assert np.array_equal(p, po)
    assert t.tobytes() == to.tobytes()
    rays2 = layout.make_rays(o, d, tmin=1e-4, tmax=0.2)
    assert np.array_equal(S.trace_any(rays2), oracle_any(orc, sc, nodes, bounds, rays2))
    S.close()


def test_primary_rays_box_room(ctx, orc):
    sc = scenes.box_room(160, 120)
    S, nodes, bounds = gpu_scene(ctx, orc, sc)
    rays = np.zeros(160 * 120, layout.RAY)
    seed = np.array([536870923, 805306457], np.int32)
    orc.lib.or_raygen(ptr(sc.camera), ptr(rays), ptr(seed), 1.0, rays.shape[0], 0)
    t, p = S.trace_closest(rays)
    to, po = oracle_trace(orc, sc, nodes, bounds, rays)
    assert np.array_equal(p, po) and t.tobytes() == to.tobytes()
    assert (p >= 0).mean() > 0.7  # the open front of the room shows the background
    S.close()


def test_axis_aligned_and_degenerate_rays(ctx, orc):
    """Zero direction components give infinite 1/d and NaN slab terms (Util.cl:707-732);
    the GPU must take the same branches."""
    sc = scenes.box_room(8, 8)
    S, nodes, bounds = gpu_scene(ctx, orc, sc)
    rng = np.random.default_rng(3)
    n = 20000
    o = rng.uniform(-0.2, 1.2, size=(n, 3)).astype(np.float32)
    o[: n // 4, 0] = 0.5  # origins on slab planes
    o[n // 4: n // 2, 1] = 0.0
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32)
    d[::3, 0] = 0.0
    d[1::3, 1] = 0.0
    d[2::5, 2] = 0.0
    d[::7] = np.array([0.0, 0.0, -1.0], np.float32)
    rays = layout.make_rays(o, d)
    t, p = S.trace_closest(rays)
    to, po = oracle_trace(orc, sc, nodes, bounds, rays)
    assert np.array_equal(p, po) and t.tobytes() == to.tobytes()
    rays2 = layout.make_rays(o, d, tmin=1e-4, tmax=0.3)
    assert np.array_equal(S.trace_any(rays2), oracle_any(orc, sc, nodes, bounds, rays2))
    S.close()


def test_single_triangle(ctx, orc):
    room = scenes.box_room(8, 8)
    sc = scenes.Scene(points=room.points[:3].copy(), faces=room.faces[:1].copy(), materials=room.materials)
    S, nodes, bounds = gpu_scene(ctx, orc, sc)
    o = np.tile(np.array([[0.3, 0.5, 0.6]], np.float32), (4, 1))  # above (0.3, 0, 0.6), inside the triangle
    d = np.array([[0, -1, 0], [0, 1, 0], [1, 0, 0], [0, -1, 0.0001]], np.float32)
    rays = layout.make_rays(o, d)
    t, p = S.trace_closest(rays)
    to, po = oracle_trace(orc, sc, nodes, bounds, rays)
    assert p[0] == 0 and np.array_equal(p, po) and t.tobytes() == to.tobytes()
    S.close()


def test_too_deep_bvh_is_rejected(ctx):
    """The reference traversal keeps a 64-bit bitstack (NormalBVH.cl:20); deeper trees are refused."""
    k = 120  # depth 71 with this spacing
    pts = []
    for i in range(k):
        x = 2.0 ** (-i)
        pts += [(x, 0, 0), (x, 0.001, 0), (x, 0, 0.001)]
    p4 = np.zeros((len(pts), 4), np.float32)
    p4[:, :3] = pts
    room = scenes.box_room(8, 8)
    faces = np.zeros(k, layout.FACE)
    idx = np.arange(3 * k, dtype=np.int32).reshape(-1, 3)
    faces["vx"], faces["vy"], faces["vz"] = idx[:, 0], idx[:, 1], idx[:, 2]
    faces["uvx"] = faces["uvy"] = faces["uvz"] = faces["nx"] = faces["ny"] = faces["nz"] = -1
    sc = scenes.Scene(points=p4, faces=faces, materials=room.materials[:1])
    S = api.Scene(ctx, sc)
    with pytest.raises(_lib.MTError) as e:
        S.build_bvh()
    assert e.value.code == -4
    S.close()
