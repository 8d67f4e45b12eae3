"""The oracle's pixel-subset frames (oracle.check.subset_frames, used by the image
error check of the benchmark configurations): in benchmark semantics every sample
is keyed on its pixel, so rendering a subset gives, pixel for pixel, the film and
the queue lengths of the full frame, in FP32 and in FP64."""
import numpy as np
import pytest

from mambatracer_gb300 import scenes
from oracle import check
from tests.helpers import bvh_build, oracle_frames, oracle_grid


@pytest.mark.parametrize("fp64", [False, True])
def test_subset_equals_full_frame(orc, fp64):
    sc = scenes.soup(20000, seed=6, extent=0.8, edge_sigma=0.015, width=64, height=48)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    env = (scenes.sky_env(256, 128), 256, 128)
    func, gsat = oracle_grid(orc, env, 160, 160, 16, 32)
    grid = dict(func=func, sat=gsat, nu=160, nv=160, rx=16, ry=32)
    for fc in (4, 5):
        full, cnt, rays = oracle_frames(orc, sc, nodes, bounds, 64, 48, 6, 1, 3, [None], env=env, fp64=fp64,
                                        first_frame=fc, grid=grid)
        px = check.strided_pixels(64, 48, 4)
        acc, _, _ = check.subset_frames(orc, sc, nodes, bounds, 64, 48, 6, 3, [fc], px, env, fp64, grid=grid)
        assert np.array_equal(acc, full[px].astype(np.float64))
        allpx = np.arange(64 * 48, dtype=np.int32)
        acc, c, r = check.subset_frames(orc, sc, nodes, bounds, 64, 48, 6, 3, [fc], allpx, env, fp64, grid=grid,
                                        chunks=5)
        assert np.array_equal(acc, full.astype(np.float64))
        assert np.array_equal(c, cnt.sum(0)) and np.array_equal(r, rays)


def test_subset_refused_in_reference_semantics(orc):
    sc = scenes.box_room(8, 8)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    from oracle.oracle import ptr
    acc = np.zeros((4, 4), np.float32)
    px = np.arange(4, dtype=np.int32)
    seeds = np.arange(1, 2 * (1 + 2 * 2) + 1, dtype=np.int32)
    z = np.zeros(4, np.float32)
    rc = orc.lib.or_render_frame_subset(ptr(sc.camera), 8, 8, 2, 0, 0, ptr(seeds), 1.0, ptr(sc.points),
                                        ptr(sc.uvs), ptr(sc.normals), ptr(sc.faces), sc.ntri, ptr(sc.materials),
                                        ptr(nodes), ptr(bounds), ptr(z), ptr(z), ptr(z), 1, 1, 0, 0, ptr(acc), None,
                                        None, None, None, None, 0, 0, 0, 0, None, 0, 0, ptr(px), 4)
    assert rc == -1


def test_edge_distance_and_hit_parity(orc):
    """Barycentric edge distance of a hit at a known point, and the parity summary."""
    from mambatracer_gb300 import layout
    sc = scenes.box_room(8, 8)
    rays = check.primary_rays(orc, sc.camera, 8, 8, 1.0)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    t, p = check.trace_oracle(orc, sc, nodes, bounds, rays)
    d = check.edge_distance(sc, rays, p)
    assert np.all((d[p >= 0] >= -1e-6) & (d[p >= 0] <= 1.0 / 3.0 + 1e-6))
    assert np.all(np.isinf(d[p < 0]))
    s = check.hit_parity(sc, rays, t, p, t, p)
    assert s["hit_id_mismatches"] == 0 and s["rays"] == 64 and s["max_t_ulps_same_id"] == 0
    p2 = p.copy()
    p2[0] = (p[0] + 1) % sc.ntri
    s = check.hit_parity(sc, rays, t, p2, t, p)
    assert s["hit_id_mismatches"] == 1 and s["mismatches_exact_t_ties"] == 1
    assert layout.RAY.itemsize == 80
