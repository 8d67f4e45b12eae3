"""The oracle against the reference kernels themselves (compiled as C++ from
the MambaTracer sources), on more and larger seeded cases than the golden
fixtures hold. Runs only where oracle/_ref was built (the reference tree is
present); the golden-fixture tests cover the same functions everywhere."""
import numpy as np
import pytest

from mambatracer_gb300 import layout, scenes
from oracle.oracle import RefOracle
from tests.helpers import bvh_build, env_tables, ptr

pytestmark = pytest.mark.skipif(not RefOracle.available(), reason="reference kernels not built here")


@pytest.fixture(scope="module")
def ref():
    return RefOracle()


@pytest.mark.parametrize("seed", [31, 32])
def test_intersect_dense(orc, ref, seed):
    sc = scenes.soup(20000, seed=seed, extent=0.5, edge_sigma=0.03)  # dense: most rays hit
    nodes, bounds, _, _ = bvh_build(orc, sc)
    o, d = scenes.random_rays(sc, 20000, seed=seed + 100)
    ra = layout.make_rays(o, d)
    rb = ra.copy()
    ia = np.zeros(len(ra), layout.INTERSECTION)
    ib = ia.copy()
    ref.lib.ref_intersect(ptr(ra), ptr(ia), len(ra), len(ra), ptr(sc.points), ptr(sc.uvs), ptr(sc.normals),
                          ptr(sc.faces), sc.ntri, ptr(nodes), ptr(bounds))
    orc.lib.or_intersect(ptr(rb), ptr(ib), len(rb), len(rb), ptr(sc.points), ptr(sc.uvs), ptr(sc.normals),
                         ptr(sc.faces), sc.ntri, ptr(nodes), ptr(bounds), None)
    assert (ia["hit"] == 1).sum() > 5000
    assert ra.tobytes() == rb.tobytes()
    m = ia["hit"] == 1
    for f in layout.INTERSECTION.names:  # named fields only: padding bytes carry no value
        assert ia[f][m].tobytes() == ib[f][m].tobytes(), f


@pytest.mark.parametrize("depth,frames", [(4, 2), (15, 1)])
def test_frames_box_room(orc, ref, depth, frames):
    sc = scenes.box_room(48, 40)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    rng = np.random.default_rng(depth)
    cam = sc.camera.copy()
    acc_a = np.zeros((48 * 40, 4), np.float32)
    acc_b = acc_a.copy()
    z = np.zeros(4, np.float32)
    for f in range(frames):
        seeds = rng.integers(2 ** 29, 2 ** 30, size=2 * (1 + 2 * depth)).astype(np.int32)
        ca = np.zeros(depth, np.int32)
        cb = ca.copy()
        ref.lib.ref_render_frame(ptr(cam), 48, 40, depth, ptr(seeds), float(f + 1), ptr(sc.points), ptr(sc.uvs),
                                 ptr(sc.normals), ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds),
                                 ptr(z), ptr(z), ptr(z), 1, 1, 0, ptr(acc_a), ptr(ca))
        orc.lib.or_render_frame(ptr(cam), 48, 40, depth, 0, 0, ptr(seeds), float(f + 1), ptr(sc.points), ptr(sc.uvs),
                                ptr(sc.normals), ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds),
                                ptr(z), ptr(z), ptr(z), 1, 1, 0, 0, ptr(acc_b), ptr(cb), None)
        assert np.array_equal(ca, cb)
    assert acc_a.tobytes() == acc_b.tobytes()


def test_frame_soup_with_env(orc, ref):
    sc = scenes.soup(40000, seed=2, extent=0.8, edge_sigma=0.02)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    env = scenes.sky_env(256, 128)
    lum, sat = env_tables(orc, env, 256, 128)
    cam = sc.camera.copy()
    acc_a = np.zeros((40 * 32, 4), np.float32)
    acc_b = acc_a.copy()
    seeds = np.random.default_rng(3).integers(2 ** 29, 2 ** 30, size=2 * (1 + 2 * 6)).astype(np.int32)
    ca, cb = np.zeros(6, np.int32), np.zeros(6, np.int32)
    ref.lib.ref_render_frame(ptr(cam), 40, 32, 6, ptr(seeds), 1.0, ptr(sc.points), ptr(sc.uvs), ptr(sc.normals),
                             ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds), ptr(env), ptr(lum),
                             ptr(sat), 256, 128, 1, ptr(acc_a), ptr(ca))
    orc.lib.or_render_frame(ptr(cam), 40, 32, 6, 0, 0, ptr(seeds), 1.0, ptr(sc.points), ptr(sc.uvs), ptr(sc.normals),
                            ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds), ptr(env), ptr(lum),
                            ptr(sat), 256, 128, 1, 0, ptr(acc_b), ptr(cb), None)
    assert ca[0] > 100 and np.array_equal(ca, cb)
    assert acc_a.tobytes() == acc_b.tobytes()


def test_sat_sampling_regions(orc, ref):
    """sampleContinuous / sampleDiscrete / getPdfSAT on sub-regions (SAT.cl:158-342)."""
    env = scenes.sky_env(64, 32)
    lum, sat = env_tables(orc, env, 64, 32)
    rng = np.random.default_rng(8)
    for k in range(300):
        x0, y0 = int(rng.integers(0, 48)), int(rng.integers(0, 24))
        reg = np.array([64, 32, x0, y0, int(rng.integers(1, 64 - x0 + 1)), int(rng.integers(1, 32 - y0 + 1))], np.int32)
        reg = np.array([64, 32, 0, 0, 64, 32], np.int32) if k % 3 == 0 else reg
        u = rng.random(2).astype(np.float32)
        outs = []
        for L, pre in ((ref.lib, "ref_"), (orc.lib, "or_")):
            uv, off, pdf = np.zeros(2, np.float32), np.zeros(2, np.int32), np.zeros(1, np.float32)
            getattr(L, pre + "sat_sample")(ptr(sat), ptr(lum), ptr(reg), float(u[0]), float(u[1]), ptr(uv), ptr(off),
                                           ptr(pdf))
            off2, pdf2 = np.zeros(2, np.int32), np.zeros(1, np.float32)
            getattr(L, pre + "sat_sample_discrete")(ptr(sat), ptr(lum), ptr(reg), float(u[0]), float(u[1]), ptr(off2),
                                                    ptr(pdf2))
            outs.append((uv, off, pdf, off2, pdf2))
        for a, b in zip(*outs):
            assert a.tobytes() == b.tobytes()
