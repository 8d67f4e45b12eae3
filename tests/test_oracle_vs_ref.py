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


def test_frame_stadium_with_env(orc, ref):
    """The plane + icosphere scene (shared edges on the plane, a dense cluster on it)."""
    sc = scenes.stadium(quads=40, level=3, width=48, height=32)
    nodes, bounds, depth, _ = bvh_build(orc, sc)
    env = scenes.sky_env(256, 128)
    lum, sat = env_tables(orc, env, 256, 128)
    cam = sc.camera.copy()
    acc_a = np.zeros((48 * 32, 4), np.float32)
    acc_b = acc_a.copy()
    seeds = np.random.default_rng(4).integers(2 ** 29, 2 ** 30, size=2 * (1 + 2 * 6)).astype(np.int32)
    ca, cb = np.zeros(6, np.int32), np.zeros(6, np.int32)
    ref.lib.ref_render_frame(ptr(cam), 48, 32, 6, ptr(seeds), 1.0, ptr(sc.points), ptr(sc.uvs), ptr(sc.normals),
                             ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds), ptr(env), ptr(lum),
                             ptr(sat), 256, 128, 1, ptr(acc_a), ptr(ca))
    orc.lib.or_render_frame(ptr(cam), 48, 32, 6, 0, 0, ptr(seeds), 1.0, ptr(sc.points), ptr(sc.uvs), ptr(sc.normals),
                            ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds), ptr(env), ptr(lum),
                            ptr(sat), 256, 128, 1, 0, ptr(acc_b), ptr(cb), None)
    assert ca[0] > 500 and np.array_equal(ca, cb)
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


def test_grid_guided_env_pieces(orc, ref):
    """The grid versions of the environment light (illuminateEnvironmentLight1,
    getRadianceEnvironmentLight1, Light.cl:140-268): cell, tile, texel, direction,
    radiance and accumulation index equal the reference's; the direction pdf is the
    reference's times the tile density pdfLL (left out in the reference), so the
    tile-local factor is compared against the reference's pdf."""
    from tests.helpers import oracle_grid
    w, h, nu, nv, rx, ry = 512, 256, 320, 320, 16, 32
    env = scenes.sky_env(w, h)
    lum, sat = env_tables(orc, env, w, h)
    func, gsat = oracle_grid(orc, (env, w, h), nu, nv, rx, ry)
    rng = np.random.default_rng(7)
    # make the cells differ: scale each cell's tiles by a random factor, zero a few tiles
    cells = rng.uniform(0.2, 3.0, size=(nv // ry, nu // rx))
    func = (func.reshape(nv // ry, ry, nu // rx, rx) * cells[:, None, :, None].astype(np.float32)).reshape(-1)
    func[rng.choice(func.size, 2000, replace=False)] = 0.0
    func = np.ascontiguousarray(func, np.float32)
    orc.lib.or_lightgrid_sat(ptr(func), ptr(gsat), nu, nv, rx, ry)
    cam = np.array([0.1, 0.2, 2.5, 0.0], np.float32)
    n_pdf = 0
    for k in range(400):
        p = np.append(rng.uniform(-1, 1, 3), 0.0).astype(np.float32)
        s4 = rng.random(4).astype(np.float32)
        out = {}
        for name, lib, fn in (("ref", ref.lib, "ref_env_grid_illuminate"), ("or", orc.lib, "or_env_grid_illuminate")):
            d = np.zeros(4, np.float32)
            c = np.zeros(4, np.float32)
            pdf = np.zeros(1, np.float32)
            extra = np.zeros(1, np.float32)
            gi = np.zeros(1, np.int32)
            if name == "ref":
                getattr(lib, fn)(ptr(env), ptr(lum), ptr(sat), w, h, ptr(func), ptr(gsat), nu, nv, rx, ry, ptr(cam),
                                 ptr(p), ptr(s4), ptr(d), ptr(pdf), ptr(c), ptr(extra), ptr(gi))
                out[name] = (d, pdf[0], c, gi[0])
            else:
                getattr(lib, fn)(ptr(env), ptr(lum), ptr(sat), w, h, ptr(func), ptr(gsat), nu, nv, rx, ry, ptr(cam),
                                 ptr(p), ptr(s4), ptr(d), ptr(pdf), ptr(extra), ptr(c), ptr(gi))
                out[name] = (d, extra[0], c, gi[0], pdf[0])
        r, o = out["ref"], out["or"]
        if o[4] == 0.0:
            continue  # an empty tile: the oracle gives no light sample, the reference divides by zero
        n_pdf += 1
        assert r[3] == o[3]
        assert r[0].tobytes() == o[0].tobytes()
        assert r[2].tobytes() == o[2].tobytes()
        assert np.float32(r[1]).tobytes() == np.float32(o[1]).tobytes()
        # radiance from the same point along the sampled direction: same tile, accumulation entry
        pdf = np.zeros(1, np.float32)
        c = np.zeros(4, np.float32)
        gi = np.zeros(1, np.int32)
        acc = np.zeros(1, np.float32)
        ref.lib.ref_env_grid_radiance(ptr(env), ptr(lum), ptr(sat), w, h, ptr(func), ptr(gsat), nu, nv, rx, ry,
                                      ptr(cam), ptr(p), ptr(o[0]), ptr(pdf), ptr(c), ptr(gi), ptr(acc))
        pdf2 = np.zeros(1, np.float32)
        c2 = np.zeros(4, np.float32)
        gi2 = np.zeros(1, np.int32)
        acc2 = np.zeros(1, np.float32)
        orc.lib.or_env_grid_radiance(ptr(env), ptr(lum), ptr(sat), w, h, ptr(func), ptr(gsat), nu, nv, rx, ry,
                                     ptr(cam), ptr(p), ptr(o[0]), ptr(pdf2), ptr(c2), ptr(gi2), ptr(acc2))
        assert c.tobytes() == c2.tobytes()
        assert gi[0] == gi2[0] and acc[0] == acc2[0]
        # the sampled direction's pdf equals its evaluated pdf once each is multiplied by its
        # sine term (sampling: the continuous v of the sample; evaluation: the texel row's top)
        v = np.arccos(np.clip(np.float64(o[0][1]), -1, 1)) / np.pi
        y = int(v * h)
        if y > 0:  # row 0's sine term is 0: the evaluated pdf is infinite, as in the full-map version
            a, b = pdf2[0] * np.sin(y / h * np.pi), o[4] * np.sin(v * np.pi)
            assert abs(a - b) <= 1e-3 * b
    assert n_pdf > 300


def test_tonemap_frame(orc, ref):
    """The ARGB image of a rendered box-room film: oracle == reference per-pixel kernels."""
    from tests.helpers import oracle_frames
    sc = scenes.box_room(64, 48)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    acc, _, _ = oracle_frames(orc, sc, nodes, bounds, 64, 48, 4, 1, 3, [None] * 3)
    n = acc.shape[0]
    argb = np.full(n, -16777216, np.int32)
    tot = np.zeros(2, np.float32)
    orc.lib.or_tonemap(ptr(acc), n, 3.0, 0.18, 2.2, ptr(argb), None, ptr(tot))
    fb = np.zeros_like(acc)
    loglw = np.zeros(n, np.float32)
    cnt = np.zeros(n, np.int32)
    ref.lib.ref_average_accum(ptr(acc), 3.0, n, ptr(fb), ptr(loglw), ptr(cnt))
    assert tot[0] == np.float32(loglw.astype(np.float64).sum()) and tot[1] == cnt.sum()
    rargb = np.full(n, -16777216, np.int32)
    ref.lib.ref_update_frame_image(ptr(fb), ptr(rargb), float(tot[0]), int(cnt.sum()), n, 0.18, 2.2)
    assert cnt.sum() > n // 2
    assert argb.tobytes() == rargb.tobytes()


@pytest.mark.parametrize("which", ["room", "tex_room", "soup_env"])
def test_preview_frame(orc, ref, which):
    """The preview device's frame (Raytrace.cl, with its texture pass on the
    textured room): ARGB and material group per pixel."""
    if which == "room":
        sc, W, H, env = scenes.box_room(64, 48), 64, 48, None
    elif which == "tex_room":
        sc, W, H, env = scenes.textured_room(64, 48), 64, 48, None
    else:
        sc, W, H = scenes.soup(20000, seed=7, extent=0.8, edge_sigma=0.02), 64, 48
        env = scenes.sky_env(256, 128)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    envmap = env if env is not None else np.zeros((1, 4), np.float32)
    ew, eh = (256, 128) if env is not None else (1, 1)
    out = {}
    texels, table = scenes.texture_tables(sc)
    ntab = table.shape[0] if sc.textures else 0
    for name, lib, fn, st in (("ref", ref.lib, "ref_preview", "ref_set_textures"),
                              ("or", orc.lib, "or_preview", "or_set_textures")):
        argb = np.zeros(W * H, np.int32)
        group = np.zeros(W * H, np.int32)
        getattr(lib, st)(ptr(texels), ptr(table), ntab)
        try:
            getattr(lib, fn)(ptr(sc.camera), W, H, ptr(sc.points), ptr(sc.uvs), ptr(sc.normals), ptr(sc.faces),
                             sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds), ptr(envmap), ew, eh,
                             int(env is not None), ptr(argb), ptr(group))
        finally:
            getattr(lib, st)(None, None, 0)
        out[name] = (argb, group)
    assert out["ref"][1].tobytes() == out["or"][1].tobytes()
    assert out["ref"][0].tobytes() == out["or"][0].tobytes()
    assert (out["or"][1] >= 0).sum() > W * H // 4 and np.unique(out["or"][0]).size > 20


def _texture_cases(seed, n):
    """Materials with random texture flags and uvs: in [0, 1], tiled, negative,
    integers, tiny negatives, NaN and infinities."""
    rng = np.random.default_rng(seed)
    sc = scenes.textured_room()
    texels, table = scenes.texture_tables(sc)
    u = rng.uniform(-3, 3, n).astype(np.float32)
    v = rng.uniform(-3, 3, n).astype(np.float32)
    special = np.array([0, 1, -1, 2, -2, 0.5, -0.5, 1e-9, -1e-9, 0.99999994, -0.99999994, 3e9, -3e9,
                        np.nan, np.inf, -np.inf], np.float32)
    u[:special.size] = special
    v[:special.size] = special[::-1]
    mats = rng.integers(0, sc.materials.shape[0], n)
    flags = rng.integers(0, 2, (n, 3))
    return sc, texels, table, u, v, mats, flags


@pytest.mark.parametrize("seed", [51, 52])
def test_texture_pass(orc, ref, seed):
    """texturePassGI + CTextureApplyPass.process + updateToTextureColorGI
    (Render.cl:127-231) on one path: the oracle's material after the pass equals
    the reference kernels' byte for byte."""
    sc, texels, table, u, v, mats, flags = _texture_cases(seed, 4000)
    for i in range(len(u)):
        m = sc.materials[mats[i]:mats[i] + 1].copy()
        m["isDiffuseTexture"], m["isGlossyTexture"], m["isRoughnessTexture"] = flags[i]
        a = np.zeros(36, np.float32)
        b = np.zeros(36, np.float32)
        ref.lib.ref_texture_apply(ptr(m), int(mats[i]), float(u[i]), float(v[i]), ptr(texels), ptr(table),
                                  table.shape[0], ptr(a))
        orc.lib.or_texture_apply(ptr(m), int(mats[i]), float(u[i]), float(v[i]), ptr(texels), ptr(table),
                                 table.shape[0], ptr(b))
        assert a.tobytes() == b.tobytes(), (i, u[i], v[i], flags[i])


@pytest.mark.parametrize("depth", [4, 8])
def test_textured_frame(orc, ref, depth):
    """CDeviceGI.loop with the texture pass on the textured box room: film and
    queue lengths bit-identical."""
    sc = scenes.textured_room(40, 32)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    texels, table = scenes.texture_tables(sc)
    rng = np.random.default_rng(depth + 7)
    seeds = rng.integers(2 ** 29, 2 ** 30, size=2 * (1 + 2 * depth)).astype(np.int32)
    cam = sc.camera.copy()
    acc_a = np.zeros((40 * 32, 4), np.float32)
    acc_b = acc_a.copy()
    acc_c = acc_a.copy()
    z = np.zeros(4, np.float32)
    ca, cb = np.zeros(depth, np.int32), np.zeros(depth, np.int32)
    ref.lib.ref_set_textures(ptr(texels), ptr(table), table.shape[0])
    orc.lib.or_set_textures(ptr(texels), ptr(table), table.shape[0])
    try:
        ref.lib.ref_render_frame(ptr(cam), 40, 32, depth, ptr(seeds), 1.0, ptr(sc.points), ptr(sc.uvs),
                                 ptr(sc.normals), ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds),
                                 ptr(z), ptr(z), ptr(z), 1, 1, 0, ptr(acc_a), ptr(ca))
        orc.lib.or_render_frame(ptr(cam), 40, 32, depth, 0, 0, ptr(seeds), 1.0, ptr(sc.points), ptr(sc.uvs),
                                ptr(sc.normals), ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds),
                                ptr(z), ptr(z), ptr(z), 1, 1, 0, 0, ptr(acc_b), ptr(cb), None)
    finally:
        ref.lib.ref_set_textures(None, None, 0)
        orc.lib.or_set_textures(None, None, 0)
    assert np.array_equal(ca, cb)
    assert acc_a.tobytes() == acc_b.tobytes()
    # the textures change the image
    orc.lib.or_render_frame(ptr(cam), 40, 32, depth, 0, 0, ptr(seeds), 1.0, ptr(sc.points), ptr(sc.uvs),
                            ptr(sc.normals), ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds),
                            ptr(z), ptr(z), ptr(z), 1, 1, 0, 0, ptr(acc_c), None, None)
    assert (np.abs(acc_c - acc_b).max(axis=1) > 1e-3).sum() > 100
