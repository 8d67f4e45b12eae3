"""The CPU oracle against golden outputs of MambaTracer's own kernels.

tests/golden/ref_golden.npz holds outputs of the reference kernels (compiled as
C++ from src/cl/kernel/*.cl, see tests/golden/make_golden.py) on seeded inputs;
the restatement must reproduce them bit for bit.
"""
import numpy as np
import pytest

from mambatracer_gb300 import layout, scenes
from tests.golden.make_golden import bsdf_material, unit
from tests.helpers import bvh_build, ptr


def beq(a, b):
    return np.asarray(a).tobytes() == np.asarray(b).tobytes()


@pytest.fixture(scope="module")
def soup_bvh(orc, ginputs):
    nodes, bounds, depth, _ = bvh_build(orc, ginputs["soup"])
    return nodes, bounds


def test_bvh_is_the_golden_one(soup_bvh, golden):
    nodes, bounds = soup_bvh
    sha = np.frombuffer(nodes.tobytes() + bounds.tobytes(), np.uint8).sum(dtype=np.uint64)
    assert sha == golden["soup_nodes_sha"]


@pytest.mark.parametrize("key", ["rays_in", "rays_out"])
def test_intersect_primitives(orc, ginputs, golden, soup_bvh, key):
    """IntersectPrimitives (NormalBVH.cl:94-233): hit ids, t, full hit records."""
    sc = ginputs["soup"]
    nodes, bounds = soup_bvh
    rays = ginputs[key].copy()
    isects = np.zeros(rays.shape[0], layout.INTERSECTION)
    orc.lib.or_intersect(ptr(rays), ptr(isects), rays.shape[0], rays.shape[0], ptr(sc.points), ptr(sc.uvs),
                         ptr(sc.normals), ptr(sc.faces), sc.ntri, ptr(nodes), ptr(bounds), None)
    assert beq(rays["tMax"], golden[key + "_tmax"])
    ids = np.where(isects["hit"] == 1, isects["id"], -1)
    assert np.array_equal(ids, golden[key + "_id"])
    hit = isects["hit"] == 1
    g = golden[key + "_isect"]
    assert hit.sum() > 10
    for f in ("p", "n", "ng", "d", "uv", "mat"):
        assert beq(isects[f][hit], g[f][hit]), f


def test_occlusion(orc, ginputs, golden, soup_bvh):
    sc = ginputs["soup"]
    nodes, bounds = soup_bvh
    rays = ginputs["rays_shadow"]
    occ = np.zeros(rays.shape[0], np.int32)
    orc.lib.or_occlusion(ptr(rays), ptr(occ), rays.shape[0], ptr(sc.points), ptr(sc.faces), sc.ntri, ptr(nodes),
                         ptr(bounds), None)
    assert occ.sum() > 100
    assert np.array_equal(occ, golden["rays_shadow_occ"])


def test_raygen(orc, ginputs, golden):
    """InitCameraRayDataJitter (Initialize.cl:129-172)."""
    cam = ginputs["room"].camera.copy()
    rays = np.zeros(64 * 48, layout.RAY)
    seed = np.array([536870923, 805306457], np.int32)
    orc.lib.or_raygen(ptr(cam), ptr(rays), ptr(seed), 3.0, rays.shape[0], 0)
    assert beq(rays, golden["raygen_rays"])


def test_rng(orc, golden):
    """WangHash / generate_seed / get_random (Sampling.cl:15-59)."""
    assert [orc.lib.or_wanghash(i) for i in range(-50, 50)] == golden["wanghash"].tolist()
    r = np.zeros(64, np.float32)
    seed = np.array([536870923, 805306457], np.int32)
    orc.lib.or_random(ptr(seed), 2.0, 12345, 64, ptr(r))
    assert beq(r, golden["random_64"])


def test_bsdf(orc, ginputs, golden):
    """setupBsdf + SampleBsdf / EvaluateBsdf (Bsdf.cl:130-606), Lambert and GGX."""
    room = ginputs["room"]
    n4, d4, w4 = unit(ginputs["bsdf_n"]), unit(ginputs["bsdf_d"]), unit(ginputs["bsdf_w"])
    res = np.zeros((2000, 12), np.float32)
    ok = np.zeros((2000, 2), np.int32)
    for k in range(2000):
        m = bsdf_material(room, k, ginputs["bsdf_rough"][k])
        dirv, pdf, c, f, pr = (np.zeros(4, np.float32), np.zeros(1, np.float32), np.zeros(1, np.float32),
                               np.zeros(4, np.float32), np.zeros(2, np.float32))
        ok[k, 0] = orc.lib.or_bsdf_sample(ptr(m), ptr(n4[k]), ptr(n4[k]), ptr(d4[k]), ptr(ginputs["bsdf_s"][k]),
                                          ptr(dirv), ptr(pdf), ptr(c), ptr(f), ptr(pr))
        res[k, 0:4], res[k, 4], res[k, 5] = dirv, pdf[0], c[0]
        pdf2, c2, f2 = np.zeros(1, np.float32), np.zeros(1, np.float32), np.zeros(4, np.float32)
        ok[k, 1] = orc.lib.or_bsdf_eval(ptr(m), ptr(n4[k]), ptr(n4[k]), ptr(d4[k]), ptr(w4[k]), ptr(pdf2), ptr(c2),
                                        ptr(f2))
        res[k, 6:10], res[k, 10], res[k, 11] = f2, pdf2[0], c2[0]
    assert np.array_equal(ok, golden["bsdf_ok"])
    assert beq(res, golden["bsdf_res"])


def test_env_light(orc, ginputs, golden):
    """Env luminance + SAT (SAT.cl:304-311), illuminateEnvironmentLight (Light.cl:195-227),
    getRadianceEnvironmentLight (Light.cl:270-286)."""
    env = ginputs["env"]
    lum = np.zeros(128 * 64, np.float32)
    sat = np.zeros(128 * 64, np.float32)
    orc.lib.or_env_lum_sat(ptr(env), 128, 64, ptr(lum), ptr(sat))
    assert beq(lum, golden["env_lum"]) and beq(sat, golden["env_sat"])
    ill = np.zeros((2000, 9), np.float32)
    rad = np.zeros((2000, 5), np.float32)
    ed = unit(ginputs["env_d"])
    for k in range(2000):
        dirv, pdf, c = np.zeros(4, np.float32), np.zeros(1, np.float32), np.zeros(4, np.float32)
        orc.lib.or_env_illuminate(ptr(env), ptr(lum), ptr(sat), 128, 64, ptr(ginputs["env_s"][k]), ptr(dirv),
                                  ptr(pdf), ptr(c))
        ill[k, 0:4], ill[k, 4], ill[k, 5:9] = dirv, pdf[0], c
        pdf2, c2 = np.zeros(1, np.float32), np.zeros(4, np.float32)
        orc.lib.or_env_radiance(ptr(env), ptr(lum), ptr(sat), 128, 64, ptr(ed[k]), ptr(pdf2), ptr(c2))
        rad[k, 0], rad[k, 1:5] = pdf2[0], c2
    assert beq(ill, golden["env_illuminate"])
    assert beq(rad, golden["env_radiance"])


def test_lightgrid_sat_spike(orc, golden):
    """The one hand-checkable SAT in the reference's tests (test/lightgrid/TestSimpleGrid.java:39-67):
    a single 0.01 at (x=10, y=11) of a 16 x 16 grid; the SAT is 0.01 on x >= 10, y >= 11, else 0."""
    spike = np.zeros(256, np.float32)
    spike[11 * 16 + 10] = 0.01
    out = np.zeros(256, np.float32)
    orc.lib.or_lightgrid_sat(ptr(spike), ptr(out), 16, 16, 16, 16)
    expect = np.zeros((16, 16), np.float32)
    expect[11:, 10:] = np.float32(0.01)
    assert beq(out, expect.ravel())
    assert beq(out, golden["spike_sat"])


def test_lightgrid_sat_random(orc, ginputs, golden):
    out = np.zeros(64 * 64, np.float32)
    orc.lib.or_lightgrid_sat(ptr(ginputs["grid_func"]), ptr(out), 64, 64, 16, 32)
    assert beq(out, golden["grid_sat"])


def test_prefix_sum_fixture(golden):
    """PrefixSumIntegerTest (test/algorithm/PrefixSumIntegerTest.java:22-38): 200 ones scan to
    0..199 with total 200 (lane 0 of each group reads aux[-1], taken as 0)."""
    assert golden["scan200_out"].tolist() == list(range(200))
    assert int(golden["scan200_total"]) == 200


def test_light_list(orc, ginputs, golden):
    room = ginputs["room"]
    lf = np.zeros(room.ntri, np.int32)
    n = orc.lib.or_light_list(ptr(room.faces), room.ntri, ptr(room.materials), ptr(lf))
    assert n == int(golden["room_lights"]) == 2
    info = golden["room_light_info"].reshape(-1, 2)
    assert lf[:n].tolist() == info[:, 0].tolist()
    assert (info[:, 1] == 1).all()  # AREA_LIGHT


def test_frames(orc, ginputs, golden):
    """Two GI frames (CDeviceGI.loop restated) on the box room: film and queue lengths."""
    from tests.helpers import oracle_frames
    room = ginputs["room"]
    nodes, bounds, _, _ = bvh_build(orc, room)
    acc, counts, _ = oracle_frames(orc, room, nodes, bounds, 64, 48, 4, 0, 0, list(ginputs["frame_seeds"]))
    assert np.array_equal(counts, golden["frame_counts"])
    assert beq(acc, golden["frame_accum"])


def test_grid_guided_env_light(orc, ginputs, golden):
    """Grid versions of the environment light (illuminateEnvironmentLight1,
    getRadianceEnvironmentLight1, Light.cl:140-268) on a 64 x 64 grid of 4 x 2 cells of
    16 x 32 tiles over the 128 x 64 map: direction, radiance, the grid entry (cell, tile)
    and the accumulated luminance equal the reference's; the tile-local pdf factor equals
    the reference's pdf (the oracle's direction pdf also carries the tile density)."""
    from tests.golden.make_golden import GRID_CAM
    env = ginputs["env"]
    lum, sat = golden["env_lum"], golden["env_sat"]
    func, gsat = ginputs["grid_func"], golden["grid_sat"]
    gill, grad = golden["grid_illuminate"], golden["grid_radiance"]
    for k in range(500):
        p4 = np.append(ginputs["grid_p"][k], 0.0).astype(np.float32)
        d, pdf, pref, c, gi = (np.zeros(4, np.float32), np.zeros(1, np.float32), np.zeros(1, np.float32),
                               np.zeros(4, np.float32), np.zeros(1, np.int32))
        orc.lib.or_env_grid_illuminate(ptr(env), ptr(lum), ptr(sat), 128, 64, ptr(func), ptr(gsat), 64, 64, 16, 32,
                                       ptr(GRID_CAM), ptr(p4), ptr(ginputs["grid_s"][k]), ptr(d), ptr(pdf), ptr(pref),
                                       ptr(c), ptr(gi))
        assert beq(d, gill[k, 0:4]) and beq(c, gill[k, 5:9]), k
        assert beq(pref, gill[k, 4:5]), k
        assert gi[0] == int(gill[k, 10]), k
        pdf2, c2, gi2, acc = (np.zeros(1, np.float32), np.zeros(4, np.float32), np.zeros(1, np.int32),
                              np.zeros(1, np.float32))
        orc.lib.or_env_grid_radiance(ptr(env), ptr(lum), ptr(sat), 128, 64, ptr(func), ptr(gsat), 64, 64, 16, 32,
                                     ptr(GRID_CAM), ptr(p4), ptr(d), ptr(pdf2), ptr(c2), ptr(gi2), ptr(acc))
        assert beq(c2, grad[k, 1:5]) and gi2[0] == int(grad[k, 5]) and beq(acc, grad[k, 6:7]), k


def test_tonemap(orc, ginputs, golden):
    """CImage.processImage (Image.cl:29-118, RGBSpace.cl:9-106): averageAccum's log
    luminance and predicate per pixel, and updateFrameImage's ARGB (Reinhard through xyY,
    gamma 2.2, exposure 0.18) given the exact log-luminance total; zero pixels keep the
    initial opaque black."""
    film = ginputs["tone_film"]
    n = film.shape[0]
    argb = np.full(n, -16777216, np.int32)
    fb = np.zeros_like(film)
    tot = np.zeros(2, np.float32)
    orc.lib.or_tonemap(ptr(film), n, 7.0, 0.18, 2.2, ptr(argb), ptr(fb), ptr(tot))
    loglw = golden["tone_loglw"]
    assert tot[1] == golden["tone_count"].sum()
    assert tot[0] == np.float32(loglw.astype(np.float64).sum())
    assert beq(argb, golden["tone_argb"])


def test_preview_frame(orc, ginputs, golden):
    """The preview device's frame (Raytrace.cl) of the room: ARGB and material group per pixel."""
    from oracle.oracle import bvh_build
    room = ginputs["room"]
    rn, rb, _, _ = bvh_build(orc, room)
    z = np.zeros(4, np.float32)
    argb = np.zeros(64 * 48, np.int32)
    group = np.zeros(64 * 48, np.int32)
    orc.lib.or_preview(ptr(room.camera), 64, 48, ptr(room.points), ptr(room.uvs), ptr(room.normals), ptr(room.faces),
                       room.ntri, ptr(room.materials), ptr(rn), ptr(rb), ptr(z), 1, 1, 0, ptr(argb), ptr(group))
    assert beq(argb, golden["preview_argb"]) and beq(group, golden["preview_group"])


def test_texture_pass(orc, ginputs, golden):
    """texturePassGI + CTextureApplyPass.process + updateToTextureColorGI
    (Render.cl:127-231) on 600 flagged materials and uvs (tiled, negative, NaN,
    infinite): the material after the pass."""
    from tests.golden.make_golden import texture_material
    tr = ginputs["tex_room"]
    texels, table = scenes.texture_tables(tr)
    out = np.zeros_like(golden["tex_material_out"])
    for i in range(out.shape[0]):
        m = texture_material(ginputs, i)
        orc.lib.or_texture_apply(ptr(m), int(ginputs["tex_mat"][i]), float(ginputs["tex_u"][i]),
                                 float(ginputs["tex_v"][i]), ptr(texels), ptr(table), table.shape[0], ptr(out[i]))
    assert beq(out, golden["tex_material_out"])


def test_textured_frame(orc, ginputs, golden):
    """A depth-6 frame of the textured room (CDeviceGI.loop with its texture pass):
    film and queue lengths."""
    from oracle.oracle import bvh_build
    tr = ginputs["tex_room"]
    texels, table = scenes.texture_tables(tr)
    tn, tb, _, _ = bvh_build(orc, tr)
    z = np.zeros(4, np.float32)
    acc = np.zeros((40 * 32, 4), np.float32)
    c = np.zeros(6, np.int32)
    orc.lib.or_set_textures(ptr(texels), ptr(table), table.shape[0])
    try:
        orc.lib.or_render_frame(ptr(tr.camera), 40, 32, 6, 0, 0, ptr(ginputs["tex_seeds"]), 1.0, ptr(tr.points),
                                ptr(tr.uvs), ptr(tr.normals), ptr(tr.faces), tr.ntri, ptr(tr.materials), ptr(tn),
                                ptr(tb), ptr(z), ptr(z), ptr(z), 1, 1, 0, 0, ptr(acc), ptr(c), None)
    finally:
        orc.lib.or_set_textures(None, None, 0)
    assert beq(c, golden["tex_frame_counts"])
    assert beq(acc, golden["tex_frame_accum"])


def test_textured_preview_frame(orc, ginputs, golden):
    """The preview frame of the textured room with the preview's texture pass
    (textureInitPassRT, CTextureApplyPass.process, updateToTextureColorRT)."""
    from oracle.oracle import bvh_build
    tr = ginputs["tex_room"]
    texels, table = scenes.texture_tables(tr)
    tn, tb, _, _ = bvh_build(orc, tr)
    z = np.zeros(4, np.float32)
    argb = np.zeros(40 * 32, np.int32)
    group = np.zeros(40 * 32, np.int32)
    orc.lib.or_set_textures(ptr(texels), ptr(table), table.shape[0])
    try:
        orc.lib.or_preview(ptr(tr.camera), 40, 32, ptr(tr.points), ptr(tr.uvs), ptr(tr.normals), ptr(tr.faces),
                           tr.ntri, ptr(tr.materials), ptr(tn), ptr(tb), ptr(z), 1, 1, 0, ptr(argb), ptr(group))
    finally:
        orc.lib.or_set_textures(None, None, 0)
    assert beq(argb, golden["tex_preview_argb"]) and beq(group, golden["tex_preview_group"])
