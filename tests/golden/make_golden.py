"""Generate tests/golden/ref_golden.npz from MambaTracer's own kernels.

Runs the reference kernels compiled as C++ (oracle/_ref/libmtref.so, built by
oracle/ref/make_ref.py from the MambaTracer sources) on seeded inputs and stores
their outputs. The reference tree is only present where the fixtures are made;
the tests read the .npz. Inputs are regenerated from the same seeds by the tests.

  python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from mambatracer_gb300 import layout, scenes  # noqa: E402
from oracle.oracle import Oracle, RefOracle, bvh_build, ptr  # noqa: E402
from oracle.ref import make_ref  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_golden.npz")


def golden_inputs():
    """Seeded inputs shared by the generator and the tests."""
    g = {}
    g["soup"] = scenes.soup(30000, seed=21)
    o, d = scenes.random_rays(g["soup"], 20000, seed=22, inside=True)
    g["rays_in"] = layout.make_rays(o, d)
    o, d = scenes.random_rays(g["soup"], 5000, seed=23, inside=False)
    g["rays_out"] = layout.make_rays(o, d)
    o, d = scenes.random_rays(g["soup"], 20000, seed=24, inside=True)
    g["rays_shadow"] = layout.make_rays(o, d, tmin=1e-4, tmax=0.35)
    g["room"] = scenes.box_room(64, 48)
    g["env"] = scenes.sky_env(128, 64)
    rng = np.random.default_rng(25)
    g["bsdf_n"] = rng.normal(size=(2000, 3))
    g["bsdf_d"] = rng.normal(size=(2000, 3))
    g["bsdf_w"] = rng.normal(size=(2000, 3))
    g["bsdf_s"] = rng.random((2000, 3)).astype(np.float32)
    g["bsdf_rough"] = rng.uniform(0.02, 0.9, size=(2000, 2)).astype(np.float32)
    g["env_s"] = rng.random((2000, 4)).astype(np.float32)
    g["env_d"] = rng.normal(size=(2000, 3))
    g["grid_func"] = rng.random(64 * 64).astype(np.float32)
    g["scan_in"] = (rng.random(1000) < 0.3).astype(np.int32)
    g["frame_seeds"] = rng.integers(2 ** 29, 2 ** 30, size=(2, 2 * (1 + 2 * 4))).astype(np.int32)
    g["grid_p"] = rng.uniform(-1, 1, size=(500, 3))
    g["grid_s"] = rng.random((500, 4)).astype(np.float32)
    film = (rng.exponential(1.0, size=(64 * 48, 4)) * rng.choice([0.0, 0.3, 3.0, 40.0], size=(64 * 48, 1)))
    film[:, 3] = 7.0
    g["tone_film"] = film.astype(np.float32)
    # texture pass: the textured room's images, materials with random texture
    # flags, uvs in and beyond [0, 1] plus the special values
    g["tex_room"] = scenes.textured_room(40, 32)
    n = 600
    u = rng.uniform(-3, 3, n).astype(np.float32)
    v = rng.uniform(-3, 3, n).astype(np.float32)
    special = np.array([0, 1, -1, 2, -2, 0.5, -0.5, 1e-9, -1e-9, 0.99999994, -0.99999994, 3e9, -3e9,
                        np.nan, np.inf, -np.inf], np.float32)
    u[:special.size] = special
    v[:special.size] = special[::-1]
    g["tex_u"], g["tex_v"] = u, v
    g["tex_mat"] = rng.integers(0, g["tex_room"].materials.shape[0], n).astype(np.int32)
    g["tex_flags"] = rng.integers(0, 2, (n, 3)).astype(np.int32)
    g["tex_seeds"] = rng.integers(2 ** 29, 2 ** 30, size=2 * (1 + 2 * 6)).astype(np.int32)
    return g


def texture_material(g, i):
    """Golden texture case i: its material (one MATERIAL record) with the case's flags."""
    m = g["tex_room"].materials[g["tex_mat"][i]:g["tex_mat"][i] + 1].copy()
    m["isDiffuseTexture"], m["isGlossyTexture"], m["isRoughnessTexture"] = g["tex_flags"][i]
    return m


GRID_CAM = np.array([0.1, 0.2, 2.5, 0.0], np.float32)


def unit(v):
    v = np.asarray(v, np.float64)
    v = v / np.linalg.norm(v, axis=-1, keepdims=True)
    out = np.zeros(v.shape[:-1] + (4,), np.float32)
    out[..., :3] = v
    return out


def bsdf_material(room, k, rough):
    m = room.materials[3:4].copy()  # GGX over grey
    if k % 2 == 0:
        m = room.materials[0:1].copy()  # pure Lambert
    m["glossy_param"][0, 1] = rough[0]
    m["glossy_param"][0, 2] = rough[1]
    return m


def main():
    make_ref.build()
    ref = RefOracle()
    orc = Oracle()
    g = golden_inputs()
    out = {}
    soup = g["soup"]
    nodes, bounds, depth, _ = bvh_build(orc, soup)
    out["soup_nodes_sha"] = np.frombuffer(nodes.tobytes() + bounds.tobytes(), np.uint8).sum(dtype=np.uint64)
    for key in ("rays_in", "rays_out"):
        rays = g[key].copy()
        isects = np.zeros(rays.shape[0], layout.INTERSECTION)
        ref.lib.ref_intersect(ptr(rays), ptr(isects), rays.shape[0], rays.shape[0], ptr(soup.points), ptr(soup.uvs),
                              ptr(soup.normals), ptr(soup.faces), soup.ntri, ptr(nodes), ptr(bounds))
        out[key + "_tmax"] = rays["tMax"].copy()
        out[key + "_id"] = np.where(isects["hit"] == 1, isects["id"], -1).astype(np.int32)
        out[key + "_isect"] = isects
    rays = g["rays_shadow"].copy()
    occ = np.zeros(rays.shape[0], np.int32)
    ref.lib.ref_occlusion(ptr(rays), ptr(occ), rays.shape[0], ptr(soup.points), ptr(soup.uvs), ptr(soup.normals),
                          ptr(soup.faces), soup.ntri, ptr(nodes), ptr(bounds))
    out["rays_shadow_occ"] = occ

    room = g["room"]
    cam = room.camera.copy()
    rays = np.zeros(64 * 48, layout.RAY)
    seed = np.array([536870923, 805306457], np.int32)
    ref.lib.ref_raygen(ptr(cam), ptr(rays), ptr(seed), 3.0, rays.shape[0])
    out["raygen_rays"] = rays

    r = np.zeros(64, np.float32)
    ref.lib.ref_random(ptr(seed), 2.0, 12345, 64, ptr(r))
    out["random_64"] = r
    out["wanghash"] = np.array([ref.lib.ref_wanghash(int(i)) for i in range(-50, 50)], np.uint32)

    n4, d4, w4 = unit(g["bsdf_n"]), unit(g["bsdf_d"]), unit(g["bsdf_w"])
    res = np.zeros((2000, 12), np.float32)
    ok = np.zeros((2000, 2), np.int32)
    for k in range(2000):
        m = bsdf_material(room, k, g["bsdf_rough"][k])
        dirv, pdf, c, f, pr = (np.zeros(4, np.float32), np.zeros(1, np.float32), np.zeros(1, np.float32),
                               np.zeros(4, np.float32), np.zeros(2, np.float32))
        ok[k, 0] = ref.lib.ref_bsdf_sample(ptr(m), ptr(n4[k]), ptr(n4[k]), ptr(d4[k]), ptr(g["bsdf_s"][k]), ptr(dirv),
                                           ptr(pdf), ptr(c), ptr(f), ptr(pr))
        res[k, 0:4], res[k, 4], res[k, 5] = dirv, pdf[0], c[0]
        pdf2, c2, f2 = np.zeros(1, np.float32), np.zeros(1, np.float32), np.zeros(4, np.float32)
        ok[k, 1] = ref.lib.ref_bsdf_eval(ptr(m), ptr(n4[k]), ptr(n4[k]), ptr(d4[k]), ptr(w4[k]), ptr(pdf2), ptr(c2),
                                         ptr(f2))
        res[k, 6:10], res[k, 10], res[k, 11] = f2, pdf2[0], c2[0]
    out["bsdf_res"] = res
    out["bsdf_ok"] = ok

    env = g["env"]
    lum = np.zeros(128 * 64, np.float32)
    sat = np.zeros(128 * 64, np.float32)
    ref.lib.ref_env_lum_sat(ptr(env), 128, 64, ptr(lum), ptr(sat))
    out["env_lum"], out["env_sat"] = lum, sat
    ill = np.zeros((2000, 9), np.float32)
    ed = unit(g["env_d"])
    rad = np.zeros((2000, 5), np.float32)
    for k in range(2000):
        dirv, pdf, c = np.zeros(4, np.float32), np.zeros(1, np.float32), np.zeros(4, np.float32)
        ref.lib.ref_env_illuminate(ptr(env), ptr(lum), ptr(sat), 128, 64, ptr(g["env_s"][k]), ptr(dirv), ptr(pdf),
                                   ptr(c))
        ill[k, 0:4], ill[k, 4], ill[k, 5:9] = dirv, pdf[0], c
        pdf2, c2 = np.zeros(1, np.float32), np.zeros(4, np.float32)
        ref.lib.ref_env_radiance(ptr(env), ptr(lum), ptr(sat), 128, 64, ptr(ed[k]), ptr(pdf2), ptr(c2))
        rad[k, 0], rad[k, 1:5] = pdf2[0], c2
    out["env_illuminate"] = ill
    out["env_radiance"] = rad

    spike = np.zeros(256, np.float32)
    spike[11 * 16 + 10] = 0.01  # test/lightgrid/TestSimpleGrid.java:39-57
    s16 = np.zeros(256, np.float32)
    ref.lib.ref_lightgrid_sat(ptr(spike), ptr(s16), 16, 16, 16, 16)
    out["spike_sat"] = s16
    gs = np.zeros(64 * 64, np.float32)
    ref.lib.ref_lightgrid_sat(ptr(g["grid_func"]), ptr(gs), 64, 64, 16, 32)
    out["grid_sat"] = gs

    # grid versions of the environment light on the 64 x 64 grid (4 x 2 cells of 16 x 32 tiles)
    gill = np.zeros((500, 11), np.float32)
    grad = np.zeros((500, 7), np.float32)
    for k in range(500):
        p4 = np.append(g["grid_p"][k], 0.0).astype(np.float32)
        dirv, pdf, c = np.zeros(4, np.float32), np.zeros(1, np.float32), np.zeros(4, np.float32)
        lv, gi = np.zeros(1, np.float32), np.zeros(1, np.int32)
        ref.lib.ref_env_grid_illuminate(ptr(env), ptr(lum), ptr(sat), 128, 64, ptr(g["grid_func"]), ptr(gs), 64, 64,
                                        16, 32, ptr(GRID_CAM), ptr(p4), ptr(g["grid_s"][k]), ptr(dirv), ptr(pdf),
                                        ptr(c), ptr(lv), ptr(gi))
        gill[k, 0:4], gill[k, 4], gill[k, 5:9], gill[k, 9], gill[k, 10] = dirv, pdf[0], c, lv[0], gi[0]
        pdf2, c2, gi2, acc = np.zeros(1, np.float32), np.zeros(4, np.float32), np.zeros(1, np.int32), \
            np.zeros(1, np.float32)
        ref.lib.ref_env_grid_radiance(ptr(env), ptr(lum), ptr(sat), 128, 64, ptr(g["grid_func"]), ptr(gs), 64, 64, 16,
                                      32, ptr(GRID_CAM), ptr(p4), ptr(dirv), ptr(pdf2), ptr(c2), ptr(gi2), ptr(acc))
        grad[k, 0], grad[k, 1:5], grad[k, 5], grad[k, 6] = pdf2[0], c2, gi2[0], acc[0]
    out["grid_illuminate"] = gill
    out["grid_radiance"] = grad

    # CImage.processImage per-pixel kernels on a 7-frame film, with the exact totals
    film = g["tone_film"]
    fb = np.zeros_like(film)
    loglw = np.zeros(film.shape[0], np.float32)
    cnt = np.zeros(film.shape[0], np.int32)
    ref.lib.ref_average_accum(ptr(film), 7.0, film.shape[0], ptr(fb), ptr(loglw), ptr(cnt))
    total = np.float32(loglw.astype(np.float64).sum())
    argb = np.full(film.shape[0], -16777216, np.int32)  # InitIntDataRGB: opaque black
    ref.lib.ref_update_frame_image(ptr(fb), ptr(argb), float(total), int(cnt.sum()), film.shape[0], 0.18, 2.2)
    out["tone_loglw"], out["tone_count"], out["tone_argb"] = loglw, cnt, argb

    sc_out = np.zeros(1000, np.int32)
    total = ref.lib.ref_scan_int(ptr(g["scan_in"]), 1000, ptr(sc_out), 128)
    out["scan_out"], out["scan_total"] = sc_out, np.int32(total)
    ones = np.ones(200, np.int32)
    o200 = np.zeros(200, np.int32)
    t200 = ref.lib.ref_scan_int(ptr(ones), 200, ptr(o200), 128)  # test/algorithm/PrefixSumIntegerTest.java:22-38
    out["scan200_out"], out["scan200_total"] = o200, np.int32(t200)

    lf = np.zeros(2 * room.ntri, np.int32)
    out["room_lights"] = np.int32(ref.lib.ref_light_list(ptr(room.faces), room.ntri, ptr(room.materials), ptr(lf)))
    out["room_light_info"] = lf[: 2 * int(out["room_lights"])]

    rn, rb, _, _ = bvh_build(orc, room)
    acc = np.zeros((64 * 48, 4), np.float32)
    counts = []
    z = np.zeros(4, np.float32)
    for f in range(2):
        c = np.zeros(4, np.int32)
        ref.lib.ref_render_frame(ptr(cam), 64, 48, 4, ptr(g["frame_seeds"][f]), float(f + 1), ptr(room.points),
                                 ptr(room.uvs), ptr(room.normals), ptr(room.faces), room.ntri, ptr(room.materials),
                                 ptr(rn), ptr(rb), ptr(z), ptr(z), ptr(z), 1, 1, 0, ptr(acc), ptr(c))
        counts.append(c)
    out["frame_accum"] = acc
    out["frame_counts"] = np.stack(counts)
    # the preview device's frame of the room (Raytrace.cl): ARGB and material group
    pa = np.zeros(64 * 48, np.int32)
    pg = np.zeros(64 * 48, np.int32)
    ref.lib.ref_preview(ptr(cam), 64, 48, ptr(room.points), ptr(room.uvs), ptr(room.normals), ptr(room.faces),
                        room.ntri, ptr(room.materials), ptr(rn), ptr(rb), ptr(z), 1, 1, 0, ptr(pa), ptr(pg))
    out["preview_argb"], out["preview_group"] = pa, pg
    # the texture pass (texturePassGI, CTextureApplyPass.process, updateToTextureColorGI)
    tr = g["tex_room"]
    texels, table = scenes.texture_tables(tr)
    mo = np.zeros((len(g["tex_u"]), 36), np.float32)
    for i in range(len(g["tex_u"])):
        m = texture_material(g, i)
        ref.lib.ref_texture_apply(ptr(m), int(g["tex_mat"][i]), float(g["tex_u"][i]), float(g["tex_v"][i]),
                                  ptr(texels), ptr(table), table.shape[0], ptr(mo[i]))
    out["tex_material_out"] = mo
    # a textured room frame, depth 6
    tn, tb, _, _ = bvh_build(orc, tr)
    tacc = np.zeros((40 * 32, 4), np.float32)
    tc = np.zeros(6, np.int32)
    ref.lib.ref_set_textures(ptr(texels), ptr(table), table.shape[0])
    ref.lib.ref_render_frame(ptr(tr.camera), 40, 32, 6, ptr(g["tex_seeds"]), 1.0, ptr(tr.points), ptr(tr.uvs),
                             ptr(tr.normals), ptr(tr.faces), tr.ntri, ptr(tr.materials), ptr(tn), ptr(tb), ptr(z),
                             ptr(z), ptr(z), 1, 1, 0, ptr(tacc), ptr(tc))
    ref.lib.ref_set_textures(None, None, 0)
    out["tex_frame_accum"], out["tex_frame_counts"] = tacc, tc
    # the preview frame of the textured room, with the preview's texture pass
    pa = np.zeros(40 * 32, np.int32)
    pg = np.zeros(40 * 32, np.int32)
    ref.lib.ref_set_textures(ptr(texels), ptr(table), table.shape[0])
    ref.lib.ref_preview(ptr(tr.camera), 40, 32, ptr(tr.points), ptr(tr.uvs), ptr(tr.normals), ptr(tr.faces),
                        tr.ntri, ptr(tr.materials), ptr(tn), ptr(tb), ptr(z), 1, 1, 0, ptr(pa), ptr(pg))
    ref.lib.ref_set_textures(None, None, 0)
    out["tex_preview_argb"], out["tex_preview_group"] = pa, pg
    np.savez_compressed(OUT, **out)
    print(OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
