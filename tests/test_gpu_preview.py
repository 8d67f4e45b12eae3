"""The preview device (CDeviceRT, Raytrace.cl): the fused frame (mt_preview_frame) and
the reference's kernels by name, against the oracle's frame. Material groups are
bit-exact; ARGB is bit-exact except where CUDA's powf/acosf/atan2f in the environment
lookup round differently from the host's (a channel moves by at most one 8-bit step).
"""
import numpy as np
import pytest

from mambatracer_gb300 import api, plain, scenes
from tests.helpers import bvh_build, ptr

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("which", ["room", "tex_room", "soup_env", "stadium_env"])
def test_preview_frame(ctx, orc, which):
    if which == "room":
        sc, W, H, env = scenes.box_room(96, 64), 96, 64, None
    elif which == "tex_room":  # the preview's texture pass (textureInitPassRT .. updateToTextureColorRT)
        sc, W, H, env = scenes.textured_room(96, 64), 96, 64, None
    elif which == "soup_env":
        sc, W, H = scenes.soup(30000, seed=7, extent=0.8, edge_sigma=0.02), 96, 64
        env = scenes.sky_env(256, 128)
    else:
        sc, W, H = scenes.stadium(quads=60, level=4, width=96, height=64), 96, 64
        env = scenes.sky_env(256, 128)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    envmap = env if env is not None else np.zeros((1, 4), np.float32)
    ew, eh = (256, 128) if env is not None else (1, 1)
    if env is not None:
        S.set_env(env, ew, eh)
    argb, group = S.preview(sc.camera, W, H)
    ra = np.zeros(W * H, np.int32)
    rg = np.zeros(W * H, np.int32)
    texels, table = scenes.texture_tables(sc)
    orc.lib.or_set_textures(ptr(texels), ptr(table), table.shape[0] if sc.textures else 0)
    try:
        orc.lib.or_preview(ptr(sc.camera), W, H, ptr(sc.points), ptr(sc.uvs), ptr(sc.normals), ptr(sc.faces),
                           sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds), ptr(envmap), ew, eh,
                           int(env is not None), ptr(ra), ptr(rg))
    finally:
        orc.lib.or_set_textures(None, None, 0)
    assert group.tobytes() == rg.tobytes()
    a = argb.view(np.uint8).reshape(-1, 4).astype(np.int32)
    b = ra.view(np.uint8).reshape(-1, 4).astype(np.int32)
    assert np.abs(a - b).max() <= 1 and np.mean(argb == ra) > 0.95
    # the same frame through the reference's kernels by name
    N = W * H
    cam = np.array(sc.camera, copy=True).reshape(-1)[:1]
    cam["dimension"] = (W, H)
    bufs = {"camera": plain.Buf(ctx, host=np.frombuffer(cam.tobytes(), np.uint8)),
            "rays": plain.Buf(ctx, 80 * N), "isects": plain.Buf(ctx, 96 * N), "bsdfs": plain.Buf(ctx, 256 * N),
            "argb": plain.Buf(ctx, 4 * N), "group": plain.Buf(ctx, 4 * N), "count": plain.int_buf(ctx, N),
            "points": plain.Buf(ctx, host=sc.points), "uvs": plain.Buf(ctx, host=sc.uvs),
            "normals": plain.Buf(ctx, host=sc.normals), "faces": plain.Buf(ctx, host=sc.faces),
            "size": plain.int_buf(ctx, sc.ntri), "materials": plain.Buf(ctx, host=sc.materials),
            "nodes": plain.Buf(ctx, host=nodes), "bounds": plain.Buf(ctx, host=bounds),
            "env": plain.Buf(ctx, host=envmap), "grid": plain.Buf(ctx, plain.GRID_BYTES),
            "tex": plain.Buf(ctx, 80 * N), "texels": plain.Buf(ctx, host=texels), "texref": plain.Buf(ctx, host=table)}
    bufs["tex"].write(np.zeros(80 * N, np.uint8))
    hdr = np.zeros(12, np.int32)
    hdr[0], hdr[2], hdr[3] = int(env is not None), ew, eh
    bufs["grid"].write(hdr.view(np.uint8))
    b_ = bufs
    G = plain.global_size(N, 100)
    ks = [plain.Kernel(ctx, "InitCameraRayData", b_["camera"], b_["rays"]),
          plain.Kernel(ctx, "IntersectPrimitives", b_["rays"], b_["isects"], b_["count"], b_["points"], b_["uvs"],
                       b_["normals"], b_["faces"], b_["size"], b_["nodes"], b_["bounds"]),
          plain.Kernel(ctx, "SetupBSDFRaytrace", b_["isects"], b_["rays"], b_["bsdfs"], b_["materials"]),
          plain.Kernel(ctx, "textureInitPassRT", b_["bsdfs"], b_["isects"], b_["tex"]),
          plain.Kernel(ctx, "textureApplyPass", b_["tex"], b_["count"], b_["texels"], b_["texref"]),
          plain.Kernel(ctx, "updateToTextureColorRT", b_["bsdfs"], b_["tex"]),
          plain.Kernel(ctx, "backgroundShade", b_["isects"], b_["camera"], b_["argb"], b_["rays"], b_["env"],
                       b_["grid"]),
          plain.Kernel(ctx, "fastShade", b_["isects"], b_["bsdfs"], b_["argb"]),
          plain.Kernel(ctx, "updateGroupbufferShadeImage", b_["isects"], b_["camera"], b_["group"])]
    for k in ks:
        k.run(G, 100)
    pa = b_["argb"].read(np.zeros(N, np.int32))
    pg = b_["group"].read(np.zeros(N, np.int32))
    assert pg.tobytes() == group.tobytes()
    assert pa.tobytes() == argb.tobytes()
    for k in ks:
        k.free()
    for b in bufs.values():
        b.free()
    S.close()


def test_find_bound(ctx, orc):
    """findBound (Util.cl:830-884): the bound of the faces of one material."""
    sc = scenes.box_room(32, 32)
    mats = sc.faces["mat"] & 0xFFFF
    grp = int(mats[0])
    pts = sc.points[:, :3]
    sel = np.stack([pts[sc.faces[k]] for k in ("vx", "vy", "vz")], 1)[mats == grp].reshape(-1, 3)
    init = np.array([np.inf, np.inf, np.inf, -np.inf, -np.inf, -np.inf], np.float32)
    bound = plain.Buf(ctx, host=init)
    args = [plain.int_buf(ctx, grp), plain.Buf(ctx, host=sc.points), plain.Buf(ctx, host=sc.uvs),
            plain.Buf(ctx, host=sc.normals), plain.Buf(ctx, host=sc.faces), plain.int_buf(ctx, sc.ntri), bound]
    k = plain.Kernel(ctx, "findBound", *args)
    k.run(plain.global_size(sc.ntri, 128), 128)
    got = bound.read(init)
    assert np.array_equal(got[:3], sel.min(0).astype(np.float32)) and np.array_equal(got[3:], sel.max(0).astype(np.float32))
    k.free()
    for b in args:
        b.free()
