"""The reference's kernel set by name (mt_kernel_create / mt_kernel_set_arg_buf /
mt_launch_1d), driven the way the reference's host drives it (mambatracer_gb300.plain:
CDeviceGI.loop, CCompact, CLightConfiguration, CImage) on buffers in the reference's
layouts.

Against the fused path (mt_render_frame, reference semantics, plain film adds) queue
lengths and film are identical: the same shading functions and the same traversal order,
only the buffer layouts and the launch structure differ. Against the oracle the box room
matches exactly in queue lengths and within 1e-5 in film; the sunlit soup as the fused
path does (a path whose last-ulp transcendental rounds differently can change one queue
slot, and a sun sample carries much energy: counts within 1 %, film within 1e-3).
"""
import numpy as np
import pytest

from mambatracer_gb300 import api, plain, scenes
from tests.helpers import bvh_build, env_tables, oracle_frames, ptr, rel_rmse

pytestmark = pytest.mark.gpu


def seeds_for(depth, frames, seed=9):
    rng = np.random.default_rng(seed)
    return [rng.integers(2 ** 29, 2 ** 30, size=2 * (1 + 2 * depth)).astype(np.int32) for _ in range(frames)]


@pytest.mark.parametrize("which", ["room", "tex_room", "soup_env"])
def test_plain_loop_matches_oracle_and_fused_path(ctx, orc, which):
    if which == "room":
        sc, W, H, depth, env = scenes.box_room(64, 48), 64, 48, 4, None
    elif which == "tex_room":  # texturePassGI, textureApplyPass (the device lookup), updateToTextureColorGI
        sc, W, H, depth, env = scenes.textured_room(64, 48), 64, 48, 6, None
    else:
        sc = scenes.soup(30000, seed=5, extent=0.8, edge_sigma=0.015)
        W, H, depth, env = 48, 40, 5, (scenes.sky_env(256, 128), 256, 128)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    penv = None
    if env is not None:
        lum, sat = env_tables(orc, env[0], env[1], env[2])
        penv = (env[0], lum, sat, env[1], env[2])
    dev = plain.PlainDeviceGI(ctx, sc, nodes, bounds, W, H, max_depth=depth, env=penv)
    if which == "room":
        nl = np.zeros(2 * sc.ntri, np.int32)
        expect = orc.lib.or_light_list(ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nl))
        assert dev.nlights == expect > 0
        info = dev.light_info.read(np.zeros(2 * expect, np.int32)).reshape(-1, 2)  # LightInfo {faceId, type}
        assert np.array_equal(info[:, 0], nl[:expect]) and not info[:, 1].any()
    dev.set_camera(sc.camera)
    seeds = seeds_for(depth, 2)
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    if env is not None:
        S.set_env_with_sat(env[0], penv[1], penv[2], env[1], env[2])
    J = api.Job(ctx, S, W, H, max_depth=depth, mode=0, film_kahan=0)
    J.set_camera(sc.camera)
    acc = None
    for f, s in enumerate(seeds):
        counts = dev.frame(s, float(f + 1), record_counts=True)
        acc, oc, _ = oracle_frames(orc, sc, nodes, bounds, W, H, depth, 0, 0, [s], env=env, acc=acc,
                                   first_frame=f + 1)
        J.render(s, float(f + 1))
        _, jc = J.stats()
        assert counts == jc.tolist(), (counts, jc)
        if which != "soup_env":
            assert counts == oc[0].tolist(), (counts, oc[0])
        else:
            assert np.abs(np.array(counts) - oc[0]).max() <= max(1, 0.01 * oc[0].max()), (counts, oc[0])
    ctx.finish()
    film = dev.film()
    assert rel_rmse(film, acc) < (1e-3 if which == "soup_env" else 1e-5)
    assert film[:, :3].tobytes() == J.film()[:, :3].tobytes()
    # CImage.processImage through averageAccum, the reference's scans and updateFrameImage
    argb = dev.process_image(2.0)
    total = np.array([dev.scan_loglw.count(), dev.scan_count.count()], np.float32)
    lw = np.zeros(W * H, np.float32)
    ref = np.full(W * H, -16777216, np.int32)
    orc.lib.or_tonemap_with_total(ptr(film), W * H, 2.0, 0.18, 2.2, ptr(total), ptr(ref), None, None)
    fb = film[:, :3] / np.float32(2.0)
    lw = 0.2989 * fb[:, 0] + 0.5866 * fb[:, 1] + 0.1145 * fb[:, 2]
    assert int(total[1]) == int((lw > 0).sum())
    a = argb.view(np.uint8).reshape(-1, 4).astype(np.int32)
    b = ref.view(np.uint8).reshape(-1, 4).astype(np.int32)
    assert np.abs(a - b).max() <= 1 and np.mean(argb == ref) > 0.99
    dev.free()
    J.close()
    S.close()


def test_kernel_names_and_argument_errors(ctx):
    from mambatracer_gb300._lib import MTError, lib
    names = lib().mt_kernel_names().decode().split(",")
    for n in ("InitCameraRayDataJitter", "IntersectPrimitives", "SetupBSDFPath", "LightHitPass", "DirectLight",
              "SampleBSDFRayDirection", "CompactAtomic", "averageAccum", "updateFrameImage", "localScanInteger",
              "prefixSumRowSubgrid", "identifyMeshLights"):
        assert n in names
    with pytest.raises(MTError, match="unknown kernel"):
        plain.Kernel(ctx, "NoSuchKernel")
    k = plain.Kernel(ctx, "InitPathData")
    with pytest.raises(MTError, match="not set"):
        k.run(100, 100)
    k.free()


def test_light_grid_kernels(ctx, orc):
    """CAdaptiveEnvironment's kernels on the LightGrid struct: initLightGrid, calculateFunc,
    prefixSumRowSubgrid (groups of 16) and prefixSumColSubgrid (groups of 32) give the
    per-cell SAT of the reference's order (the oracle's, pinned to the reference)."""
    nu = nv = 1600
    n = nu * nv
    grid = plain.Buf(ctx, plain.GRID_BYTES)
    hdr = np.zeros(12, np.int32)
    hdr[0], hdr[2], hdr[3], hdr[4], hdr[5], hdr[6], hdr[7] = 1, 2048, 1024, nu, nv, 16, 32
    grid.write(hdr.view(np.uint8))
    ks = {name: plain.Kernel(ctx, name, grid) for name in ("initLightGrid", "calculateFunc", "prefixSumRowSubgrid",
                                                             "prefixSumColSubgrid")}
    ks["prefixSumRowSubgrid"].put_local(1, 16 * 4)
    ks["prefixSumColSubgrid"].put_local(1, 32 * 4)
    ks["initLightGrid"].run(n, 128)
    accum = np.random.default_rng(3).random(n).astype(np.float32)
    grid.write(accum, offset=48)  # accum array
    ks["calculateFunc"].run(n, 128)
    ks["prefixSumRowSubgrid"].run(n, 16)
    ks["prefixSumColSubgrid"].run(n, 32)
    whole = grid.read(np.zeros(plain.GRID_BYTES // 4, np.float32))
    func, sat = whole[12 + n:12 + 2 * n], whole[12 + 2 * n:12 + 3 * n]
    assert func.tobytes() == accum.tobytes()
    expect = np.zeros(n, np.float32)
    orc.lib.or_lightgrid_sat(ptr(accum), ptr(expect), nu, nv, 16, 32)
    assert sat.tobytes() == expect.tobytes()
    for k in ks.values():
        k.free()
    grid.free()
