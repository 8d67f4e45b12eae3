"""Shared helpers for the parity tests (oracle calls on the test side)."""
import numpy as np

from oracle.oracle import bvh_build, ptr


def oracle_trace(orc, sc, nodes, bounds, rays, counts=False):
    t = np.zeros(rays.shape[0], np.float32)
    p = np.zeros(rays.shape[0], np.int32)
    c = np.zeros((rays.shape[0], 2), np.int64) if counts else None
    orc.lib.or_trace_closest(ptr(rays), rays.shape[0], ptr(sc.points), ptr(sc.faces), sc.ntri, ptr(nodes),
                             ptr(bounds), ptr(t), ptr(p), ptr(c))
    return (t, p, c) if counts else (t, p)


def oracle_any(orc, sc, nodes, bounds, rays):
    o = np.zeros(rays.shape[0], np.int32)
    orc.lib.or_occlusion(ptr(rays), ptr(o), rays.shape[0], ptr(sc.points), ptr(sc.faces), sc.ntri, ptr(nodes),
                         ptr(bounds), None)
    return o


def env_tables(orc, envmap, w, h):
    lum = np.zeros(w * h, np.float32)
    sat = np.zeros(w * h, np.float32)
    orc.lib.or_env_lum_sat(ptr(envmap), w, h, ptr(lum), ptr(sat))
    return lum, sat


def oracle_grid(orc, env, nu, nv, rx, ry):
    """Initial light grid of an environment map: (func, per-cell SAT), both float32."""
    envmap, ew, eh = env
    lum, sat = env_tables(orc, envmap, ew, eh)
    func = np.zeros(nu * nv, np.float32)
    orc.lib.or_grid_init_func(None, ptr(sat), ew, eh, nu, nv, rx, ry, ptr(func))
    gsat = np.zeros(nu * nv, np.float32)
    orc.lib.or_lightgrid_sat(ptr(func), ptr(gsat), nu, nv, rx, ry)
    return func, gsat


def oracle_frames(orc, sc, nodes, bounds, W, H, depth, mode, rr, seeds_list, env=None, fp64=False, acc=None,
                  first_frame=1, grid=None):
    """Run len(seeds_list) frames of the oracle; returns (accum, counts per frame, ray counts).
    grid: dict(func, sat, nu, nv, rx, ry[, accum]) turns on grid-guided environment sampling;
    with an accum array, environment hits add into it."""
    if env is not None:
        envmap, ew, eh = env
        lum, sat = env_tables(orc, envmap, ew, eh)
        if fp64:
            lum64 = lum.astype(np.float64)
            sat64 = np.zeros(ew * eh, np.float64)
            orc.lib.or_env_sat_fp64(ptr(lum), ew, eh, ptr(sat64))
            lum, sat = lum64, sat64
    else:
        ew = eh = 1
        envmap = np.zeros((1, 4), np.float32)
        lum = np.zeros(1, np.float64 if fp64 else np.float32)
        sat = lum.copy()
    if acc is None:
        acc = np.zeros((W * H, 4), np.float64 if fp64 else np.float32)
    cam = sc.camera.copy()
    counts, rays = [], np.zeros(3, np.int64)
    textures = getattr(sc, "textures", None)
    if textures:
        from mambatracer_gb300 import scenes
        texels, table = scenes.texture_tables(sc)
        orc.lib.or_set_textures(ptr(texels), ptr(table), table.shape[0])
    try:
        _frames(orc, sc, nodes, bounds, W, H, depth, mode, rr, seeds_list, env is not None, fp64, acc, first_frame,
                grid, cam, envmap, lum, sat, ew, eh, counts, rays)
    finally:
        if textures:
            orc.lib.or_set_textures(None, None, 0)
    return acc, np.stack(counts), rays


def _frames(orc, sc, nodes, bounds, W, H, depth, mode, rr, seeds_list, has_env, fp64, acc, first_frame, grid, cam,
            envmap, lum, sat, ew, eh, counts, rays):
    for f, seeds in enumerate(seeds_list):
        c = np.zeros(depth, np.int32)
        rc = np.zeros(3, np.int64)
        s = None if seeds is None else np.ascontiguousarray(seeds, np.int32)
        args = [ptr(cam), W, H, depth, mode, rr, ptr(s), float(first_frame + f), ptr(sc.points), ptr(sc.uvs),
                ptr(sc.normals), ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds), ptr(envmap),
                ptr(lum), ptr(sat), ew, eh, int(has_env), int(fp64), ptr(acc), ptr(c), ptr(rc)]
        if grid is None:
            orc.lib.or_render_frame(*args)
        else:
            pos = np.ascontiguousarray(cam["position"].reshape(-1)[:4], np.float32)
            gacc = grid.get("accum")
            orc.lib.or_render_frame_grid(*args, ptr(grid["func"]), ptr(grid["sat"]), ptr(gacc), grid["nu"],
                                         grid["nv"], grid["rx"], grid["ry"], ptr(pos), 1, int(gacc is not None))
        counts.append(c)
        rays += rc


def rel_rmse(a, b):
    a = np.asarray(a, np.float64)[:, :3]
    b = np.asarray(b, np.float64)[:, :3]
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-30))


__all__ = ["oracle_trace", "oracle_any", "env_tables", "oracle_frames", "oracle_grid", "rel_rmse", "bvh_build",
           "ptr"]
