"""Image-error and parity checks of benchmark-configuration frames against the
CPU oracle (test infrastructure: tests/ and the checking leg of bench.py call it,
after the timed region; the product never does).

The FP64 oracle renders a pixel subset of a full-size frame (or_render_frame_subset:
benchmark semantics key every random number on the pixel, so a subset renders
exactly the samples the full frame renders there). Frames and pixel chunks run in
a thread pool; each call is single-threaded C++ and releases the GIL.

Quantities (benchmark semantics, mode 1):
  * relative RMSE of the linear film (accumulated radiance, as CImage's accum
    buffer, src/cl/algorithms/CImage.java:86, before the per-frame average of
    src/cl/kernel/Image.cl:29-67, which divides both sides by the same count)
    against the FP64 oracle at matched samples;
  * queue lengths after every bounce of one full frame against the FP32 oracle;
  * primary-ray hit ids against the FP32 oracle traversal, with the rays whose
    hit lies within 1e-6 (barycentric) of a triangle edge counted apart
    (Moller-Trumbore, src/cl/kernel/Primitive.cl:3-29).
"""
from __future__ import annotations

import concurrent.futures as cf
import os

import numpy as np

from .oracle import ptr


def env_tables(orc, envmap, w, h, fp64):
    """Luminance and inclusive SAT of the map: FP32 (the reference's order) or FP64."""
    lum = np.zeros(w * h, np.float32)
    sat = np.zeros(w * h, np.float32)
    orc.lib.or_env_lum_sat(ptr(envmap), w, h, ptr(lum), ptr(sat))
    if not fp64:
        return lum, sat
    sat64 = np.zeros(w * h, np.float64)
    orc.lib.or_env_sat_fp64(ptr(lum), w, h, ptr(sat64))
    return lum.astype(np.float64), sat64


def strided_pixels(width, height, step):
    """Every step-th pixel in x and y, offset to the middle of each step x step block."""
    ys = np.arange(step // 2, height, step)
    xs = np.arange(step // 2, width, step)
    return (ys[:, None] * width + xs[None, :]).reshape(-1).astype(np.int32)


def subset_frames(orc, sc, nodes, bounds, width, height, depth, rr, frame_counts, pixels, env, fp64, grid=None,
                  threads=None, chunks=None):
    """Benchmark-semantics frames over a pixel subset.

    env: (envmap, w, h) or None; grid: dict(func, sat, nu, nv, rx, ry) for
    grid-guided environment sampling on that frozen grid (the camera position of
    the scene's camera). Returns (accum float64[len(pixels), 4] summed over the
    frames, queue lengths int64[depth] summed over frames and chunks, ray counts
    int64[3] [primary, extension, shadow])."""
    threads = threads or os.cpu_count() or 1
    pixels = np.ascontiguousarray(pixels, np.int32)
    if env is not None:
        envmap, ew, eh = env
        lum, sat = env_tables(orc, envmap, ew, eh, fp64)
    else:
        ew = eh = 1
        envmap = np.zeros((1, 4), np.float32)
        lum = np.zeros(1, np.float64 if fp64 else np.float32)
        sat = lum.copy()
    cam = sc.camera.copy()
    cam["dimension"] = (width, height)
    pos = np.ascontiguousarray(cam["position"].reshape(-1)[:4], np.float32)
    nchunk = chunks or max(1, (threads * 2) // max(1, len(frame_counts)))
    parts = [np.ascontiguousarray(c) for c in np.array_split(np.arange(len(pixels)), nchunk) if len(c)]
    dt = np.float64 if fp64 else np.float32

    def work(item):
        fc, idx = item
        px = np.ascontiguousarray(pixels[idx])
        acc = np.zeros((len(px), 4), dt)
        c = np.zeros(depth, np.int32)
        rc = np.zeros(3, np.int64)
        g = grid or {}
        rcode = orc.lib.or_render_frame_subset(
            ptr(cam), width, height, depth, 1, rr, None, float(fc), ptr(sc.points), ptr(sc.uvs), ptr(sc.normals),
            ptr(sc.faces), sc.ntri, ptr(sc.materials), ptr(nodes), ptr(bounds), ptr(envmap), ptr(lum), ptr(sat), ew,
            eh, int(env is not None), int(fp64), ptr(acc), ptr(c), ptr(rc), ptr(g.get("func")), ptr(g.get("sat")),
            None, g.get("nu", 0), g.get("nv", 0), g.get("rx", 0), g.get("ry", 0), ptr(pos), int(grid is not None), 0,
            ptr(px), len(px))
        assert rcode >= 0
        return idx, acc, c, rc

    acc = np.zeros((len(pixels), 4), np.float64)
    counts = np.zeros(depth, np.int64)
    rays = np.zeros(3, np.int64)
    items = [(fc, idx) for fc in frame_counts for idx in parts]
    with cf.ThreadPoolExecutor(threads) as ex:
        for idx, a, c, rc in ex.map(work, items):
            acc[idx] += a
            counts += c
            rays += rc
    return acc, counts, rays


def rel_rmse(a, b):
    """Relative RMSE of the RGB channels of two linear films (float4 per pixel)."""
    a = np.asarray(a, np.float64)[:, :3]
    b = np.asarray(b, np.float64)[:, :3]
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(np.sqrt(np.mean(b ** 2)), 1e-30))


def trace_oracle(orc, sc, nodes, bounds, rays, threads=None):
    """FP32 oracle closest hits of reference-layout rays: (t, prim)."""
    threads = threads or os.cpu_count() or 1
    n = rays.shape[0]
    t = np.zeros(n, np.float32)
    p = np.zeros(n, np.int32)

    def work(idx):
        r = np.ascontiguousarray(rays[idx])
        tt = np.zeros(len(idx), np.float32)
        pp = np.zeros(len(idx), np.int32)
        orc.lib.or_trace_closest(ptr(r), len(idx), ptr(sc.points), ptr(sc.faces), sc.ntri, ptr(nodes), ptr(bounds),
                                 ptr(tt), ptr(pp), None)
        t[idx] = tt
        p[idx] = pp

    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(work, [c for c in np.array_split(np.arange(n), threads * 4) if len(c)]))
    return t, p


def primary_rays(orc, cam, width, height, frame_count):
    """The benchmark-semantics camera rays of one frame (reference Ray layout)."""
    from mambatracer_gb300 import layout
    n = width * height
    rays = np.zeros(n, layout.RAY)
    cam = cam.copy()
    cam["dimension"] = (width, height)
    orc.lib.or_raygen(ptr(cam), ptr(rays), None, float(frame_count), n, 1)
    return rays


def edge_distance(sc, rays, prim):
    """min(b1, b2, 1 - b1 - b2) of each hit (FP64 Moller-Trumbore on the hit
    triangle; +inf where prim < 0)."""
    out = np.full(len(prim), np.inf)
    h = prim >= 0
    if not h.any():
        return out
    f = sc.faces[prim[h]]
    pts = sc.points.reshape(-1, 4)[:, :3].astype(np.float64)
    p1, p2, p3 = pts[f["vx"]], pts[f["vy"]], pts[f["vz"]]
    o = np.stack([rays["o"][h][:, k] for k in range(3)], 1).astype(np.float64)
    d = np.stack([rays["d"][h][:, k] for k in range(3)], 1).astype(np.float64)
    e1, e2 = p2 - p1, p3 - p1
    hv = np.cross(d, e2)
    a = np.einsum("ij,ij->i", e1, hv)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / a
        s = o - p1
        b1 = inv * np.einsum("ij,ij->i", s, hv)
        q = np.cross(s, e1)
        b2 = inv * np.einsum("ij,ij->i", d, q)
    out[h] = np.minimum(np.minimum(b1, b2), 1.0 - b1 - b2)
    return out


def hit_parity(sc, rays, t_gpu, p_gpu, t_ref, p_ref, eps=1e-6):
    """Hit-id parity summary: differing ids, how many of them are exact-distance
    ties or rays within eps of an edge, and how many rays overall are within eps."""
    diff = p_gpu != p_ref
    tie = diff & (t_gpu.view(np.uint32) == t_ref.view(np.uint32))
    edge_ref = edge_distance(sc, rays, p_ref) < eps
    edge_gpu = edge_distance(sc, rays, p_gpu) < eps
    near_edge = edge_ref | edge_gpu
    t_ulps = np.abs(t_gpu.view(np.int32).astype(np.int64) - t_ref.view(np.int32).astype(np.int64))
    same = ~diff
    return {
        "rays": int(len(p_ref)),
        "hit_id_mismatches": int(diff.sum()),
        "mismatches_exact_t_ties": int(tie.sum()),
        "mismatches_within_eps_of_edge": int((diff & near_edge).sum()),
        "mismatches_unexplained": int((diff & ~tie & ~near_edge).sum()),
        "rays_within_eps_of_edge": int(edge_ref.sum()),
        "edge_eps": eps,
        "max_t_ulps_same_id": int(t_ulps[same].max()) if same.any() else 0,
    }
