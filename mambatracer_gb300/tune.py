"""Launch-shape autotuner: searches the hot kernels' launch shapes (mt_tuning) on a
render workload and persists the best as JSON.

The reference fixes its OpenCL local sizes (src/cl/device/CDeviceGI.java:122) and
launches every kernel over the whole frame. Here the shapes that decide the speed are
the traversal and shading builds (resident blocks per SM their registers are bounded
for: the block size), the persistent traversal grid of a launch that shares the GPU
with other frames (how much of the queue one launch takes on at once) and the
traversal steps a lane runs between refills (the regeneration threshold). Every
choice renders the same films, so the search compares speed alone: coordinate descent
from the current shapes over SPACE, each candidate timed over `frames` frames of a
render job after warm-up and scored by device-counted rays per second. Measurements
of one shape vary by a percent or two, so a candidate must beat the best by
`min_gain` to replace it, and the winner must beat the starting shapes again, by the
same margin, in alternating re-measurements before it is kept.

The served scheduler's merged queues add two shapes of their own: how many requests
share the queues (the queue length, in requests) and over how many streams. With
--served the search also times a batch of uneven requests through a merged server for
each pair of SERVED_SPACE and keeps the best beside the launch shapes.

    python -m mambatracer_gb300.tune --out tuning.json [--served]   # the 1M soup at 1080p
"""
from __future__ import annotations

import argparse
import json
import time

from . import api

SPACE = {
    "closest_minb": (8, 12, 16),
    "shadow_minb": (8, 12, 16),
    "closest_grid": (0, 3, 4, 6, 8),
    "shadow_grid": (0, 3, 4, 6),
    "shade_minb": (3, 4, 5),
    "refill_steps": (32, 64, 128),
    "shadow_stream": (0, 1),
}


SERVED_SPACE = {"lanes": (32, 48, 64), "merge_streams": (2, 4, 8)}


def search(measure, start: dict, space: dict = SPACE, rounds: int = 2, log=None, min_gain: float = 0.0,
           confirm: int = 0):
    """Coordinate descent: each field in turn takes the value of `space` that scores
    best with the other fields fixed (a candidate replaces the best only when it scores
    more than (1 + min_gain) times as much); repeats until a round changes nothing or
    after `rounds` rounds. measure(tuning) -> score, higher is better; each distinct
    tuning is measured once. With confirm > 0, the start and the winner are measured
    `confirm` more times each, alternately, and the winner is kept only when its mean
    beats the start's by the same margin. Returns (best tuning, its score, trials as
    (tuning, score))."""
    trials = []
    cache = {}

    def score(t):
        key = tuple(sorted(t.items()))
        if key not in cache:
            cache[key] = float(measure(dict(t)))
            trials.append((dict(t), cache[key]))
            if log:
                log(f"{cache[key]:9.2f}  {t}")
        return cache[key]

    best = dict(start)
    best_score = score(best)
    for _ in range(rounds):
        changed = False
        for field, values in space.items():
            for v in values:
                if v == best[field]:
                    continue
                cand = dict(best, **{field: v})
                s = score(cand)
                if s > best_score * (1.0 + min_gain):
                    best, best_score, changed = cand, s, True
        if not changed:
            break
    if confirm and best != start:
        a, b = [cache[tuple(sorted(start.items()))]], [best_score]
        for _ in range(confirm):
            for t, acc in ((start, a), (best, b)):
                acc.append(float(measure(dict(t))))
                trials.append((dict(t), acc[-1]))
                if log:
                    log(f"{acc[-1]:9.2f}  {t} (again)")
        ma, mb = sum(a) / len(a), sum(b) / len(b)
        if mb > ma * (1.0 + min_gain):
            return best, mb, trials
        return dict(start), ma, trials
    return best, best_score, trials


def job_measure(ctx, scene, camera, width: int, height: int, max_depth: int = 8, rr_depth: int = 3,
                inflight: int = 6, frames: int = 24, warmup: int = 3):
    """measure(tuning) for search(): installs the tuning, renders warm-up frames, then
    times `frames` frames of a benchmark-semantics job (CUDA graphs, `inflight` frames
    on their own streams, the light grid, if on, updated during the warm-up only) and
    returns its device-counted Mrays/s."""
    def measure(t):
        api.set_tuning(t)
        job = api.Job(ctx, scene, width, height, max_depth=max_depth, mode=1, rr_depth=rr_depth, film_kahan=1,
                      use_graph=1, inflight=inflight, grid_updates=warmup)
        try:
            job.set_camera(camera)
            for f in range(warmup):
                job.render(None, float(f + 1))
            ctx.finish()
            r0 = job.total_rays().sum()
            t0 = time.perf_counter()
            for f in range(frames):
                job.render(None, float(warmup + f + 1))
            ctx.finish()
            dt = time.perf_counter() - t0
            return float(job.total_rays().sum() - r0) / dt / 1e6
        finally:
            job.close()
    return measure


def served_requests(nreq: int = 64, seed: int = 3, lo: int = 128 * 128, hi: int = 1920 * 1080):
    """A batch of uneven requests: pixel counts log-uniform in [lo, hi] (16:9 when wide
    enough), cameras uniform on a sphere of radius 3 looking at the origin (fov 45),
    4 spp; request k goes to scene k mod the number of scenes."""
    import numpy as np
    from . import layout
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nreq):
        px = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        w = int(min(1920, max(8, round(np.sqrt(px * 16 / 9)))))
        h = int(min(1080, max(8, round(px / w))))
        g = rng.normal(size=3)
        pos = 3.0 * g / np.linalg.norm(g)
        up = (0.0, 1.0, 0.0) if abs(pos[1]) < 0.99 * 3.0 else (1.0, 0.0, 0.0)
        out.append((k, layout.make_camera(tuple(pos), (0.0, 0.0, 0.0), up, 45.0, w, h), w, h, 4))
    return out


def served_measure(ctx, scenes_, reqs, max_depth: int = 8, rr_depth: int = 3):
    """measure(shape) for search() over SERVED_SPACE: submits every request at once to a
    merged server with shape["lanes"] slots on shape["merge_streams"] streams and
    returns the device-counted Mrays/s from the first submission to the last film."""
    def measure(t):
        srv = api.Server(ctx, lanes=t["lanes"], max_width=1920, max_height=1080, max_spp=64, max_depth=max_depth,
                         rr_depth=rr_depth, film_kahan=1, merged=t["merge_streams"])
        try:
            for k, cam, w, h, spp in reqs:
                srv.submit(scenes_[k % len(scenes_)], cam, w, h, spp, float(1 + 64 * k), film=False)
            srv.drain()
            st = srv.stats()
            return sum(st["rays"]) / (st["span_ms"] * 1e-3) / 1e6
        finally:
            srv.close()
    return measure


def device_info(device: int = 0) -> dict:
    import torch
    p = torch.cuda.get_device_properties(device)
    return {"name": p.name, "sms": p.multi_processor_count}


def autotune(ctx, scene, camera, width: int, height: int, workload: str, out: str | None = None,
             rounds: int = 2, space: dict = SPACE, log=None, min_gain: float = 0.01, confirm: int = 2,
             workload_key: str | None = None, **job_kw) -> dict:
    """Searches the launch shapes on a render job of `scene`, installs the best and
    returns (and, with `out`, writes) the result: device, workload, the tuning and its
    Mrays/s, the starting tuning and its Mrays/s, and every trial."""
    start = api.get_tuning()
    measure = job_measure(ctx, scene, camera, width, height, **job_kw)
    measure(start)  # a first job pays one-time costs; not a trial
    best, score, trials = search(measure, start, space, rounds, log, min_gain, confirm)
    api.set_tuning(best)
    result = {
        "device": device_info(), "workload": workload, "workload_key": workload_key, "tuning": best,
        "mrays_per_s": round(score, 2), "min_gain": min_gain,
        "start": {"tuning": start, "mrays_per_s": round(trials[0][1], 2)},
        "trials": [{"tuning": t, "mrays_per_s": round(s, 2)} for t, s in trials],
    }
    if out:
        save(out, result)
    return result


def save(path: str, result: dict):
    with open(path, "w") as f:
        json.dump(result, f, indent=1)
        f.write("\n")


def load(path: str, device: int = 0, require_match: bool = True) -> dict | None:
    """Installs the tuning a search persisted in `path`. With require_match, only when
    the file was measured on a GPU of the same name and SM count; returns the file's
    contents when installed, else None."""
    with open(path) as f:
        result = json.load(f)
    if require_match and result.get("device") != device_info(device):
        return None
    api.set_tuning(result["tuning"])
    return result


def main():
    from . import build, scenes
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", required=True)
    ap.add_argument("--triangles", type=int, default=1_000_000)
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--frames", type=int, default=24)
    ap.add_argument("--rounds", type=int, default=2)
    ap.add_argument("--served", action="store_true", help="also search the merged server's slots and streams")
    ap.add_argument("--precision", type=int, default=3, choices=[0, 1, 2, 3],
                    help="traversal format of the scenes (mt_scene_set_bvh_precision; the bench's is 3)")
    args = ap.parse_args()
    build.build()
    ctx = api.Context(0)
    sc = scenes.soup(args.triangles, seed=1, width=args.width, height=args.height)
    S = api.Scene(ctx, sc)
    S.build_bvh_device(want_arrays=False)
    S.set_precision(args.precision)
    S.set_env(scenes.sky_env(2048, 1024), 2048, 1024)
    S.grid_config(1600, 1600, 16, 32, enable=2)
    records = {0: "FP32 records", 1: "FP16 records", 2: "wide BVH", 3: "4-wide FP16"}[args.precision]
    workload = (f"soup {args.triangles} triangles, {args.width}x{args.height}, depth 8, RR from 3, 2048x1024 sky, "
                f"1600x1600 light grid (FP64 cell SATs), 6 frames in flight, {records}")
    log = lambda m: print(m, flush=True)  # noqa: E731
    key = f"soup{args.triangles}_{args.width}x{args.height}"
    res = autotune(ctx, S, sc.camera, args.width, args.height, workload, out=args.out, rounds=args.rounds,
                   log=log, frames=args.frames, workload_key=key)
    print(json.dumps({k: res[k] for k in ("tuning", "mrays_per_s", "start")}), flush=True)
    if args.served:
        st = scenes.stadium(width=args.width, height=args.height)
        S2 = api.Scene(ctx, st)
        S2.build_bvh_device(want_arrays=False)
        S2.set_precision(args.precision)
        S2.set_env(scenes.sky_env(2048, 1024), 2048, 1024)
        reqs = served_requests()
        served_measure(ctx, [S, S2], reqs[:4])({"lanes": 4, "merge_streams": 2})  # warm-up
        best, score, trials = search(served_measure(ctx, [S, S2], reqs), {"lanes": 64, "merge_streams": 4},
                                     SERVED_SPACE, args.rounds, log, min_gain=0.01, confirm=2)
        res["served"] = {
            "workload": "64 requests at once, soup and stadium alternately, pixel counts log-uniform "
                        "128^2..1920x1080, 4 spp, depth 8, RR from 3, full-map sky sampling",
            "lanes": best["lanes"], "merge_streams": best["merge_streams"], "mrays_per_s": round(score, 2),
            "trials": [{"shape": t, "mrays_per_s": round(v, 2)} for t, v in trials],
        }
        save(args.out, res)
        print(json.dumps({k: res["served"][k] for k in ("lanes", "merge_streams", "mrays_per_s")}), flush=True)
        S2.close()
    S.close()
    ctx.close()


if __name__ == "__main__":
    main()
