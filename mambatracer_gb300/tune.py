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
render job after warm-up and scored by device-counted rays per second.

    python -m mambatracer_gb300.tune --out tuning.json     # the 1M soup at 1080p
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
}


def search(measure, start: dict, space: dict = SPACE, rounds: int = 2, log=None):
    """Coordinate descent: each field in turn takes the value of `space` that scores
    best with the other fields fixed; repeats until a round changes nothing or after
    `rounds` rounds. measure(tuning) -> score, higher is better; each distinct tuning
    is measured once. Returns (best tuning, its score, trials as (tuning, score))."""
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
                if s > best_score:
                    best, best_score, changed = cand, s, True
        if not changed:
            break
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


def device_info(device: int = 0) -> dict:
    import torch
    p = torch.cuda.get_device_properties(device)
    return {"name": p.name, "sms": p.multi_processor_count}


def autotune(ctx, scene, camera, width: int, height: int, workload: str, out: str | None = None,
             rounds: int = 2, space: dict = SPACE, log=None, **job_kw) -> dict:
    """Searches the launch shapes on a render job of `scene`, installs the best and
    returns (and, with `out`, writes) the result: device, workload, the tuning and its
    Mrays/s, the starting tuning and its Mrays/s, and every trial."""
    start = api.get_tuning()
    measure = job_measure(ctx, scene, camera, width, height, **job_kw)
    best, score, trials = search(measure, start, space, rounds, log)
    api.set_tuning(best)
    result = {
        "device": device_info(), "workload": workload, "tuning": best, "mrays_per_s": round(score, 2),
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
    args = ap.parse_args()
    build.build()
    ctx = api.Context(0)
    sc = scenes.soup(args.triangles, seed=1, width=args.width, height=args.height)
    S = api.Scene(ctx, sc)
    S.build_bvh_device(want_arrays=False)
    S.set_env(scenes.sky_env(2048, 1024), 2048, 1024)
    S.grid_config(1600, 1600, 16, 32, enable=2)
    workload = (f"soup {args.triangles} triangles, {args.width}x{args.height}, depth 8, RR from 3, 2048x1024 sky, "
                "1600x1600 light grid (FP64 cell SATs), 6 frames in flight")
    res = autotune(ctx, S, sc.camera, args.width, args.height, workload, out=args.out, rounds=args.rounds,
                   log=lambda m: print(m, flush=True), frames=args.frames)
    print(json.dumps({k: res[k] for k in ("tuning", "mrays_per_s", "start")}), flush=True)
    S.close()
    ctx.close()


if __name__ == "__main__":
    main()
