#!/usr/bin/env python
"""Benchmark: Mrays/s of the wavefront GI path on the 1M-triangle soup with the
HDR environment at 1920x1080 (1 spp per step, max depth 8, Russian roulette
from bounce 3), one GB300 per rank.

A step is one GI frame (one pass of every pixel). `value` counts primary,
extension and shadow rays traced on the device, over the timed frames, divided
by the device time (CUDA events on the library's stream); inputs are resident.
`e2e` is the same metric through the C-ABI with host buffers: every step
uploads the camera from pinned host memory, renders, and reads the film back
into pinned host memory.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) each rank renders its own frames of the same job
(weak scaling: per-GPU work fixed), with no collective on the data path.
The reference arm times the reference algorithm on the host cores: the
restatement in oracle/ (the reference's OpenCL C needs an OpenCL runtime, and the
machine that runs the benchmark has none, nor the reference sources).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W_DEFAULT, H_DEFAULT, DEPTH, RR = 1920, 1080, 8, 3
ENV_ON = True  # the sky environment and its light grid (off for the box room)
NTRI = 1_000_000
ENV_W, ENV_H = 2048, 1024
GRID = (1600, 1600, 16, 32)  # light grid: nu, nv, tiles per cell (reference defaults, CLightGrid.java)
GRID_UPDATES = 5             # CDeviceGI.loop updates the grid after its first 5 frames
METRIC = "Mrays/s (primary + extension + shadow rays traced, device-counted)"
# soup: the 1M-triangle soup at 1 spp (the headline configuration); stadium: the
# 3.3M-triangle plane + displaced icosphere at 4 spp
WORKLOADS = {
    "soup": dict(name="soup1M_1920x1080_depth8_rr3_env2048x1024", spp=1,
                 scene="1,000,000-triangle soup, centroids U[-1,1]^3, edges N(0,0.005^2), GGX r U[0.05,0.8], "
                       "albedo U[0.2,0.9]",
                 l2="no flush: per-step working set (path state + queues ~420 MB, traversal records + triangles "
                    "80-112 MB) exceeds "
                    "the 129 MB L2"),
    "room": dict(name="boxroom36_256x256_depth4", spp=1, width=256, height=256, depth=4, rr=0, env=False,
                 scene="box room: 36 triangles (walls, two GGX boxes r 0.3, a 0.25 x 0.25 ceiling emitter of "
                       "radiance 15), pinhole fov 40, no environment",
                 l2="no flush: the working set (path state + queues of 4 frames ~50 MB, BVH 3 KB) stays in the "
                    "129 MB L2; an in-cache, launch-bound case"),
    "stadium": dict(name="stadium3.3M_1920x1080_spp4_depth8_rr3_env2048x1024", spp=4,
                    scene="200x200 ground plane of 2,000,000 triangles + icosphere level 8 (1,310,720 triangles, "
                          "r 0.05) displaced by 3-octave value noise of amplitude 0.005; Lambert/GGX 50/50, "
                          "r U[0.05,0.8], albedo U[0.2,0.9]",
                    l2="no flush: per-step working set (path state + queues ~420 MB, BVH+triangles ~370 MB) exceeds "
                       "the 129 MB L2"),
}
WORKLOAD = WORKLOADS["soup"]["name"]
# traversal formats (mt_scene_set_bvh_precision)
RECORDS = {0: "FP32 child boxes, binary, 64 B records",
           1: "FP16 child boxes rounded outward, binary, 32 B records",
           2: "wide BVH: up to 8 children with 8-bit child boxes rounded outward, 96 B nodes",
           3: "4-wide: a record's grandchildren with FP16 boxes rounded outward, 64 B nodes"}


def make_scene(kind, small, width, height):
    from mambatracer_gb300 import scenes
    if kind == "room":
        return scenes.box_room(width, height)
    if kind == "stadium":
        return scenes.stadium(quads=300 if small else 1000, level=6 if small else 8, width=width, height=height)
    return scenes.soup(200_000 if small else NTRI, seed=1, width=width, height=height)


TUNED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "mambatracer_gb300", "tuning_gb300.json")


def apply_tuning(workload_key=None):
    """Installs the launch shapes the autotuner (mambatracer_gb300.tune) persisted for
    this GPU model and for this workload, when the file exists and matches; returns
    what the run uses."""
    from mambatracer_gb300 import api, tune
    res = None
    if workload_key and os.path.exists(TUNED):
        with open(TUNED) as f:
            if json.load(f).get("workload_key") == workload_key:
                res = tune.load(TUNED)
    if res is None:
        return {"source": "built-in defaults", "tuning": api.get_tuning()}
    return {"source": "autotuned (mambatracer_gb300/tuning_gb300.json: " + res["workload"] + ")",
            "tuning": api.get_tuning()}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def config_dict(kind, width, height, ntri, world, inflight=1, small=False):
    w = WORKLOADS[kind]
    return {
        "workload": w["name"] if not small else f"{kind}{ntri}_{width}x{height}_depth{DEPTH}_rr{RR}_env{ENV_W}x{ENV_H}",
        "scene": w["scene"] if not small else f"{ntri}-triangle {kind} (reduced)",
        "environment": (f"{ENV_W}x{ENV_H} FP32 lat-long sky gradient + 0.5 deg Gaussian sun (peak 5e4); SAT built in FP64"
                        if ENV_ON else "none (the ceiling emitter lights the room)"),
        "light_grid": (f"{GRID[0]}x{GRID[1]} grid of {GRID[2]}x{GRID[3]}-tile cells, FP64 per-cell SATs, updated from "
                       f"environment hits after each of the first {GRID_UPDATES} warm-up frames, then fixed"
                       if ENV_ON else "none"),
        "resolution": f"{width}x{height}", "spp_per_step": w["spp"], "max_depth": DEPTH, "rr_from_bounce": RR,
        "rng": "per-pixel seed pixel ^ 0x9E3779B9 into the reference WangHash chain",
        "film": "FP32 Kahan-compensated",
        "launch": ("CUDA graph per frame, its shadow rays of bounce b on a second stream beside its extension rays "
                   "of bounce b+1" + (f", {inflight} frames in flight on separate streams" if inflight > 1 else "")),
        "l2": w["l2"],
        "parallelism": f"replicas x{world} (pixels/frames independent, no collective)",
    }


# ----------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=2)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------- CPU side
def cpu_grid(orc, sat):
    """The light grid's initial function and per-cell SATs for the environment."""
    from oracle.oracle import ptr
    nu, nv, rx, ry = GRID
    func = np.zeros(nu * nv, np.float32)
    orc.lib.or_grid_init_func(None, ptr(sat), ENV_W, ENV_H, nu, nv, rx, ry, ptr(func))
    gsat = np.zeros(nu * nv, np.float32)
    orc.lib.or_lightgrid_sat(ptr(func), ptr(gsat), nu, nv, rx, ry)
    return func, gsat


def cpu_render_rate(orc, sc, nodes, bounds, env, lum, sat, width, height, seconds, threads, grid):
    """Oracle frames (benchmark semantics, grid-guided environment sampling on the
    given grid) rendered in parallel threads for about `seconds`; returns (rays,
    wall seconds, frames)."""
    from oracle.oracle import ptr
    cam = sc.camera.copy()
    pos = np.ascontiguousarray(cam["position"].reshape(-1)[:4], np.float32)
    gfunc, gsat = grid
    stop = time.perf_counter() + seconds
    lock = threading.Lock()
    total = {"rays": 0, "frames": 0}

    def worker(tid):
        f = 0
        while time.perf_counter() < stop or f == 0:
            acc = np.zeros((width * height, 4), np.float32)
            c = np.zeros(DEPTH, np.int32)
            rc = np.zeros(3, np.int64)
            orc.lib.or_render_frame_grid(ptr(cam), width, height, DEPTH, 1, RR, None, float(1 + tid + 1000 * f),
                                         ptr(sc.points), ptr(sc.uvs), ptr(sc.normals), ptr(sc.faces), sc.ntri,
                                         ptr(sc.materials), ptr(nodes), ptr(bounds), ptr(env), ptr(lum), ptr(sat),
                                         ENV_W, ENV_H, int(ENV_ON), 0, ptr(acc), ptr(c), ptr(rc), ptr(gfunc), ptr(gsat),
                                         None, *GRID, ptr(pos), int(ENV_ON), 0)
            with lock:
                total["rays"] += int(rc.sum())
                total["frames"] += 1
            f += 1

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(worker, range(threads)))
    return total["rays"], time.perf_counter() - t0, total["frames"]


def cpu_scene(orc, kind):
    from mambatracer_gb300 import scenes
    from oracle.oracle import bvh_build, ptr
    sc = make_scene(kind, False, W_DEFAULT, H_DEFAULT)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    env = scenes.sky_env(ENV_W, ENV_H)
    lum = np.zeros(ENV_W * ENV_H, np.float32)
    sat = np.zeros(ENV_W * ENV_H, np.float32)
    orc.lib.or_env_lum_sat(ptr(env), ENV_W, ENV_H, ptr(lum), ptr(sat))
    return sc, nodes, bounds, env, lum, sat


def algorithmic_bytes(orc, sc, nodes, bounds, cam, width, height, frame_count, threads, rec_bytes=64):
    """Per-launch algorithmic bytes of the primary-ray closest-hit launch:
    sum over rays of 32 (ray in) + 16 (hit out) + rec_bytes per interior visit
    (64 for FP32 records, 32 for FP16 ones) + 48 per triangle test, the visit
    counts taken from the FP32 oracle traversal of the same rays
    (benchmark-semantics raygen of this frame)."""
    from mambatracer_gb300 import layout
    from oracle.oracle import ptr
    n = width * height
    rays = np.zeros(n, layout.RAY)
    cam = cam.copy()
    cam["dimension"] = (width, height)
    orc.lib.or_raygen(ptr(cam), ptr(rays), None, float(frame_count), n, 1)
    chunks = np.array_split(np.arange(n), threads * 4)
    res = np.zeros((n, 2), np.int64)

    def work(idx):
        r = np.ascontiguousarray(rays[idx])
        t = np.zeros(len(idx), np.float32)
        p = np.zeros(len(idx), np.int32)
        c = np.zeros((len(idx), 2), np.int64)
        orc.lib.or_trace_closest(ptr(r), len(idx), ptr(sc.points), ptr(sc.faces), sc.ntri, ptr(nodes), ptr(bounds),
                                 ptr(t), ptr(p), ptr(c))
        res[idx] = c

    with cf.ThreadPoolExecutor(threads) as ex:
        list(ex.map(work, [c for c in chunks if len(c)]))
    v_int, tri = res[:, 0].sum(), res[:, 1].sum()
    return int(n * 48 + rec_bytes * v_int + 48 * tri), float(v_int) / n, float(tri) / n


def kernel_rooflines(kprof, per_kernel, peak, rays, counts, closest_alg_bytes, closest_ms):
    """Per-kernel roofline of the bounce-1 launches: each memory level's bytes per
    launch from one ncu capture of that launch (profiles/kernels_soup1M_1080p.json)
    over the launch's CUDA-event time in this run, with the warp efficiency and the
    stalls that bound it. Algorithmic fractions: the closest-hit traversal's (the
    headline roofline); shading's over the whole frame, from the frame's device
    counts as a lower bound (queue entry 32 + hit 8 + path state 36 B read by the
    hit phase; for every path that goes on, list 8 + the same 76 read + path state
    36 + next queue 32 written; 48 B per shadow ray written; the paths that Russian
    roulette ends after their sample and the film adds are left out); the shadow
    rays' visit counts are not known off the device, so their fraction is absent."""
    if kprof is None:
        return None
    ks = kprof["kernels"]
    out = {}

    def level_rates(names, ms):
        d = {k: sum(ks[n][k] for n in names) for k in ("dram_bytes", "l2_bytes", "l1_global_bytes", "l1_local_bytes")}
        s = ms * 1e-3
        r = {"launch_ms": round(ms, 4), **d,
             "dram_gbs": round(d["dram_bytes"] / s / 1e9, 1), "l2_gbs": round(d["l2_bytes"] / s / 1e9, 1),
             "l1_global_gbs": round(d["l1_global_bytes"] / s / 1e9, 1),
             "l1_local_gbs": round(d["l1_local_bytes"] / s / 1e9, 1),
             "dram_frac_of_measured_peak": round(d["dram_bytes"] / s / 1e9 / peak, 4)}
        for k in ("simt_efficiency", "stall_long_scoreboard_per_issue", "stall_no_instruction_per_issue",
                  "issue_active_pct", "registers", "grid"):
            r[k] = [ks[n][k] for n in names] if len(names) > 1 else ks[names[0]][k]
        return r

    out["k_trace_closest"] = level_rates(["k_trace_closest"], per_kernel["trace_closest_b1"])
    out["k_trace_closest"]["alg_gbs"] = round(closest_alg_bytes / (closest_ms * 1e-3) / 1e9, 1)
    out["k_trace_shadow"] = level_rates(["k_trace_shadow"], per_kernel["trace_shadow_b1"])
    out["k_shade_hit+k_shade_cont"] = level_rates(["k_shade_hit", "k_shade_cont"], per_kernel["shade_b1"])
    queue = int(rays[0] + rays[1])
    goes_on = int(np.sum(counts))
    alg = queue * 76 + goes_on * (8 + 76 + 68) + int(rays[2]) * 48
    shade_ms = sum(v for k, v in per_kernel.items() if k.startswith("shade_"))
    out["k_shade_hit+k_shade_cont"]["frame_alg_bytes_lower_bound"] = alg
    out["k_shade_hit+k_shade_cont"]["frame_ms"] = round(shade_ms, 4)
    out["k_shade_hit+k_shade_cont"]["frame_alg_frac_lower_bound"] = round(alg / (shade_ms * 1e-3) / 1e9 / peak, 4)
    return out


# ------------------------------------------------------------- GPU arm
def bench_scene(ctx, kind, small, width, height, precision):
    """The workload's scene on the device as every step renders it: the BVH built on
    the GPU (CNormalBVH.build's tree), the record format, the sky environment with
    its FP64 SAT and the light grid with FP64 per-cell SATs. Returns (host scene,
    device scene, reference-layout nodes and bounds, environment map, build ms)."""
    from mambatracer_gb300 import api, scenes
    sc = make_scene(kind, small, width, height)
    env = scenes.sky_env(ENV_W, ENV_H)
    S = api.Scene(ctx, sc)
    t_bvh = time.perf_counter()
    nodes, bounds = S.build_bvh_device()  # CNormalBVH.build's tree, built level by level on the GPU
    bvh_build_ms = (time.perf_counter() - t_bvh) * 1e3
    if precision:
        S.set_precision(precision)  # 1: FP16 records; 2: wide BVH, 8-bit boxes; 3: 4-wide, FP16 boxes
    if ENV_ON:
        S.set_env(env, ENV_W, ENV_H)
        S.grid_config(*GRID, enable=2)  # grid-guided environment sampling, FP64 per-cell SATs
    return sc, S, nodes, bounds, env, bvh_build_ms


def bench_job(ctx, S, width, height, spp, inflight, grid_updates):
    """The render job every soup/stadium/room step runs: benchmark semantics, depth
    DEPTH, Russian roulette from RR, Kahan film, one CUDA graph per frame."""
    from mambatracer_gb300 import api
    return api.Job(ctx, S, width, height, max_depth=DEPTH, mode=1, rr_depth=RR, film_kahan=1, use_graph=1,
                   inflight=inflight, grid_updates=grid_updates, spp=spp)


def image_check(ctx, S, sc, nodes, bounds, env, width, height, spp, inflight, steps=16, stride=8, orc=None,
                parity=True):
    """The benchmark job's film against the FP64 oracle, and its parity figures.

    Renders a fresh job exactly as the timed one (same scene, environment, light
    grid, job settings, GRID_UPDATES grid-updating warm-up frames, then `steps`
    steps of spp passes from a cleared film), then with the oracle (after all GPU
    work; it is the checker here):
      * the FP64 oracle renders every stride-th pixel in x and y at the same frame
        counts on the grid the GPU froze: relative RMSE of the linear film;
      * (parity) the FP32 oracle, the reference's algorithm in the reference's
        precision, renders the same samples: its own error against the FP64
        oracle (the image error of any FP32 run of this algorithm at these samples:
        discrete decisions, an edge hit or missed, a Russian-roulette or lobe
        choice, flip between FP32 and FP64 on a few samples, and a flipped path
        that then sees the sun moves its pixel by a lot), and the GPU's against it;
      * (parity) the FP32 oracle renders the last pass in full: its queue lengths and ray
        counts against the GPU's (benchmark semantics: the reference's RR and BSDF
        branches flip on last-ulp differences of CUDA's transcendentals, so counts
        drift a little);
      * the first pass's primary rays traced through the C-ABI (mt_trace_closest)
        against the FP32 oracle traversal: hit-id mismatches, exact-t ties, rays
        within 1e-6 barycentric of an edge.
    env: (rgb, w, h) or None. Returns a dict."""
    from oracle import check
    from oracle.oracle import Oracle
    orc = orc or Oracle()
    job = bench_job(ctx, S, width, height, spp, inflight, GRID_UPDATES if env is not None else 0)
    job.set_camera(sc.camera)
    frame0 = lambda i: 1.0 + i * spp  # noqa: E731  (passes of a step take consecutive counts)
    for i in range(GRID_UPDATES):
        job.render(None, frame0(i))
    job.clear()
    fcs = []
    for i in range(steps):
        job.render(None, frame0(GRID_UPDATES + i))
        fcs += [frame0(GRID_UPDATES + i) + k for k in range(spp)]
    film = job.film()
    rays_gpu, counts_gpu = job.stats()  # the last step; counts of its last pass
    grid = None
    if env is not None and S.grid[4]:
        func, gsat, _ = job.grid()
        grid = dict(func=func, sat=gsat, nu=S.grid[0], nv=S.grid[1], rx=S.grid[2], ry=S.grid[3])
    job.close()
    t0 = time.perf_counter()
    px = check.strided_pixels(width, height, stride)
    acc64, _, _ = check.subset_frames(orc, sc, nodes, bounds, width, height, DEPTH, RR, fcs, px, env, True, grid)
    err = check.rel_rmse(film[px], acc64)
    res = {"rel_rmse_fp64": float(f"{err:.4e}"), "spp": len(fcs), "pixels": int(len(px)),
           "pixel_subset": f"every {stride}th pixel in x and y ({len(px)} of {width * height})",
           "film": "linear accumulated radiance (CImage accum), Kahan FP32 on the GPU, FP64 in the oracle"}
    if not parity:
        res["oracle_seconds"] = round(time.perf_counter() - t0, 1)
        return res
    acc32, _, _ = check.subset_frames(orc, sc, nodes, bounds, width, height, DEPTH, RR, fcs, px, env, False, grid)
    res["reference_fp32_rel_rmse_fp64"] = float(f"{check.rel_rmse(acc32, acc64):.4e}")
    res["rel_rmse_vs_reference_fp32"] = float(f"{check.rel_rmse(film[px], acc32):.4e}")
    allpx = np.arange(width * height, dtype=np.int32)
    _, c32, r32 = check.subset_frames(orc, sc, nodes, bounds, width, height, DEPTH, RR, [fcs[-1]], allpx, env, False,
                                      grid)
    rays = check.primary_rays(orc, sc.camera, width, height, fcs[0])
    t_gpu, p_gpu = S.trace_closest(rays)
    t_ref, p_ref = check.trace_oracle(orc, sc, nodes, bounds, rays)
    hits = check.hit_parity(sc, rays, t_gpu, p_gpu, t_ref, p_ref)
    last_rays_gpu = rays_gpu if spp == 1 else None
    drift = (np.abs(counts_gpu.astype(np.int64) - c32) / np.maximum(c32, 1)).tolist()
    res.update({
        "queue_lengths_gpu": counts_gpu.tolist(), "queue_lengths_fp32_oracle": c32.tolist(),
        "queue_length_rel_drift": [round(x, 5) for x in drift],
        "rays_last_pass_gpu": None if last_rays_gpu is None else last_rays_gpu.tolist(),
        "rays_last_pass_fp32_oracle": r32.tolist(),
        "primary_hits": hits, "oracle_seconds": round(time.perf_counter() - t0, 1),
    })
    return res


def run_gpu(args):
    import torch
    rank, world, local = dist_env()
    if world > 1:
        torch.cuda.set_device(local)
        torch.distributed.init_process_group("nccl", device_id=torch.device("cuda", local))
    from mambatracer_gb300 import api, build
    build.build()
    default_shapes = api.get_tuning()
    launch_shapes = apply_tuning(f"soup{NTRI}_{W_DEFAULT}x{H_DEFAULT}"
                                 if args.workload == "soup" and not args.small else None)

    width, height = (640, 360) if args.small and args.workload != "room" else (W_DEFAULT, H_DEFAULT)
    spp = WORKLOADS[args.workload]["spp"]
    ctx = api.Context(local)
    sc, S, nodes, bounds, env, bvh_build_ms = bench_scene(ctx, args.workload, args.small, width, height,
                                                          args.precision)
    ntri = sc.ntri
    job = bench_job(ctx, S, width, height, spp, args.inflight, min(GRID_UPDATES, args.warmup))
    cam = sc.camera.copy()
    job.set_camera(cam)

    from mambatracer_gb300.dist import frame_number

    def frame_no(step):
        # State.frameCount of the step's first pass; passes of one step take consecutive counts
        return 1.0 + (frame_number(step, rank, world) - 1.0) * spp

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    for i in range(args.warmup):
        job.render(None, frame_no(i))
    ctx.finish()
    job.clear()
    barrier()
    ctx.finish()
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = job.launches()
    ctx.record(0)
    for i in range(args.steps):
        job.render(None, frame_no(args.warmup + i))
    ctx.record(1)
    gpu_launches = job.launches() - launches0
    ctx.finish()
    barrier()
    ms = ctx.elapsed_ms(0, 1)
    clk = clocks.stop()
    rays = job.total_rays()
    total_rays = int(rays.sum())
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
        rr = torch.tensor([total_rays], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(rr)
        total_rays = int(rr.item())
    value = total_rays / (ms * 1e-3) / 1e6

    # e2e through the C-ABI with host buffers: camera in (pinned), film out (pinned)
    import ctypes as C

    from mambatracer_gb300._lib import check, lib
    nbuf = 9  # read i completes when read i + 8 is enqueued (eight stay pending): its buffer is free for read i + 9
    film_host = [torch.empty((width * height, 4), dtype=torch.float32, pin_memory=True) for _ in range(nbuf)]
    cam_host = torch.empty(64, dtype=torch.uint8, pin_memory=True)
    cam_host.numpy()[:] = np.frombuffer(cam.tobytes(), np.uint8)
    L = lib()
    e2e_steps = args.steps
    job.clear()
    barrier()
    ctx.finish()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        # camera in, frame submitted, the film after this frame read back while
        # the next frames render (a ring of pinned host films)
        check(L.mt_job_set_camera(job.h, C.c_void_p(cam_host.data_ptr())))
        check(L.mt_render_frame(job.h, None, frame_no(10000 + i)))
        check(L.mt_film_read_async(job.h, C.c_void_p(film_host[i % nbuf].data_ptr()), 0))
    check(L.mt_film_wait(job.h))
    e2e_s = time.perf_counter() - t0
    e2e_rays = int(job.total_rays().sum())
    if world > 1:
        t = torch.tensor([e2e_s], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_s = float(t.item())
        rr = torch.tensor([e2e_rays], device="cuda", dtype=torch.float64)
        torch.distributed.all_reduce(rr)
        e2e_rays = int(rr.item())
    e2e = {"value": e2e_rays / e2e_s / 1e6, "unit": "Mrays/s",
           "h2d_bytes_per_step": 64 + 416, "d2h_bytes_per_step": width * height * 16,
           "note": ("camera (64 B) and the pass parameters (416 B) in, the float4 film after each frame out "
                    "(mt_film_read_async into a ring of pinned buffers), per frame")}

    out = None
    if rank == 0:
        # per-launch device times (profiled frames, no graph) for the roofline
        pj = api.Job(ctx, S, width, height, max_depth=DEPTH, mode=1, rr_depth=RR, film_kahan=1, profile=1,
                     grid_updates=0)
        pj.set_camera(cam)
        prof_frames = 5
        kms = []
        for i in range(prof_frames + 1):
            pj.render(None, frame_no(i))
            if i:
                kms.append(pj.kernel_ms()[0])
        kms = np.mean(np.stack(kms), axis=0)
        names = ["raygen"] + [f"{k}_b{b}" for b in range(1, DEPTH + 1) for k in ("trace_closest", "shade",
                                                                                 "trace_shadow")]
        per_kernel = {n: round(float(v), 4) for n, v in zip(names, kms)}
        trace_total = float(sum(v for n, v in per_kernel.items() if n.startswith("trace_")))
        frame_total = float(kms.sum())
        prof_rays, prof_counts = pj.stats()  # the last profiled frame
        pj.close()
        from oracle.oracle import Oracle
        orc = Oracle()
        threads = os.cpu_count() or 1
        t_alg = time.perf_counter()
        if args.precision in (2, 3):
            # the wide formats have no oracle traversal: their node visits are counted
            # on the device by the same traversal one ray per thread (mt_trace_counts)
            from oracle import check
            prays = check.primary_rays(orc, cam, width, height, frame_no(1))
            _, _, cnt = S.trace_counts(prays)
            v_int, tri = float(cnt[:, 0].mean()), float(cnt[:, 1].mean())
            nb = 96 if args.precision == 2 else 64
            alg_bytes = int(width * height * 48 + nb * int(cnt[:, 0].sum()) + 48 * int(cnt[:, 1].sum()))
            visit_src = (f"{'wide-BVH' if args.precision == 2 else '4-wide'} node visits ({nb} B) counted on the "
                         "device (mt_trace_counts)")
        else:
            alg_bytes, v_int, tri = algorithmic_bytes(orc, sc, nodes, bounds, cam, width, height, frame_no(1),
                                                      threads, rec_bytes=32 if args.precision == 1 else 64)
            visit_src = (f"interior visits ({32 if args.precision == 1 else 64} B records) counted by the FP32 oracle "
                         "traversal of the same rays")
        t_alg = time.perf_counter() - t_alg
        peaks = {}
        try:
            peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        except OSError:
            pass
        peak = float(peaks.get("hbm_gbs", 6800.0))
        t_b1 = per_kernel["trace_closest_b1"]
        traffic, traffic_src = None, None
        kp = os.path.join(ROOT, "profiles", "kernels_soup1M_1080p.json")
        kprof = None
        if not args.small and args.workload == "soup" and os.path.exists(kp):
            kprof = json.load(open(kp))
            if kprof.get("precision") != args.precision:
                kprof = None  # captured with another traversal format
        if kprof is not None:
            traffic = kprof["kernels"]["k_trace_closest"]["dram_bytes"]
            traffic_src = "profiles/kernels_soup1M_1080p.json (" + kprof["source"] + ")"
        achieved = alg_bytes / (t_b1 * 1e-3) / 1e9
        per_kernel_roofline = kernel_rooflines(kprof, per_kernel, peak, prof_rays, prof_counts, alg_bytes, t_b1)
        roofline = {"bound": "hbm", "kernel": "k_trace_closest (bounce 1, primary rays)",
                    "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                    "peak_source": "measured" if "hbm_gbs" in peaks else "fallback",
                    "traffic": traffic,
                    "traffic_source": traffic_src,
                    "alg_bytes_per_launch": alg_bytes, "rays_per_launch": width * height,
                    "interior_visits_per_ray": round(v_int, 2), "triangle_tests_per_ray": round(tri, 2),
                    "visit_counts": visit_src,
                    "launch_ms": round(t_b1, 4),
                    "trace_share_of_frame": round(trace_total / frame_total, 3), "per_kernel_ms": per_kernel,
                    "per_kernel": per_kernel_roofline}
        # CPU baseline: the oracle on the host cores, a bounded sample
        cw, ch = width // 4, height // 4
        csc, cn, cb, cenv, clum, csat = sc, nodes, bounds, env, None, None
        from oracle.oracle import ptr
        clum = np.zeros(ENV_W * ENV_H, np.float32)
        csat = np.zeros(ENV_W * ENV_H, np.float32)
        orc.lib.or_env_lum_sat(ptr(cenv), ENV_W, ENV_H, ptr(clum), ptr(csat))
        crays, csec, cframes = cpu_render_rate(orc, csc, cn, cb, cenv, clum, csat, cw, ch, args.cpu_seconds, threads,
                                               cpu_grid(orc, csat))
        cpu_baseline = {"value": round(crays / csec / 1e6, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                        "sample": f"{cframes} frames of {cw}x{ch} (1/16 of the pixels, same scene, camera, depth, RR) "
                                  f"in {threads} threads for {csec:.1f} s; oracle/mt_oracle.cpp (FP32)"}
        # the same job's film against the FP64 oracle, and its parity figures (a check, after the timed region)
        image_error = None
        if not args.no_check:
            image_error = image_check(ctx, S, sc, nodes, bounds, (env, ENV_W, ENV_H) if ENV_ON else None, width,
                                      height, spp, args.inflight, steps=max(1, 16 // spp), orc=orc)
        out = {
            "metric": METRIC, "value": round(value, 2), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (procedural soup and sky; no dataset)",
            "config": config_dict(args.workload, width, height, ntri, world, args.inflight, args.small),
            "rays_per_step": round(total_rays / args.steps / world), "rays_split": rays.tolist(),
            "roofline": roofline, "cpu_baseline": cpu_baseline, "e2e": e2e,
            "gpu_launches": gpu_launches, "clocks": clk,
            "inflight_frames": args.inflight,
            "msamples_per_s": round(width * height * spp * args.steps * world / (ms * 1e-3) / 1e6, 2),
            "bvh_depth": S.depth, "bvh_build_ms": round(bvh_build_ms, 2), "bvh_build": "GPU, level-synchronous",
            "bvh_records": RECORDS[args.precision],
            "alg_bytes_seconds": round(t_alg, 1), "launch_shapes": launch_shapes, "image_error": image_error,
        }
    job.close()
    S.close()
    ctx.close()
    if out is not None and world == 1 and not args.small and args.workload == "soup" and not args.no_arms:
        api.set_tuning(default_shapes)  # the other arms' own launch shapes (run_served installs the merged ones)
        out["batched"], out["plain"] = baseline_metric_arms(args)
        b, pl = out["batched"], out["plain"]
        out["batched_vs_plain"] = round(b["merged_queues"]["mrays_per_s"] / pl["plain_mrays_per_s"], 3)
    if world > 1:
        torch.distributed.destroy_process_group()
    if out is not None:
        print(json.dumps(out), flush=True)


def baseline_metric_arms(args):
    """The workload metric's own arms, run after the timed soup steps: the batched
    configuration (64 jobs of uneven size, soup and stadium, 4 spp) through the
    merged-queue server against the same requests one at a time, with job
    latencies; and the reference's plain wavefront loop (its kernels by name,
    CDeviceGI.loop and CCompact, host-driven) against the fused frame on the same
    soup frames."""
    ns = argparse.Namespace(**vars(args))
    ns.workload, ns.arms = "batched", "served_merged,sequential"
    ns.merged_lanes = ns.merge_streams = None
    r = run_served(ns, emit=False)
    batched = {
        "requests": r["requests"], "samples": r["samples"],
        "merged_queues": {k: r["served_merged"][k] for k in ("lanes", "merge_streams", "mrays_per_s", "p50_ms",
                                                             "p95_ms", "p99_ms", "max_ms", "span_s")},
        "sequential": {k: r["sequential"][k] for k in ("mrays_per_s", "p50_ms", "p95_ms", "p99_ms", "max_ms",
                                                       "span_s")},
        "speedup_vs_sequential": r["speedup_vs_sequential"],
        "config": {k: r["config"][k] for k in ("requests", "resolution", "camera", "max_depth", "rr_from_bounce",
                                               "latency", "equal_error")},
    }
    ns = argparse.Namespace(**vars(args))
    ns.workload, ns.warmup, ns.steps = "plain", 2, 4
    p = run_plain(ns, emit=False)
    plain = {"plain_mrays_per_s": p["value"], "plain_ms_per_frame": p["plain_ms_per_frame"],
             "fused_mrays_per_s": p["fused_mrays_per_s"], "fused_ms_per_frame": p["fused_ms_per_frame"],
             "fused_inflight4_mrays_per_s": p["fused_inflight4_mrays_per_s"],
             "speedup_fused_vs_plain": p["speedup_fused_vs_plain"], "frames": ns.steps,
             "rays_per_frame": p["rays_per_frame"], "config": p["config"]}
    return batched, plain


# --------------------------------------------------- batched and served
def request_list(kind, rng, duration, rate):
    """Requests (arrival s, scene key, width, height, spp, camera seed) of the batched
    configuration (64 jobs at t = 0: soup and stadium alternately, 4 spp) or the served
    one (Poisson arrivals: box room, soup or stadium uniformly, spp in {1, 4, 16, 64});
    pixel counts log-uniform between the configuration's smallest frame and 1920 x 1080,
    aspect 16:9 when the frame is wide enough."""
    out = []
    if kind == "batched":
        lo, n = 128 * 128, 64
        times = np.zeros(n)
    else:
        lo = 64 * 64
        gaps = rng.exponential(1.0 / rate, size=int(rate * duration * 1.5) + 16)
        times = np.cumsum(gaps)
        times = times[times < duration]
        n = len(times)
    hi = 1920 * 1080
    for k in range(n):
        px = float(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        w = int(min(1920, max(8, round(np.sqrt(px * 16 / 9)))))
        h = int(min(1080, max(8, round(px / w))))
        if kind == "batched":
            key, spp = ("soup", "stadium")[k % 2], 4
        else:
            key, spp = ("room", "soup", "stadium")[int(rng.integers(0, 3))], int(rng.choice([1, 4, 16, 64]))
        out.append((float(times[k]), key, w, h, spp, int(rng.integers(0, 2 ** 31))))
    return out


def sphere_camera(seed, width, height, radius=3.0):
    from mambatracer_gb300 import layout
    g = np.random.default_rng(seed).normal(size=3)
    pos = radius * g / np.linalg.norm(g)
    up = (0.0, 1.0, 0.0) if abs(pos[1]) < 0.99 * radius else (1.0, 0.0, 0.0)
    return layout.make_camera(tuple(pos), (0.0, 0.0, 0.0), up, 45.0, width, height)


def run_requests(ctx, S, reqs, lanes, budget, api, merged=0):
    """Submits every request at its arrival time to a server with `lanes` lanes (merged=m:
    sharing wavefront queues on m streams), waits for all; returns the server's stats and
    wall seconds."""
    srv = api.Server(ctx, lanes=lanes, max_width=1920, max_height=1080, max_spp=64, max_depth=DEPTH, rr_depth=RR,
                     film_kahan=1, budget_bytes=budget, merged=merged)
    t0 = time.perf_counter()
    for k, (t, key, w, h, spp, cseed) in enumerate(reqs):
        now = time.perf_counter() - t0
        if t > now:
            time.sleep(t - now)
        srv.submit(S[key], sphere_camera(cseed, w, h), w, h, spp, float(1 + 64 * k), film=False)
    srv.drain()
    wall = time.perf_counter() - t0
    st = srv.stats()
    srv.close()
    return st, wall


def run_served(args, emit=True):
    """Batched (64 uneven jobs at once) or served (Poisson arrivals) rendering through
    the served-mode scheduler, against the same requests run one at a time. Prints
    the JSON line (emit) and returns it."""
    from mambatracer_gb300 import api, build, scenes
    build.build()
    launch_shapes = apply_tuning()  # the built-in launch shapes: the file's are for the soup
    served_shape = {"lanes": 64, "merge_streams": 4, "source": "built-in defaults"}
    if os.path.exists(TUNED):
        from mambatracer_gb300 import tune
        with open(TUNED) as f:
            tuned_file = json.load(f)
        tuned = tuned_file.get("served") if tuned_file.get("device") == tune.device_info() else None
        if tuned:
            served_shape = {"lanes": tuned["lanes"], "merge_streams": tuned["merge_streams"],
                            "source": "autotuned (mambatracer_gb300/tuning_gb300.json)"}
    if args.workload == "served":
        # a request stream keeps thousands queued: more slots fill each merged round
        # (measured on this stream: 64 1287, 96 1348, 128 1390, 160 1418, 192 1429, 256 1436
        # Mrays/s on 4 streams); the batched search above sees only 64 requests
        served_shape = {"lanes": 192, "merge_streams": served_shape["merge_streams"],
                        "source": "measured on the served request stream (192 slots)"}
    if args.merged_lanes is not None or args.merge_streams is not None:
        served_shape = {"lanes": args.merged_lanes or served_shape["lanes"],
                        "merge_streams": args.merge_streams or served_shape["merge_streams"], "source": "command line"}
    launch_shapes["merged_queues"] = served_shape
    ctx = api.Context(0)
    env = scenes.sky_env(ENV_W, ENV_H)
    S = {}
    depth_of = {}
    keys = ("soup", "stadium") if args.workload == "batched" else ("room", "soup", "stadium")
    for key in keys:
        sc = scenes.box_room(64, 64) if key == "room" else make_scene(key, False, W_DEFAULT, H_DEFAULT)
        sc_h = api.Scene(ctx, sc)
        sc_h.build_bvh_device(want_arrays=False)
        if args.precision:
            sc_h.set_precision(args.precision)
        depth_of[key] = sc_h.depth
        if key != "room":
            sc_h.set_env(env, ENV_W, ENV_H)
        S[key] = sc_h
    rng = np.random.default_rng(3 if args.workload == "batched" else 4)
    reqs = request_list(args.workload, rng, args.duration, args.rate)
    budget = int(150e9)
    # warm-up: a few small requests through a one-lane server
    run_requests(ctx, S, [(0.0, k, 64, 64, 1, 1) for k in keys], 1, budget, api)
    res = {}
    arms = set(args.arms.split(",")) | {"served_merged"}
    for name, lanes, merged in (("served_merged", served_shape["lanes"], served_shape["merge_streams"]),
                                ("concurrent", args.lanes, 0), ("sequential", 1, 0)):
        if name not in arms:
            continue
        st, wall = run_requests(ctx, S, reqs, lanes, budget, api, merged)
        rays = int(sum(st["rays"]))
        res[name] = {"lanes": lanes, "merge_streams": merged, "mrays_per_s": round(rays / (st["span_ms"] * 1e-3) / 1e6, 2),
                     "p50_ms": round(st["p50_ms"], 2), "p95_ms": round(st["p95_ms"], 2),
                     "p99_ms": round(st["p99_ms"], 2), "max_ms": round(st["max_ms"], 2),
                     "span_s": round(st["span_ms"] * 1e-3, 3), "wall_s": round(wall, 3),
                     "completed": st["completed"], "max_queue": st["max_queue"], "rays": st["rays"]}
    if args.workload == "batched" and "merged" in arms:
        # merged: each scene's requests as one batch through shared wavefront queues
        t0 = time.perf_counter()
        rays3 = np.zeros(3, np.int64)
        lat = []
        for key in keys:
            frames = [(sphere_camera(cseed, w, h), w, h, spp, float(1 + 64 * k))
                      for k, (t, kk, w, h, spp, cseed) in enumerate(reqs) if kk == key]
            _, r = api.batch_render(ctx, S[key], frames, max_depth=DEPTH, rr_depth=RR, film_kahan=1)
            rays3 += r
            lat += [(time.perf_counter() - t0) * 1e3] * len(frames)
        wall = time.perf_counter() - t0
        lat = np.array(lat)
        res["merged"] = {"mrays_per_s": round(int(rays3.sum()) / wall / 1e6, 2),
                         "p50_ms": round(float(np.percentile(lat, 50)), 2),
                         "p95_ms": round(float(np.percentile(lat, 95)), 2),
                         "p99_ms": round(float(np.percentile(lat, 99)), 2), "max_ms": round(float(lat.max()), 2),
                         "wall_s": round(wall, 3), "batches": len(keys), "rays": rays3.tolist(),
                         "how": "mt_batch_render per scene (its 32 requests through one set of queues), "
                                "queues allocated and films copied to host inside the timed region"}
    pixels = sum(w * h * spp for _, _, w, h, spp, _ in reqs)
    # the scheduler with merged queues (autotuned requests in flight and streams); the batched
    # workload also reports one mt_batch_render call per scene ("merged")
    head = res["served_merged"]
    out = {
        "metric": METRIC, "value": head["mrays_per_s"], "unit": "Mrays/s", "n_gpus": 1,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (procedural scenes and sky; no dataset)",
        "workload": args.workload, "requests": len(reqs), "samples": pixels,
        "latency_ms": {k: head[k] for k in ("p50_ms", "p95_ms", "p99_ms", "max_ms")},
        "served_merged": res["served_merged"], "concurrent": res.get("concurrent"),
        "sequential": res.get("sequential"), "merged": res.get("merged"),
        "speedup_vs_sequential": (round(head["mrays_per_s"] / res["sequential"]["mrays_per_s"], 3)
                                  if "sequential" in res else None),
        "config": {
            "requests": ("64 jobs submitted at once, soup and stadium alternately, 4 spp" if args.workload == "batched"
                         else f"Poisson arrivals at {args.rate}/s for {args.duration} s, box room / soup / stadium "
                              "uniformly, spp in {1, 4, 16, 64}"),
            "resolution": ("pixel count log-uniform 128^2..1920x1080" if args.workload == "batched"
                           else "pixel count log-uniform 64^2..1920x1080"),
            "camera": "uniform on a sphere of radius 3 around the origin, looking at it, fov 45",
            "max_depth": DEPTH, "rr_from_bounce": RR, "semantics": "benchmark (mode 1), full-map environment sampling",
            "admission_budget_bytes": budget, "bvh_depth": depth_of,
            "bvh_records": RECORDS[args.precision],
            "latency": "submission to film in host memory (pinned staging), host clock",
            "equal_error": "the sequential run renders the same requests with the same spp",
            "launch_shapes": launch_shapes,
        },
    }
    for sc_h in S.values():
        sc_h.close()
    ctx.close()
    if emit:
        print(json.dumps(out), flush=True)
    return out


# ------------------------------------------------------ plain wavefront
def run_plain(args, emit=True):
    """The reference's own loop through the kernel-by-name layer (one launch per
    reference kernel, reference buffer layouts, host-driven) against the fused path
    on the same frames: reference semantics (seeds per allocateState call, no
    Russian roulette), the 1M soup and sky at 1920 x 1080, depth 8. Both trace the
    same rays (their films are bit-identical), counted by the fused path."""
    from mambatracer_gb300 import api, build, plain, scenes
    from oracle.oracle import Oracle, bvh_build, ptr
    build.build()
    orc = Oracle()
    ctx = api.Context(0)
    sc = make_scene("soup", False, W_DEFAULT, H_DEFAULT)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    env = scenes.sky_env(ENV_W, ENV_H)
    lum = np.zeros(ENV_W * ENV_H, np.float32)
    sat = np.zeros(ENV_W * ENV_H, np.float32)
    orc.lib.or_env_lum_sat(ptr(env), ENV_W, ENV_H, ptr(lum), ptr(sat))
    rng = np.random.default_rng(17)
    frames = args.warmup + args.steps
    seeds = [rng.integers(2 ** 29, 2 ** 30, size=2 * (1 + 2 * DEPTH)).astype(np.int32) for _ in range(frames)]
    dev = plain.PlainDeviceGI(ctx, sc, nodes, bounds, W_DEFAULT, H_DEFAULT, max_depth=DEPTH,
                              env=(env, lum, sat, ENV_W, ENV_H))
    dev.set_camera(sc.camera)
    for f in range(args.warmup):
        dev.frame(seeds[f], float(f + 1))
    ctx.finish()
    t0 = time.perf_counter()
    for f in range(args.warmup, frames):
        dev.frame(seeds[f], float(f + 1))
    ctx.finish()
    t_plain = time.perf_counter() - t0
    dev.free()
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    S.set_env_with_sat(env, lum, sat, ENV_W, ENV_H)
    res = {}
    for name, inflight in (("fused", 1), ("fused_inflight4", 4)):
        J = api.Job(ctx, S, W_DEFAULT, H_DEFAULT, max_depth=DEPTH, mode=0, film_kahan=0, use_graph=1,
                    inflight=inflight)
        J.set_camera(sc.camera)
        for f in range(args.warmup):
            J.render(seeds[f], float(f + 1))
        ctx.finish()
        J.clear()
        ctx.finish()
        ctx.record(0)
        for f in range(args.warmup, frames):
            J.render(seeds[f], float(f + 1))
        ctx.record(1)
        ctx.finish()
        res[name] = (ctx.elapsed_ms(0, 1) * 1e-3, int(J.total_rays().sum()))
        J.close()
    rays = res["fused"][1]
    out = {
        "metric": METRIC, "workload": "plain", "unit": "Mrays/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "dtype": "f32", "data": "synthetic (procedural soup and sky; no dataset)",
        "value": round(rays / t_plain / 1e6, 2),
        "plain_ms_per_frame": round(t_plain / args.steps * 1e3, 3),
        "fused_mrays_per_s": round(rays / res["fused"][0] / 1e6, 2),
        "fused_ms_per_frame": round(res["fused"][0] / args.steps * 1e3, 3),
        "fused_inflight4_mrays_per_s": round(res["fused_inflight4"][1] / res["fused_inflight4"][0] / 1e6, 2),
        "speedup_fused_vs_plain": round(t_plain / res["fused"][0], 3),
        "rays_per_frame": rays // args.steps,
        "config": {"scene": WORKLOADS["soup"]["scene"], "resolution": f"{W_DEFAULT}x{H_DEFAULT}", "max_depth": DEPTH,
                   "semantics": "reference (mode 0): allocateState seeds, no Russian roulette, Q1/Q2 kept",
                   "plain": "mambatracer_gb300.plain: CDeviceGI.loop + CCompact through mt_launch_1d, wall clock",
                   "fused": "mt_render_frame, one CUDA graph per frame, device clock"},
    }
    S.close()
    ctx.close()
    if emit:
        print(json.dumps(out), flush=True)
    return out


# ------------------------------------------------------- reference arm
def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import build as ob
    from oracle.oracle import Oracle
    ob.build()
    orc = Oracle()
    threads = os.cpu_count() or 1
    sc, nodes, bounds, env, lum, sat = cpu_scene(orc, args.workload)
    grid = cpu_grid(orc, sat)
    width, height = W_DEFAULT // 4, H_DEFAULT // 4
    for _ in range(args.warmup):
        cpu_render_rate(orc, sc, nodes, bounds, env, lum, sat, width, height, 0.0, threads, grid)
    rays = secs = frames = 0
    for _ in range(args.steps):
        r, s, f = cpu_render_rate(orc, sc, nodes, bounds, env, lum, sat, width, height, 0.0, threads, grid)
        rays, secs, frames = rays + r, secs + s, frames + f
    value = rays / secs / 1e6
    sample = (f"each step: {threads} frames of {width}x{height} (1/16 of the 1080p pixels) rendered in parallel, "
              f"one per host thread; oracle/mt_oracle.cpp, the FP32 restatement pinned bit-exact to the reference kernels")
    cfg = config_dict(args.workload, width, height, sc.ntri, world)
    cfg.update({
        "resolution": f"{width}x{height} sample frames (1/16 of the {W_DEFAULT}x{H_DEFAULT} pixels), one per thread",
        "threads": threads,
        "film": "FP32, plain adds (the reference's addAccum order)",
        "launch": "host threads, one frame each; no graphs, no streams",
        "light_grid": (f"{GRID[0]}x{GRID[1]} grid of {GRID[2]}x{GRID[3]}-tile cells, FP32 per-cell SATs in the "
                       "reference's order, initial function (tile integrals of the map), not updated"
                       if ENV_ON else "none"),
        "parallelism": f"{threads} host threads (rank 0 only)",
    })
    if ENV_ON:
        cfg["environment"] = (f"{ENV_W}x{ENV_H} FP32 lat-long sky gradient + 0.5 deg Gaussian sun (peak 5e4); SAT "
                              "built in FP32 in the reference's order")
    cfg.pop("l2", None)
    out = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(secs / args.steps * 1e3, 2),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (procedural soup and sky; no dataset)",
        "config": cfg,
        "cpu_baseline": {"value": round(value, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("the reference's OpenCL kernels need an OpenCL runtime (none on this host: no ICD, no PoCL) and "
                 "its sources do not ship with this repository; its algorithm runs as the oracle restatement, whose "
                 "frames are pinned bit for bit to the reference's kernels compiled as C++. That compiled reference "
                 "(unoptimised: optimised builds of it corrupt memory) renders the same frame 25x slower than the "
                 "restatement at the same optimisation level (oracle/ref/time_ref.py), so this arm overstates the "
                 "reference's own CPU speed"),
    }
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="mambatracer", choices=["mambatracer", "reference"])
    ap.add_argument("--small", action="store_true", help="small case for profiler captures")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-check", action="store_true", help="skip the image-error check against the oracle")
    ap.add_argument("--no-arms", action="store_true", help="skip the batched and plain-wavefront arms")
    ap.add_argument("--inflight", type=int, default=6, help="frames kept in flight on separate streams (1..8)")
    ap.add_argument("--precision", type=int, default=3, choices=[0, 1, 2, 3],
                    help="traversal format: 0 FP32 child boxes (64 B records), 1 FP16 outward-rounded (32 B), 2 wide "
                         "BVH with 8-bit outward-rounded child boxes (96 B nodes), 3 4-wide nodes of a record's "
                         "grandchildren with FP16 outward-rounded boxes (64 B, the default: the same hits up to "
                         "exact-distance ties, fastest)")
    ap.add_argument("--workload", default="soup", choices=sorted(WORKLOADS) + ["batched", "served", "plain"])
    ap.add_argument("--lanes", type=int, default=8, help="batched/served: requests in flight, a stream each")
    ap.add_argument("--merged-lanes", type=int, default=None,
                    help="batched/served: requests sharing the merged queues (default: the autotuned value, else 64)")
    ap.add_argument("--merge-streams", type=int, default=None,
                    help="batched/served: streams of the merged queues (default: the autotuned value, else 4)")
    ap.add_argument("--rate", type=float, default=200.0, help="served: arrivals per second")
    ap.add_argument("--duration", type=float, default=60.0, help="served: seconds of arrivals")
    ap.add_argument("--arms", default="served_merged,concurrent,sequential,merged",
                    help="batched/served: the schedulers to run (served_merged always runs: it is the value)")
    args = ap.parse_args()
    w = WORKLOADS.get(args.workload)
    if w is not None and "depth" in w:  # a workload with its own frame, depth and lighting
        global W_DEFAULT, H_DEFAULT, DEPTH, RR, ENV_ON
        W_DEFAULT, H_DEFAULT, DEPTH, RR, ENV_ON = w["width"], w["height"], w["depth"], w["rr"], w["env"]
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        run_reference(args)
    elif args.workload in ("batched", "served"):
        run_served(args)
    elif args.workload == "plain":
        run_plain(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
