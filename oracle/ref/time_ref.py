"""Times the reference's own kernels (compiled as C++, oracle/_ref) against the
oracle restatement (oracle/mt_oracle.cpp) on the same frame, single-threaded.

Test infrastructure, run by hand where the reference tree is present (the
machine that runs the benchmark has no reference sources):

    python -m oracle.ref.time_ref [--ntri N] [--width W] [--height H] [--frames F]

The frame is the reference's semantics (CDeviceGI.loop: allocateState seeds,
no Russian roulette) on the triangle soup under the sky environment (full-map
sampling, the reference's own path), depth 8. The reference's translation unit
runs only unoptimised: built with -O1 or -O2 it corrupts memory (its sources
leave behaviour undefined that -O0 happens to tolerate, e.g. non-void functions
that flow off their end). So the oracle is also built at -O0 (into
oracle/_ref/liboracle_O0.so) and the two are compared at the same optimisation
level, beside the -O2 oracle that the CPU baseline times. The script checks that
all three frames are bit-identical, then prints one JSON line of times and ratios.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def main():
    import ctypes as C

    from mambatracer_gb300 import scenes
    from oracle.oracle import Oracle, RefOracle, bvh_build, ptr
    from oracle.ref import make_ref

    ap = argparse.ArgumentParser()
    ap.add_argument("--ntri", type=int, default=1_000_000)
    ap.add_argument("--width", type=int, default=192)
    ap.add_argument("--height", type=int, default=108)
    ap.add_argument("--frames", type=int, default=3)
    ap.add_argument("--depth", type=int, default=8)
    args = ap.parse_args()
    if not make_ref.build():
        print(json.dumps({"unavailable": "reference sources not present"}))
        return
    import subprocess

    from oracle import build as ob
    orc = Oracle()
    ref0 = RefOracle()
    lib_o0 = os.path.join(make_ref.OUT, "liboracle_O0.so")
    subprocess.run(["g++", "-std=c++20", "-O0", "-fPIC", "-shared", "-fwrapv", "-ffp-contract=off", "-fno-fast-math",
                    *ob.SRC, "-o", lib_o0], check=True)
    port0 = C.CDLL(lib_o0)
    port0.or_render_frame.restype = orc.lib.or_render_frame.restype
    port0.or_render_frame.argtypes = orc.lib.or_render_frame.argtypes

    sc = scenes.soup(args.ntri, seed=1, width=args.width, height=args.height)
    nodes, bounds, _, _ = bvh_build(orc, sc)
    ew, eh = 2048, 1024
    env = scenes.sky_env(ew, eh)
    lum = np.zeros(ew * eh, np.float32)
    sat = np.zeros(ew * eh, np.float32)
    orc.lib.or_env_lum_sat(ptr(env), ew, eh, ptr(lum), ptr(sat))
    cam = sc.camera.copy()
    W, H, D = args.width, args.height, args.depth
    rng = np.random.default_rng(5)
    seeds = [rng.integers(2 ** 29, 2 ** 30, size=2 * (1 + 2 * D)).astype(np.int32) for _ in range(args.frames)]

    def run(kind):
        acc = np.zeros((W * H, 4), np.float32)
        counts = []
        t0 = time.perf_counter()
        for f, s in enumerate(seeds):
            c = np.zeros(D, np.int32)
            common = (ptr(cam), W, H, D)
            tail = (ptr(s), float(f + 1), ptr(sc.points), ptr(sc.uvs), ptr(sc.normals), ptr(sc.faces), sc.ntri,
                    ptr(sc.materials), ptr(nodes), ptr(bounds), ptr(env), ptr(lum), ptr(sat), ew, eh, 1)
            if kind == "ref_O0":
                ref0.lib.ref_render_frame(*common, *tail, ptr(acc), ptr(c))
            else:
                (port0 if kind == "port_O0" else orc.lib).or_render_frame(*common, 0, 0, *tail, 0, ptr(acc), ptr(c),
                                                                          None)
            counts.append(c)
        secs = time.perf_counter() - t0
        c = np.stack(counts)
        return acc, c, secs, None

    res = {k: run(k) for k in ("ref_O0", "port_O0", "port_O2")}
    a0 = res["ref_O0"]
    for k in ("port_O0", "port_O2"):
        assert res[k][0].tobytes() == a0[0].tobytes() and np.array_equal(res[k][1], a0[1]), f"{k} differs"
    out = {"frame": f"soup {args.ntri} triangles, {W}x{H}, depth {D}, sky environment, reference semantics",
           "frames": args.frames, "threads": 1, "films_bit_identical": True}
    for k, (_, _, secs, _) in res.items():
        out[f"{k}_seconds"] = round(secs, 3)
    out["ref_O0_over_port_O0_time"] = round(res["ref_O0"][2] / res["port_O0"][2], 3)
    out["port_O0_over_port_O2_time"] = round(res["port_O0"][2] / res["port_O2"][2], 3)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
