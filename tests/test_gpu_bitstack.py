"""The stackless traversal (MT_TRAVERSAL=bitstack, read once per process, so it
runs in a child process): the reference's own algorithm, a 64-bit bitstack with
parent links and no deferred-node stack (src/cl/kernel/NormalBVH.cl:14-92).

Its hits are the reference's bit for bit (golden outputs of the reference's
kernels; the oracle on a 200k soup and on axis-aligned rays through the box
room), its work is the reference's exactly (interior visits and triangle tests
per ray equal the oracle's counts: it has no culling of deferred nodes), and a
frame rendered with it equals the frame rendered with the stack traversal."""
import os
import subprocess
import sys

import numpy as np
import pytest

from mambatracer_gb300 import api, layout, scenes
from tests.helpers import bvh_build, oracle_any, oracle_trace

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _child(tmp_path, script):
    path = str(tmp_path / "child.py")
    with open(path, "w") as f:
        f.write(script)
    env = dict(os.environ, MT_TRAVERSAL="bitstack")
    subprocess.run([sys.executable, path], env=env, check=True, timeout=900, cwd=ROOT)


_SCRIPT = r"""
import sys, numpy as np
sys.path.insert(0, {root!r})
from mambatracer_gb300 import api, layout, scenes
from oracle.oracle import Oracle, bvh_build
from tests.golden.make_golden import golden_inputs
from tests.test_gpu_bitstack import cases, frame
out = {{}}
orc = Oracle()
ctx = api.Context(0)
g = golden_inputs()
sc = g["soup"]
nodes, bounds, _, _ = bvh_build(orc, sc)
S = api.Scene(ctx, sc)
S.import_bvh(nodes, bounds)
for key in ("rays_in", "rays_out"):
    out[key + "_t"], out[key + "_p"] = S.trace_closest(g[key])
out["rays_shadow_occ"] = S.trace_any(g["rays_shadow"])
S.close()
for name, (sc, rays, srays) in cases().items():
    nodes, bounds, _, _ = bvh_build(orc, sc)
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    for prec in (0, 1):
        S.set_precision(prec)
        out[f"{{name}}_{{prec}}_t"], out[f"{{name}}_{{prec}}_p"] = S.trace_closest(rays)
        out[f"{{name}}_{{prec}}_any"] = S.trace_any(srays)
        out[f"{{name}}_{{prec}}_counts"] = S.trace_counts(rays[:20000])[2]
    S.close()
out["frame"] = frame(ctx)
np.savez({out!r}, **out)
"""


def cases():
    """Scenes and rays of the comparison: a 200k soup (rays inside), and the box
    room with zero direction components and origins on box planes."""
    soup = scenes.soup(200000, seed=41, extent=0.6, edge_sigma=0.01)
    o, d = scenes.random_rays(soup, 100000, seed=42, inside=True)
    room = scenes.box_room(8, 8)
    rng = np.random.default_rng(3)
    n = 20000
    ro = rng.uniform(-0.2, 1.2, size=(n, 3)).astype(np.float32)
    ro[: n // 4, 0] = 0.5
    ro[n // 4: n // 2, 1] = 0.0
    rd = rng.normal(size=(n, 3))
    rd /= np.linalg.norm(rd, axis=1, keepdims=True)
    rd = rd.astype(np.float32)
    rd[::3, 0] = 0.0
    rd[1::3, 1] = 0.0
    rd[2::5, 2] = 0.0
    rd[::7] = np.array([0.0, 0.0, -1.0], np.float32)
    return {
        "soup": (soup, layout.make_rays(o, d), layout.make_rays(o, d, tmin=1e-4, tmax=0.2)),
        "room": (room, layout.make_rays(ro, rd), layout.make_rays(ro, rd, tmin=1e-4, tmax=0.3)),
    }


def frame(ctx):
    """Four benchmark-semantics frames of a 20k soup under the sky (FP16 records)."""
    from oracle.oracle import Oracle, bvh_build
    sc = scenes.soup(20000, seed=8, extent=0.8, width=96, height=64)
    nodes, bounds, _, _ = bvh_build(Oracle(), sc)
    S = api.Scene(ctx, sc)
    S.import_bvh(nodes, bounds)
    S.set_precision(1)
    S.set_env(scenes.sky_env(256, 128), 256, 128)
    J = api.Job(ctx, S, 96, 64, max_depth=6, mode=1, rr_depth=3, film_kahan=1, use_graph=1, inflight=1)
    J.set_camera(sc.camera)
    for f in range(4):
        J.render(None, float(f + 1))
    film = J.film()
    J.close()
    S.close()
    return film


def test_stackless_traversal_is_the_reference(ctx, orc, golden, tmp_path):
    out_path = str(tmp_path / "bitstack.npz")
    _child(tmp_path, _SCRIPT.format(root=ROOT, out=out_path))
    got = dict(np.load(out_path))
    for key in ("rays_in", "rays_out"):
        assert np.array_equal(got[key + "_p"], golden[key + "_id"]), key
        assert got[key + "_t"].tobytes() == golden[key + "_tmax"].tobytes(), key
    assert np.array_equal(got["rays_shadow_occ"], golden["rays_shadow_occ"])
    for name, (sc, rays, srays) in cases().items():
        nodes, bounds, _, _ = bvh_build(orc, sc)
        to, po, oc = oracle_trace(orc, sc, nodes, bounds, rays, counts=True)
        ao = oracle_any(orc, sc, nodes, bounds, srays)
        _, _, oc20 = oracle_trace(orc, sc, nodes, bounds, np.ascontiguousarray(rays[:20000]), counts=True)
        for prec in (0, 1):
            t, p = got[f"{name}_{prec}_t"], got[f"{name}_{prec}_p"]
            assert t.tobytes() == to.tobytes(), (name, prec)
            assert np.array_equal(p, po) if prec == 0 else (p != po).sum() <= 1e-4 * len(p), (name, prec)
            assert np.array_equal(got[f"{name}_{prec}_any"], ao), (name, prec)
        # the reference's work, visit for visit (FP32 records)
        assert np.array_equal(got[f"{name}_0_counts"], oc20), name
    # the frame equals the stack traversal's (this process)
    assert got["frame"].tobytes() == frame(ctx).tobytes()
