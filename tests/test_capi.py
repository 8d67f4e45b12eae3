"""The C-ABI library without a GPU: it loads, exports every entry point the
header declares, its host-side BVH build equals the oracle's (and so the
reference layout), and argument errors come back as MT_ERR_* codes."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from mambatracer_gb300 import _lib, api, scenes
from tests.helpers import bvh_build, ptr

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    text = open(os.path.join(ROOT, "include", "mambatracer.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mt_[a-z0-9_]+)\s*\(", text)))


def test_library_loads_and_exports_the_header():
    L = _lib.lib()
    syms = header_symbols()
    assert len(syms) >= 40
    missing = [s for s in syms if not hasattr(L, s)]
    assert not missing, missing
    # every declared entry point has a ctypes signature in the binding
    assert set(syms) <= set(_lib.SIGNATURES)
    assert b"sm_103a" in L.mt_version()


@pytest.mark.parametrize("make", [lambda: scenes.box_room(8, 8), lambda: scenes.soup(50000, seed=9)])
def test_host_bvh_build_equals_oracle(orc, make):
    """CNormalBVH.build (src/cl/scene/CNormalBVH.java:45-148): product and oracle agree bit for bit."""
    sc = make()
    n1, b1, d1 = api.bvh_build_host(sc)
    n2, b2, d2, _ = bvh_build(orc, sc)
    assert np.array_equal(n1, n2)
    assert b1.tobytes() == b2.tobytes()
    assert d1 == d2
    # layout invariants of the reference: 2N-1 nodes, node.bound = index, siblings adjacent
    assert n1.shape[0] == 2 * sc.ntri - 1
    assert (n1[:, 0] == np.arange(n1.shape[0])).all()
    interior = n1[:, 5] == 0
    assert (n1[interior, 3] == n1[interior, 2] + 1).all()
    leaves = n1[~interior, 6]
    assert sorted(leaves.tolist()) == list(range(sc.ntri))


def test_host_bvh_rejects_bad_faces():
    sc = scenes.box_room(8, 8)
    faces = sc.faces.copy()
    faces["vy"][3] = 10 ** 6
    n = sc.ntri
    nodes = np.zeros((2 * n - 1, 7), np.int32)
    bounds = np.zeros((2 * n - 1, 8), np.float32)
    d = C.c_int()
    rc = _lib.lib().mt_bvh_build_host(ptr(sc.points), sc.points.shape[0], ptr(faces), n, ptr(nodes), ptr(bounds),
                                      C.byref(d))
    assert rc == -1
    assert b"face 3" in _lib.lib().mt_last_error()


def test_null_arguments_are_errors():
    L = _lib.lib()
    assert L.mt_ctx_create(0, None) == -1
    assert L.mt_finish(None) == -1
    assert L.mt_buf_write(None, 0, None, 0) == -1
    assert L.mt_job_stats(None, None, None) == -1
    assert L.mt_trace_closest(None, None, 0, None, None) == -1
    assert L.mt_job_launches(None, None) == -1
    assert L.mt_scene_set_bvh_precision(None, 3) == -1


def test_single_triangle_bvh():
    sc = scenes.box_room(8, 8)
    one = scenes.Scene(points=sc.points[:3].copy(), faces=sc.faces[:1].copy(), materials=sc.materials)
    nodes, bounds, depth = api.bvh_build_host(one)
    assert nodes.shape == (1, 7) and nodes[0, 5] == 1 and nodes[0, 6] == 0 and depth == 0
