"""The OBJ ingest path (mt_obj_parse; TracerAPI.initMesh, src/cl/ui/fx/main/
TracerAPI.java:393-438, feeds CMesh from an OBJ parser): the reference's mesh
arrays from OBJ text, on hand-checked cases."""
import ctypes as C

import numpy as np
import pytest

from mambatracer_gb300 import _lib, api, scenes

# A unit quad floor (a polygon split into a fan), a textured and shaded triangle
# with negative indices, and a second object; comments and ignored statements.
OBJ = """# a test scene
mtllib scene.mtl
v 0 0 0
v 1 0 0
v 1 0 1
v 0 0 1
vn 0 1 0
o floor
usemtl grey
s off
f 1//1 2//1 3//1 4//1   # quad
v 0 1 0
v 1 1 0
v 0 2 0
vt 0 0
vt 1 0
vt 0 1
vn 0 0 -1
o panel.001
f -3/-3/-1 -2/-2/-1 -1/-1/-1
o floor
f 1 3 4
"""


def test_obj_arrays():
    sc = scenes.from_obj(OBJ)
    assert sc.points.shape == (7, 4) and not sc.points[:, 3].any()
    assert np.array_equal(sc.points[:4, :3], [[0, 0, 0], [1, 0, 0], [1, 0, 1], [0, 0, 1]])
    assert sc.uvs.shape == (3, 2) and sc.normals.shape == (2, 4)
    f = sc.faces
    assert len(f) == 4
    # the quad as a fan (1 2 3), (1 3 4), normals from the v//vn corners, no uvs
    assert [tuple(f[k][["vx", "vy", "vz"]]) for k in range(2)] == [(0, 1, 2), (0, 2, 3)]
    assert (f["nx"][:2] == 0).all() and (f["uvx"][:2] == -1).all()
    # the panel: negative indices resolve to the last three points, uvs and the last normal
    assert tuple(f[2][["vx", "vy", "vz"]]) == (4, 5, 6)
    assert tuple(f[2][["uvx", "uvy", "uvz"]]) == (0, 1, 2)
    assert tuple(f[2][["nx", "ny", "nz"]]) == (1, 1, 1)
    # materials by object name in order of first appearance; group in the high bits
    assert list(f["mat"] & 0xFFFF) == [0, 0, 1, 0] and list(f["mat"] >> 16) == [0, 0, 1, 0]
    assert sc.materials.shape[0] == 2


def test_obj_faces_before_any_name():
    sc = scenes.from_obj("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\ng a\nf 3 2 1\ng b\nf 1 3 2\ng a\nf 2 1 3\n")
    assert list(sc.faces["mat"] & 0xFFFF) == [0, 1, 2, 1]


@pytest.mark.parametrize("text,what", [("v 0 0\n", "coordinate"), ("v 0 0 0\nf 1 2 3\n", "vertex index"),
                                       ("v 0 0 0\nv 1 0 0\nf 1 2\n", "three corners"),
                                       ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1/5 2 3\n", "texture index"),
                                       ("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 0 1 2\n", "vertex index")])
def test_obj_errors(text, what):
    counts = np.zeros(5, np.int32)
    rc = _lib.lib().mt_obj_parse(text.encode(), len(text), counts.ctypes.data_as(C.c_void_p), None, None, None, None)
    assert rc == -1
    msg = _lib.lib().mt_last_error()
    assert what.encode() in msg and b"line" in msg


def test_obj_scene_builds_a_bvh():
    sc = scenes.from_obj(OBJ)
    nodes, bounds, depth = api.bvh_build_host(sc)
    assert nodes.shape[0] == 2 * sc.ntri - 1 and depth >= 1


def _reference_cornell_box():
    """The default scene's OBJ text as TracerAPI.initDefaultMesh spells it
    (TracerAPI.java:205-318), read from the reference tree where it exists (the
    tree the reference-kernel recipe reads)."""
    import os
    import re

    from oracle.ref.make_ref import REF_ROOT
    REF_TRACER_API = os.path.join(REF_ROOT, "src", "cl", "ui", "fx", "main", "TracerAPI.java")
    if not os.path.exists(REF_TRACER_API):
        pytest.skip("reference tree not present")
    src = open(REF_TRACER_API, encoding="latin-1").read()
    start = src.index("String cube =")
    end = src.index(";", start)
    pieces = re.findall(r'"((?:[^"\\]|\\.)*)"', src[start:end])
    return "".join(p.replace("\\n", "\n") for p in pieces)


def test_reference_default_scene():
    """The reference's own default mesh: 8 objects whose materials its caller
    numbers 0 floor, 1 ceiling, 2 back wall, 3 right wall, 4 small box, 5 tall
    box, 6 emitter, 7 left wall (TracerAPI.java:325-335), quads split into
    triangles, one normal per face corner."""
    text = _reference_cornell_box()
    sc = scenes.from_obj(text)
    mats = sc.faces["mat"] & 0xFFFF
    assert sc.materials.shape[0] == 8
    assert sorted(set(mats.tolist())) == list(range(8))
    assert (sc.faces["nx"] >= 0).all() and (sc.faces["uvx"] == -1).all()
    # the emitter (material 6) is the small quad just under the ceiling
    light = sc.points[np.concatenate([sc.faces[mats == 6][k] for k in ("vx", "vy", "vz")]), :3]
    ceiling = sc.points[np.concatenate([sc.faces[mats == 1][k] for k in ("vx", "vy", "vz")]), :3]
    assert len(sc.faces[mats == 6]) == 2
    assert light[:, 1].max() < ceiling[:, 1].min() and light[:, 1].min() > 0.9
    # every quad of the text became two triangles
    quads = sum(1 for line in text.splitlines() if line.startswith("f ") and len(line.split()) == 5)
    tris = sum(1 for line in text.splitlines() if line.startswith("f ") and len(line.split()) == 4)
    assert sc.ntri == 2 * quads + tris
