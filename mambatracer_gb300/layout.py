"""Byte layouts of the reference's device structs, as numpy dtypes.

Every struct that crosses the C-ABI keeps MambaTracer's OpenCL layout so a Java
host can pass its `coordinate.struct.Structure` buffers through unchanged:

  Ray           80 B  src/cl/kernel/Util.cl:129-138
  Intersection  96 B  src/cl/kernel/Util.cl:141-151 (84 B padded to 16)
  BVHNode       28 B  src/cl/kernel/NormalBVH.cl:1-11
  BoundingBox   32 B  src/cl/kernel/Util.cl:116-121
  Face          40 B  src/cl/kernel/Util.cl:95-102
  Material     144 B  src/cl/kernel/Bsdf.cl:24-50
  CameraStruct  64 B  src/cl/kernel/Util.cl:78-85
  State         16 B  src/cl/kernel/Sampling.cl:2-6
"""
from __future__ import annotations

import numpy as np

RAY = np.dtype({
    "names": ["o", "d", "inv_d", "sign", "extra", "tMin", "tMax"],
    "formats": [("<f4", 4), ("<f4", 4), ("<f4", 4), ("<i4", 4), ("<i4", 2), "<f4", "<f4"],
    "offsets": [0, 16, 32, 48, 64, 72, 76],
    "itemsize": 80,
})

INTERSECTION = np.dtype({
    "names": ["p", "n", "ng", "d", "uv", "mat", "id", "hit"],
    "formats": [("<f4", 4), ("<f4", 4), ("<f4", 4), ("<f4", 4), ("<f4", 2), "<i4", "<i4", "<i4"],
    "offsets": [0, 16, 32, 48, 64, 72, 76, 80],
    "itemsize": 96,
})

BVH_NODE = np.dtype({
    "names": ["bound", "sibling", "left", "right", "parent", "isLeaf", "child"],
    "formats": ["<i4"] * 7,
    "offsets": [0, 4, 8, 12, 16, 20, 24],
    "itemsize": 28,
})

BOUNDING_BOX = np.dtype({
    "names": ["minimum", "maximum"],
    "formats": [("<f4", 4), ("<f4", 4)],
    "offsets": [0, 16],
    "itemsize": 32,
})

FACE = np.dtype({
    "names": ["vx", "vy", "vz", "uvx", "uvy", "uvz", "nx", "ny", "nz", "mat"],
    "formats": ["<i4"] * 10,
    "offsets": [0, 4, 8, 12, 16, 20, 24, 28, 32, 36],
    "itemsize": 40,
})

MATERIAL = np.dtype({
    "names": ["isDiffuseTexture", "isGlossyTexture", "isRoughnessTexture", "isMirrorTexture",
              "diffuse_color", "diffuse_param", "glossy_color", "glossy_param",
              "mirror_color", "mirror_param", "emission_color", "emission_param"],
    "formats": ["<i4"] * 4 + [("<f4", 4)] * 8,
    "offsets": [0, 4, 8, 12, 16, 32, 48, 64, 80, 96, 112, 128],
    "itemsize": 144,
})

CAMERA = np.dtype({
    "names": ["position", "lookat", "up", "dimension", "fov"],
    "formats": [("<f4", 4), ("<f4", 4), ("<f4", 4), ("<f4", 2), "<f4"],
    "offsets": [0, 16, 32, 48, 56],
    "itemsize": 64,
})

STATE = np.dtype({
    "names": ["seed", "frameCount"],
    "formats": [("<i4", 2), "<f4"],
    "offsets": [0, 8],
    "itemsize": 16,
})

assert RAY.itemsize == 80 and INTERSECTION.itemsize == 96 and BVH_NODE.itemsize == 28
assert BOUNDING_BOX.itemsize == 32 and FACE.itemsize == 40 and MATERIAL.itemsize == 144
assert CAMERA.itemsize == 64 and STATE.itemsize == 16


def default_material() -> np.ndarray:
    """CSurfaceParameter2 defaults (src/cl/struct/CSurfaceParameter2.java:33-48)."""
    m = np.zeros((), dtype=MATERIAL)
    m["diffuse_color"] = (0.95, 0.95, 0.95, 1.0)
    m["diffuse_param"] = (1.0, 0.0, 0.0, 0.0)
    m["glossy_color"] = (0.95, 0.95, 0.95, 1.0)
    m["mirror_color"] = (0.95, 0.95, 0.95, 1.0)
    m["emission_color"] = (1.0, 1.0, 1.0, 1.0)
    return m


def make_camera(position, lookat, up, fov_deg, width=0, height=0) -> np.ndarray:
    """CameraStruct from CCameraModel.getCameraStruct (src/cl/struct/CCameraModel.java:31-40);
    points and vectors carry w = 0 (src/cl/data/CPoint3.java:65-67)."""
    c = np.zeros((), dtype=CAMERA)
    c["position"] = (*position, 0.0)
    c["lookat"] = (*lookat, 0.0)
    c["up"] = (*up, 0.0)
    c["dimension"] = (width, height)
    c["fov"] = fov_deg
    return c


def make_rays(o: np.ndarray, d: np.ndarray, tmin: float = 0.001, tmax: float = np.inf) -> np.ndarray:
    """Rays as initGlobalRay (src/cl/kernel/Util.cl:577-587) fills them."""
    n = o.shape[0]
    r = np.zeros(n, dtype=RAY)
    r["o"][:, :3] = o
    r["d"][:, :3] = d
    with np.errstate(divide="ignore"):
        inv = np.float32(1.0) / d.astype(np.float32)
    r["inv_d"][:, :3] = inv
    r["sign"][:, :3] = (inv < 0).astype(np.int32)
    r["tMin"] = np.float32(tmin)
    r["tMax"] = np.float32(tmax)
    return r
