"""Procedural scenes and environment maps for the benchmark configurations.

Scenes are built as the reference's host arrays (src/cl/scene/CMesh.java:339-357):
points float4 (w = 0), uvs float2, normals float4, faces 10 x int32 with
`mat = group << 16 | material`, materials 144 B each. Synthetic throughout; the
generators are seeded so every run sees the same scene.

  box_room      the box room (36 triangles, 256 x 256, depth 4)
  textured_room the box room with texture images on the floor, a wall and the boxes
  from_obj      a scene from Wavefront OBJ text (the library's OBJ reader)
  soup          uniform triangle soup (1M triangles) in [-1, 1]^3
  stadium       ground plane of 2M triangles plus a displaced icosphere
  sky_env       zenith-to-horizon gradient plus a Gaussian sun, lat-long FP32 RGB

Material conventions (stated because the reference leaves them open): GGX
"roughness r" is the alpha of the GGX lobe, glossy_param.y = glossy_param.z = r
(no squaring); F0 0.04 is glossy_color = 0.04 with glossy scale 1. Per-triangle
roughness/albedo draws are quantised to a 64 x 64 palette because the reference
encodes the material index in 16 bits (src/cl/kernel/Util.cl:11-14).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from .layout import FACE, default_material, make_camera


@dataclass
class Scene:
    points: np.ndarray            # float32 [V, 4]
    faces: np.ndarray             # FACE [N]
    materials: np.ndarray         # MATERIAL [M]
    uvs: np.ndarray = field(default_factory=lambda: np.zeros((1, 2), np.float32))
    normals: np.ndarray = field(default_factory=lambda: np.zeros((1, 4), np.float32))
    camera: np.ndarray | None = None
    name: str = ""
    # texture images: (material, kind 0 diffuse / 1 glossy / 2 roughness / 3 mirror,
    # ARGB int32 [H, W] in PixelReader.getArgb order)
    textures: list = field(default_factory=list)

    @property
    def ntri(self) -> int:
        return int(self.faces.shape[0])


def _faces(tri_idx: np.ndarray, mat: np.ndarray) -> np.ndarray:
    f = np.zeros(tri_idx.shape[0], dtype=FACE)
    f["vx"], f["vy"], f["vz"] = tri_idx[:, 0], tri_idx[:, 1], tri_idx[:, 2]
    f["uvx"] = f["uvy"] = f["uvz"] = -1
    f["nx"] = f["ny"] = f["nz"] = -1
    f["mat"] = mat.astype(np.int32)
    return f


def _points(p: np.ndarray) -> np.ndarray:
    out = np.zeros((p.shape[0], 4), np.float32)
    out[:, :3] = p
    return out


def _material(diffuse=(0.75, 0.75, 0.75), glossy=None, alpha=0.0, emission=None, power=0.0):
    m = default_material()
    m["diffuse_color"] = (*diffuse, 1.0)
    m["diffuse_param"] = (1.0, 0.0, 0.0, 0.0)
    if glossy is not None:
        m["glossy_color"] = (glossy, glossy, glossy, 1.0)
        m["glossy_param"] = (1.0, alpha, alpha, 0.0)
    if emission is not None:
        m["emission_color"] = (*emission, 1.0)
        m["emission_param"] = (1.0, power, 0.0, 0.0)
    return m


def _quad(p0, p1, p2, p3):
    return [(p0, p1, p2), (p0, p2, p3)]


def _box(center, size, height, angle_deg):
    cx, cz = center
    h = size / 2.0
    a = math.radians(angle_deg)
    ca, sa = math.cos(a), math.sin(a)

    def pt(x, y, z):
        return (cx + ca * x + sa * z, y, cz - sa * x + ca * z)

    c = [pt(-h, 0, -h), pt(h, 0, -h), pt(h, 0, h), pt(-h, 0, h),
         pt(-h, height, -h), pt(h, height, -h), pt(h, height, h), pt(-h, height, h)]
    tris = []
    tris += _quad(c[0], c[1], c[2], c[3])  # bottom
    tris += _quad(c[4], c[7], c[6], c[5])  # top
    tris += _quad(c[0], c[4], c[5], c[1])  # sides
    tris += _quad(c[1], c[5], c[6], c[2])
    tris += _quad(c[2], c[6], c[7], c[3])
    tris += _quad(c[3], c[7], c[4], c[0])
    return tris


def box_room(width=256, height=256) -> Scene:
    """Unit-cube room: 5 quads (grey 0.75, red left wall, green right wall), two
    boxes of side 0.3 and 0.6 rotated +15 / -18 degrees about y (GGX r 0.3,
    F0 0.04 over a 0.75 grey base), a 0.25 x 0.25 ceiling emitter of radiance 15.
    36 triangles. Pinhole camera, vertical fov 40 degrees."""
    tris, mats = [], []
    room = [
        (_quad((0, 0, 0), (0, 0, 1), (1, 0, 1), (1, 0, 0)), 0),      # floor
        (_quad((0, 1, 0), (1, 1, 0), (1, 1, 1), (0, 1, 1)), 0),      # ceiling
        (_quad((0, 0, 0), (1, 0, 0), (1, 1, 0), (0, 1, 0)), 0),      # back
        (_quad((0, 0, 0), (0, 1, 0), (0, 1, 1), (0, 0, 1)), 1),      # left (red)
        (_quad((1, 0, 0), (1, 0, 1), (1, 1, 1), (1, 1, 0)), 2),      # right (green)
    ]
    for quad, m in room:
        for t in quad:
            tris.append(t)
            mats.append(m)
    for t in _box((0.68, 0.62), 0.3, 0.3, 15.0):
        tris.append(t)
        mats.append(3)
    for t in _box((0.33, 0.36), 0.6 * 0.5, 0.6, -18.0):
        tris.append(t)
        mats.append(3)
    e0, e1 = 0.5 - 0.125, 0.5 + 0.125
    y = 0.999
    for t in _quad((e0, y, e0), (e1, y, e0), (e1, y, e1), (e0, y, e1)):
        tris.append(t)
        mats.append(4)
    pts = np.array([v for t in tris for v in t], np.float32)
    idx = np.arange(pts.shape[0], dtype=np.int32).reshape(-1, 3)
    materials = np.stack([
        _material((0.75, 0.75, 0.75)),
        _material((0.75, 0.1, 0.1)),
        _material((0.1, 0.75, 0.1)),
        _material((0.75, 0.75, 0.75), glossy=0.04, alpha=0.3),
        _material((0.75, 0.75, 0.75), emission=(1.0, 1.0, 1.0), power=15.0),
    ])
    cam = make_camera((0.5, 0.5, 2.35), (0.5, 0.5, 0.0), (0.0, 1.0, 0.0), 40.0, width, height)
    return Scene(points=_points(pts), faces=_faces(idx, np.array(mats)), materials=materials,
                 camera=cam, name="box_room")


def _argb(r, g, b, a=None) -> np.ndarray:
    """float channels in [0, 1] -> 0xAARRGGBB int32 (8 bits each, rounded)."""
    q = lambda c: np.clip(np.rint(np.asarray(c, np.float64) * 255.0), 0, 255).astype(np.uint32)
    a = np.ones_like(np.asarray(r, np.float64)) if a is None else a
    return ((q(a) << 24) | (q(r) << 16) | (q(g) << 8) | q(b)).astype(np.uint32).view(np.int32)


def textured_room(width=128, height=96, seed=3) -> Scene:
    """The box room with texture images (CTextureApplyPass's inputs): the floor
    (material 5) a 64 x 64 diffuse checkerboard tiled three times (uvs 0..3); the
    red left wall a 40 x 24 diffuse stripe image read at negative uvs (-1.3..0.7,
    wrapped by the reference's domain rule); the boxes (no uvs: the hit's
    barycentric coordinates index the images) a 32 x 16 glossy colour ramp and a
    16 x 16 roughness noise image (red = ax, green = ay)."""
    sc = box_room(width, height)
    faces = sc.faces.copy()
    n = faces.shape[0]
    uvs = np.zeros((3 * n, 2), np.float32)
    # floor: triangles 0, 1 (points (0,0,0),(0,0,1),(1,0,1) and (0,0,0),(1,0,1),(1,0,0)); uv = 3 * (x, z)
    # left wall: triangles 6, 7 (x = 0); uv = 2 * (z, y) - (1.3, 1.3)
    for t in range(n):
        p = sc.points[[faces["vx"][t], faces["vy"][t], faces["vz"][t]], :3]
        if t in (0, 1):
            uvs[3 * t:3 * t + 3] = 3.0 * p[:, [0, 2]]
        elif t in (6, 7):
            uvs[3 * t:3 * t + 3] = 2.0 * p[:, [2, 1]] - 1.3
        else:
            continue
        faces["uvx"][t], faces["uvy"][t], faces["uvz"][t] = 3 * t, 3 * t + 1, 3 * t + 2
    mats = faces["mat"].copy()
    mats[0:2] = 5
    faces["mat"] = mats
    materials = np.concatenate([sc.materials, sc.materials[:1].copy()])
    materials[5]["isDiffuseTexture"] = 1
    materials[1]["isDiffuseTexture"] = 1
    materials[3]["isGlossyTexture"] = 1
    materials[3]["isRoughnessTexture"] = 1
    rng = np.random.default_rng(seed)
    yy, xx = np.mgrid[0:64, 0:64]
    chk = ((xx // 8 + yy // 8) % 2).astype(np.float64)
    floor = _argb(0.15 + 0.7 * chk, 0.15 + 0.6 * chk, 0.2 + 0.5 * (1 - chk))
    yy, xx = np.mgrid[0:24, 0:40]
    stripe = ((xx // 5) % 2).astype(np.float64)
    wall = _argb(0.8 * stripe + 0.1, 0.1 + 0.2 * yy / 23.0, 0.1 + 0.1 * stripe)
    yy, xx = np.mgrid[0:16, 0:32]
    ramp = _argb(0.02 + 0.5 * xx / 31.0, 0.04 + 0.3 * yy / 15.0, np.full(xx.shape, 0.3))
    rough = _argb(rng.uniform(0.02, 0.9, (16, 16)), rng.uniform(0.02, 0.9, (16, 16)), np.zeros((16, 16)))
    return Scene(points=sc.points, faces=faces, materials=materials, uvs=uvs, camera=sc.camera,
                 name="textured_room", textures=[(5, 0, floor), (1, 0, wall), (3, 1, ramp), (3, 2, rough)])


def from_obj(text: str | bytes, materials: np.ndarray | None = None, camera: np.ndarray | None = None,
             name: str = "obj") -> Scene:
    """A scene from Wavefront OBJ text through the library's reader (mt_obj_parse,
    the ingest path of TracerAPI.initMesh). Each `o`/`g` name is a material; with
    `materials` None every one is the default grey diffuse (0.75)."""
    import ctypes as C

    from ._lib import check, lib
    data = text.encode() if isinstance(text, str) else bytes(text)
    counts = np.zeros(5, np.int32)
    p = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)  # noqa: E731
    check(lib().mt_obj_parse(data, len(data), p(counts), None, None, None, None))
    npt, nuv, nnr, nf, nmat = (int(x) for x in counts)
    pts = np.zeros((max(npt, 1), 4), np.float32)
    uvs = np.zeros((max(nuv, 1), 2), np.float32)
    nrm = np.zeros((max(nnr, 1), 4), np.float32)
    faces = np.zeros(nf, dtype=FACE)
    check(lib().mt_obj_parse(data, len(data), p(counts), p(pts), p(uvs), p(nrm), p(faces)))
    if materials is None:
        materials = np.stack([_material((0.75, 0.75, 0.75)) for _ in range(max(nmat, 1))])
    return Scene(points=pts, faces=faces, materials=materials, uvs=uvs, normals=nrm, camera=camera, name=name)


def texture_tables(sc: Scene) -> tuple[np.ndarray, np.ndarray]:
    """The scene's images as one ARGB texel pool and the per-material table of
    (first texel, width, height, 0) for kinds 0..3 (width 0: no image), int32
    [M * 4, 4] -- the layout of the textureApplyPass kernel's arguments."""
    nmat = sc.materials.shape[0]
    table = np.zeros((nmat * 4, 4), np.int32)
    pool, off = [], 0
    for m, kind, img in sc.textures:
        img = np.ascontiguousarray(img, np.int32)
        table[4 * m + kind] = (off, img.shape[1], img.shape[0], 0)
        pool.append(img.reshape(-1))
        off += img.size
    texels = np.concatenate(pool) if pool else np.zeros(1, np.int32)
    return texels, table


def _palette_materials(levels=64, glossy_fraction=1.0):
    """64 x 64 palette: roughness r in [0.05, 0.8] x albedo a in [0.2, 0.9]."""
    mats = []
    for ri in range(levels):
        r = 0.05 + 0.75 * (ri + 0.5) / levels
        for ai in range(levels):
            a = 0.2 + 0.7 * (ai + 0.5) / levels
            mats.append(_material((a, a, a), glossy=0.04, alpha=r))
    return np.stack(mats)


def soup(ntri=1_000_000, seed=1, width=1920, height=1080, extent=1.0, edge_sigma=0.005) -> Scene:
    """Triangle soup: centroids U[-1,1]^3, edge vectors i.i.d. N(0, 0.005^2) per
    axis, per-triangle GGX roughness U[0.05, 0.8] and albedo U[0.2, 0.9]."""
    rng = np.random.Generator(np.random.PCG64(seed))
    c = rng.uniform(-extent, extent, size=(ntri, 3))
    e1 = rng.normal(0.0, edge_sigma, size=(ntri, 3))
    e2 = rng.normal(0.0, edge_sigma, size=(ntri, 3))
    p1 = c - (e1 + e2) / 3.0
    pts = np.empty((ntri * 3, 3), np.float64)
    pts[0::3] = p1
    pts[1::3] = p1 + e1
    pts[2::3] = p1 + e2
    ri = rng.integers(0, 64, size=ntri)
    ai = rng.integers(0, 64, size=ntri)
    idx = np.arange(ntri * 3, dtype=np.int32).reshape(-1, 3)
    cam = make_camera((0.0, 0.5, 3.2), (0.0, 0.0, 0.0), (0.0, 1.0, 0.0), 40.0, width, height)
    return Scene(points=_points(pts.astype(np.float32)), faces=_faces(idx, ri * 64 + ai),
                 materials=_palette_materials(), camera=cam, name=f"soup{ntri}")


def _icosphere(level: int):
    """Unit icosphere: the icosahedron's 20 faces split 4-way `level` times, new
    vertices at normalised edge midpoints (shared between neighbouring faces)."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array([(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
                  (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)], np.float64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    f = np.array([(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2),
                  (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5),
                  (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)], np.int64)
    for _ in range(level):
        nv = v.shape[0]
        e = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
        key = np.minimum(e[:, 0], e[:, 1]) * nv + np.maximum(e[:, 0], e[:, 1])
        uniq, inv = np.unique(key, return_inverse=True)
        a, b = uniq // nv, uniq % nv
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        v = np.concatenate([v, mid])
        m = (nv + inv).reshape(3, -1)  # midpoints of edges (0,1), (1,2), (2,0) per face
        m01, m12, m20 = m[0], m[1], m[2]
        f = np.concatenate([np.stack([f[:, 0], m01, m20], 1), np.stack([f[:, 1], m12, m01], 1),
                            np.stack([f[:, 2], m20, m12], 1), np.stack([m01, m12, m20], 1)])
    return v, f


def _value_noise(p: np.ndarray, seed: int, octaves: int = 3, base_freq: float = 4.0) -> np.ndarray:
    """Value noise in [-1, 1]: random lattice values (seeded hash of the integer
    lattice point) blended trilinearly with smoothstep weights, octaves at doubling
    frequency and halving amplitude, normalised by the amplitude sum."""
    out = np.zeros(p.shape[0], np.float64)
    amp_sum = 0.0
    for o in range(octaves):
        freq, amp = base_freq * 2 ** o, 0.5 ** o
        q = p * freq
        i0 = np.floor(q).astype(np.int64)
        t = q - i0
        w = t * t * (3.0 - 2.0 * t)
        acc = np.zeros(p.shape[0], np.float64)
        for dx in (0, 1):
            for dy in (0, 1):
                for dz in (0, 1):
                    h = ((i0[:, 0] + dx) * 73856093) ^ ((i0[:, 1] + dy) * 19349663) ^ ((i0[:, 2] + dz) * 83492791)
                    h = (h ^ (seed * 2654435761 + o * 97531)) & 0xFFFFFFFF
                    h = (h * 2246822519) & 0xFFFFFFFF
                    h ^= h >> 13
                    h = (h * 3266489917) & 0xFFFFFFFF
                    h ^= h >> 16
                    val = h.astype(np.float64) / 4294967295.0 * 2.0 - 1.0
                    wx = w[:, 0] if dx else 1.0 - w[:, 0]
                    wy = w[:, 1] if dy else 1.0 - w[:, 1]
                    wz = w[:, 2] if dz else 1.0 - w[:, 2]
                    acc += wx * wy * wz * val
        out += amp * acc
        amp_sum += amp
    return out / amp_sum


def _mixed_materials(levels=64):
    """64 x 64 GGX palette (roughness x albedo) followed by 64 Lambert albedos."""
    lam = [_material((a, a, a)) for a in (0.2 + 0.7 * (i + 0.5) / levels for i in range(levels))]
    return np.concatenate([_palette_materials(levels), np.stack(lam)])


def stadium(seed=2, quads=1000, size=200.0, level=8, radius=0.05, noise_amp=0.005, width=1920, height=1080) -> Scene:
    """Teapot in a stadium: a size x size ground plane at y = 0 of quads x quads
    quads (2 * quads^2 triangles) and an icosphere of the given subdivision level
    (20 * 4^level triangles) of radius `radius`, displaced along the normal by
    3-octave value noise of amplitude `noise_amp`, resting on the plane. Per
    triangle: Lambert or GGX with equal probability, roughness U[0.05, 0.8] and
    albedo U[0.2, 0.9] (64-level palette). The camera looks at the sphere from
    about five radii away; the plane runs to the horizon."""
    rng = np.random.Generator(np.random.PCG64(seed))
    g = np.linspace(-size / 2, size / 2, quads + 1)
    gx, gz = np.meshgrid(g, g, indexing="xy")
    plane = np.stack([gx.ravel(), np.zeros(gx.size), gz.ravel()], 1)
    r0 = np.arange(quads)[:, None] * (quads + 1) + np.arange(quads)[None, :]
    a, b, c, d = r0.ravel(), r0.ravel() + 1, r0.ravel() + quads + 1, r0.ravel() + quads + 2
    ptri = np.concatenate([np.stack([a, c, b], 1), np.stack([b, c, d], 1)])  # normals +y
    sv, sf = _icosphere(level)
    disp = radius + noise_amp * _value_noise(sv, seed)
    center = np.array([0.0, radius + noise_amp, 0.0])
    sphere = center + sv * disp[:, None]
    pts = np.concatenate([plane, sphere]).astype(np.float32)
    tri = np.concatenate([ptri, sf + plane.shape[0]]).astype(np.int32)
    n = tri.shape[0]
    ggx = rng.random(n) < 0.5
    ri = rng.integers(0, 64, size=n)
    ai = rng.integers(0, 64, size=n)
    mat = np.where(ggx, ri * 64 + ai, 64 * 64 + ai)
    cam = make_camera((0.16, 0.09, 0.2), (0.0, 0.05, 0.0), (0.0, 1.0, 0.0), 40.0, width, height)
    return Scene(points=_points(pts), faces=_faces(tri, mat), materials=_mixed_materials(), camera=cam,
                 name=f"stadium{n}")


def sky_env(width=2048, height=1024, sun_elev_deg=30.0, sun_azim_deg=40.0, sun_sigma_deg=0.5,
            sun_peak=5.0e4) -> np.ndarray:
    """FP32 RGB lat-long map (float4 texels, w = 1) in the reference's mapping
    (src/cl/kernel/Util.cl:397-439: u -> theta = 2 pi u, v -> phi = pi v, y up):
    zenith-to-horizon gradient plus a Gaussian sun lobe of the given peak."""
    u = (np.arange(width, dtype=np.float64) + 0.5) / width
    v = (np.arange(height, dtype=np.float64) + 0.5) / height
    theta = 2.0 * np.pi * u[None, :]
    phi = np.pi * v[:, None]
    dx = -np.sin(phi) * np.cos(theta)
    dy = np.cos(phi) * np.ones_like(theta)
    dz = np.sin(phi) * np.sin(theta)
    up = np.clip(dy, 0.0, 1.0)
    zenith = np.array([0.25, 0.45, 1.0])
    horizon = np.array([1.0, 0.95, 0.9])
    ground = np.array([0.25, 0.22, 0.2])
    t = np.sqrt(up)[..., None]
    sky = horizon * (1.0 - t) + zenith * t
    sky = np.where((dy < 0.0)[..., None], ground, sky)
    el, az = math.radians(sun_elev_deg), math.radians(sun_azim_deg)
    sdir = np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)])
    cosang = np.clip(dx * sdir[0] + dy * sdir[1] + dz * sdir[2], -1.0, 1.0)
    ang = np.arccos(cosang)
    sig = math.radians(sun_sigma_deg)
    sun = sun_peak * np.exp(-0.5 * (ang / sig) ** 2)
    rgb = sky + sun[..., None] * np.array([1.0, 0.95, 0.85])
    out = np.ones((height, width, 4), np.float32)
    out[..., :3] = rgb
    return out.reshape(-1, 4)


def random_rays(scene: Scene, n: int, seed: int = 7, inside: bool = True):
    """Synthetic ray set for traversal parity: origins inside the scene bound
    (or on a sphere around it), directions uniform on the sphere."""
    rng = np.random.Generator(np.random.PCG64(seed))
    p = scene.points[:, :3]
    lo, hi = p.min(0), p.max(0)
    if inside:
        o = rng.uniform(lo, hi, size=(n, 3))
    else:
        ctr, rad = (lo + hi) / 2, float(np.linalg.norm(hi - lo)) * 0.75
        w = rng.normal(size=(n, 3))
        o = ctr + rad * w / np.linalg.norm(w, axis=1, keepdims=True)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)
