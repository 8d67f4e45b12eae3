"""Host API over the C-ABI, mirroring the reference's device interface.

`DeviceGI` follows RayDeviceInterface / CDeviceGI (src/cl/abstracts/RayDeviceInterface.java:28-71,
src/cl/device/CDeviceGI.java): `set(mesh, bvh)`, `setup(w, h)`, `update_camera()`,
`execute()` (one frame), `start/pause/resume/stop` on a render thread, and
`update_image()` returning the film. Everything runs through libmambatracer.so.
"""
from __future__ import annotations

import ctypes as C
import threading

import numpy as np

from . import layout
from ._lib import BatchFrame, RenderConfig, ServedStats, ServerConfig, Tuning, check, lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Context:
    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib().mt_ctx_create(device, C.byref(h)))
        self.h = h

    def finish(self):
        check(lib().mt_finish(self.h))

    def record(self, slot: int):
        check(lib().mt_ctx_event_record(self.h, slot))

    def elapsed_ms(self, a: int, b: int) -> float:
        ms = C.c_float()
        check(lib().mt_ctx_event_elapsed(self.h, a, b, C.byref(ms)))
        return ms.value

    def close(self):
        if self.h:
            check(lib().mt_ctx_destroy(self.h))
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Scene:
    """Mesh arrays on the device (CMesh.initCLBuffers, src/cl/scene/CMesh.java:339-357)."""

    def __init__(self, ctx: Context, sc):
        self.ctx = ctx
        self.src = sc
        pts = np.ascontiguousarray(sc.points, np.float32)
        faces = np.ascontiguousarray(sc.faces)
        mats = np.ascontiguousarray(sc.materials)
        uvs = np.ascontiguousarray(sc.uvs, np.float32)
        nrm = np.ascontiguousarray(sc.normals, np.float32)
        h = C.c_void_p()
        check(lib().mt_scene_create(ctx.h, _p(pts), pts.shape[0], _p(uvs), uvs.shape[0], _p(nrm), nrm.shape[0],
                                    _p(faces), faces.shape[0], _p(mats), mats.shape[0], C.byref(h)))
        self.h = h
        self.depth = None
        self.grid = (1600, 1600, 16, 32, 0)
        for m, kind, img in getattr(sc, "textures", ()):
            self.set_texture(m, kind, img)

    def set_texture(self, material: int, kind: int, argb: np.ndarray | None):
        """Bind a material's texture image (kind 0 diffuse, 1 glossy, 2 roughness,
        3 mirror; ARGB int32 [H, W]); None removes it."""
        if argb is None:
            check(lib().mt_scene_set_texture(self.h, material, kind, None, 0, 0))
            return
        a = np.ascontiguousarray(argb).view(np.int32)
        check(lib().mt_scene_set_texture(self.h, material, kind, _p(a), a.shape[1], a.shape[0]))

    def build_bvh(self):
        """CNormalBVH.build on the host (returns nodes, bounds in the reference layout)."""
        n = self.src.ntri
        nodes = np.zeros((2 * n - 1, 7), np.int32)
        bounds = np.zeros((2 * n - 1, 8), np.float32)
        depth = C.c_int()
        check(lib().mt_bvh_build(self.h, _p(nodes), _p(bounds), C.byref(depth)))
        self.depth = depth.value
        return nodes, bounds

    def build_bvh_device(self, want_arrays: bool = True):
        """The same tree built on the GPU (returns nodes, bounds in the reference layout)."""
        n = self.src.ntri
        nodes = np.zeros((2 * n - 1, 7), np.int32) if want_arrays else None
        bounds = np.zeros((2 * n - 1, 8), np.float32) if want_arrays else None
        depth = C.c_int()
        check(lib().mt_bvh_build_device(self.h, _p(nodes), _p(bounds), C.byref(depth)))
        self.depth = depth.value
        return nodes, bounds

    def layout(self):
        """The traversal layout on the device: (records (nrec, 16) float32,
        tris (N, 12) float32, root ref)."""
        nrec, root = C.c_int(), C.c_int()
        check(lib().mt_scene_layout_read(self.h, None, None, C.byref(nrec), C.byref(root)))
        recs = np.zeros((max(nrec.value, 0), 16), np.float32)
        tris = np.zeros((self.src.ntri, 12), np.float32)
        check(lib().mt_scene_layout_read(self.h, _p(recs) if nrec.value else None, _p(tris), None, None))
        return recs, tris, root.value

    def set_precision(self, precision: int):
        """Traversal record format: 0 FP32 child boxes, 1 FP16 rounded outward."""
        check(lib().mt_scene_set_bvh_precision(self.h, precision))

    def import_bvh(self, nodes: np.ndarray, bounds: np.ndarray):
        nodes = np.ascontiguousarray(nodes, np.int32)
        bounds = np.ascontiguousarray(bounds, np.float32)
        check(lib().mt_bvh_import(self.h, _p(nodes), _p(bounds), nodes.shape[0]))

    def set_env(self, rgb: np.ndarray, w: int, h: int):
        rgb = np.ascontiguousarray(rgb, np.float32)
        check(lib().mt_env_set(self.h, _p(rgb), w, h))

    def set_env_with_sat(self, rgb, lum, sat, w, h):
        rgb = np.ascontiguousarray(rgb, np.float32)
        lum = np.ascontiguousarray(lum, np.float32)
        sat = np.ascontiguousarray(sat, np.float32)
        check(lib().mt_env_set_with_sat(self.h, _p(rgb), _p(lum), _p(sat), w, h))

    def env_arrays(self, w, h):
        lum = np.zeros(w * h, np.float32)
        sat64 = np.zeros(w * h, np.float64)
        sat32 = np.zeros(w * h, np.float32)
        check(lib().mt_env_read(self.h, _p(lum), _p(sat64), _p(sat32)))
        return lum, sat64, sat32

    def grid_config(self, nu: int = 1600, nv: int = 1600, rx: int = 16, ry: int = 32, enable: int = 1):
        """Adaptive light grid for mode-1 jobs (0 off, 1 FP32 per-cell SATs, 2 FP64)."""
        check(lib().mt_env_grid_config(self.h, nu, nv, rx, ry, enable))
        self.grid = (nu, nv, rx, ry, enable)

    def preview(self, camera: np.ndarray, width: int, height: int):
        """The preview device's frame (CDeviceRT): ARGB ints and the material group per pixel."""
        cam = np.ascontiguousarray(camera)
        assert cam.dtype == layout.CAMERA
        argb = np.zeros(width * height, np.int32)
        group = np.zeros(width * height, np.int32)
        check(lib().mt_preview_frame(self.h, _p(cam), width, height, _p(argb), _p(group)))
        return argb, group

    @property
    def light_count(self) -> int:
        return lib().mt_scene_light_count(self.h)

    def trace_closest(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays)
        assert rays.dtype == layout.RAY
        t = np.zeros(rays.shape[0], np.float32)
        prim = np.zeros(rays.shape[0], np.int32)
        check(lib().mt_trace_closest(self.h, _p(rays), rays.shape[0], _p(t), _p(prim)))
        return t, prim

    def trace_any(self, rays: np.ndarray):
        rays = np.ascontiguousarray(rays)
        assert rays.dtype == layout.RAY
        occ = np.zeros(rays.shape[0], np.int32)
        check(lib().mt_trace_any(self.h, _p(rays), rays.shape[0], _p(occ)))
        return occ

    def trace_counts(self, rays: np.ndarray, any_hit: bool = False):
        """Closest (or any) hits with the traversal work per ray: (t, prim or
        occluded, int32 [n, 2] = interior-node visits, triangle tests)."""
        rays = np.ascontiguousarray(rays)
        assert rays.dtype == layout.RAY
        n = rays.shape[0]
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        counts = np.zeros((n, 2), np.int32)
        check(lib().mt_trace_counts(self.h, _p(rays), n, int(any_hit), _p(t), _p(prim), _p(counts)))
        return t, prim, counts

    def close(self):
        if self.h:
            check(lib().mt_scene_destroy(self.h))
            self.h = None


class Job:
    """Film and path state of one render job resident on the device."""

    def __init__(self, ctx: Context, scene: Scene, width: int, height: int, max_depth: int = 15, mode: int = 0,
                 rr_depth: int = 0, film_kahan: int = 1, spp: int = 1, use_graph: int = 0, profile: int = 0,
                 inflight: int = 1, grid_updates: int = 5):
        self.cfg = RenderConfig(width, height, max_depth, mode, rr_depth, film_kahan, spp, use_graph, profile,
                                inflight, grid_updates)
        self.scene = scene
        h = C.c_void_p()
        check(lib().mt_job_create(ctx.h, scene.h, C.byref(self.cfg), C.byref(h)))
        self.h = h
        self.width, self.height = width, height

    def set_camera(self, cam: np.ndarray):
        cam = np.ascontiguousarray(cam)
        assert cam.dtype == layout.CAMERA
        check(lib().mt_job_set_camera(self.h, _p(cam)))

    def render(self, seeds: np.ndarray | None = None, frame_count: float = 1.0):
        if seeds is not None:
            seeds = np.ascontiguousarray(seeds, np.int32)
        check(lib().mt_render_frame(self.h, _p(seeds), float(frame_count)))

    def film(self, resolve: bool = False) -> np.ndarray:
        out = np.zeros((self.width * self.height, 4), np.float32)
        check(lib().mt_film_read(self.h, _p(out), int(resolve)))
        return out

    def film_async(self, out: np.ndarray, resolve: bool = False):
        """Enqueue a read of the film into `out` (float32, width*height x 4; pinned
        memory for a copy that overlaps the next frame); complete it with wait()."""
        assert out.dtype == np.float32 and out.size == self.width * self.height * 4 and out.flags.c_contiguous
        self._pending = (getattr(self, "_pending", []) + [out])[-8:]
        check(lib().mt_film_read_async(self.h, _p(out), int(resolve)))

    def wait(self):
        check(lib().mt_film_wait(self.h))
        self._pending = []

    def image(self, exposure: float = 0.18, gamma: float = 2.2):
        """The displayed ARGB image (int32 per pixel) and the log-average luminance."""
        out = np.zeros(self.width * self.height, np.int32)
        la = C.c_float()
        check(lib().mt_image_argb(self.h, _p(out), float(exposure), float(gamma), C.byref(la)))
        return out, la.value

    def grid(self):
        """The job's light grid: (func, sat, accum), each nu * nv float32."""
        nu, nv = self.scene.grid[0], self.scene.grid[1]
        out = [np.zeros(nu * nv, np.float32) for _ in range(3)]
        check(lib().mt_job_grid_read(self.h, _p(out[0]), _p(out[1]), _p(out[2])))
        return tuple(out)

    def clear(self):
        check(lib().mt_film_clear(self.h))

    def stats(self):
        rays = np.zeros(3, np.int64)
        counts = np.zeros(self.cfg.max_depth, np.int32)
        check(lib().mt_job_stats(self.h, _p(rays), _p(counts)))
        return rays, counts

    def total_rays(self) -> np.ndarray:
        out = np.zeros(3, np.int64)
        check(lib().mt_job_total_rays(self.h, _p(out)))
        return out

    def last_ms(self) -> float:
        ms = C.c_float()
        check(lib().mt_job_last_ms(self.h, C.byref(ms)))
        return ms.value

    def launches(self) -> int:
        """Kernels the job's frames have launched (mt_job_launches)."""
        n = C.c_int64()
        check(lib().mt_job_launches(self.h, C.byref(n)))
        return n.value

    def kernel_ms(self) -> np.ndarray:
        """Per-launch device times of the last frame (profiled jobs): spp x (1 + 3 * max_depth)."""
        out = np.zeros(self.cfg.spp * (1 + 3 * self.cfg.max_depth), np.float32)
        check(lib().mt_job_kernel_ms(self.h, _p(out)))
        return out.reshape(self.cfg.spp, -1)

    def close(self):
        if self.h:
            check(lib().mt_job_destroy(self.h))
            self.h = None


def bvh_build_host(sc):
    """CNormalBVH.build on host arrays (no device needed)."""
    n = sc.ntri
    nodes = np.zeros((2 * n - 1, 7), np.int32)
    bounds = np.zeros((2 * n - 1, 8), np.float32)
    depth = C.c_int()
    pts = np.ascontiguousarray(sc.points, np.float32)
    faces = np.ascontiguousarray(sc.faces)
    check(lib().mt_bvh_build_host(_p(pts), pts.shape[0], _p(faces), n, _p(nodes), _p(bounds), C.byref(depth)))
    return nodes, bounds, depth.value


class DeviceGI:
    """Progressive GI device (CDeviceGI): a render thread that calls execute()
    in a loop, with pause/resume/stop as LambdaThread offers them."""

    def __init__(self, width: int, height: int, ctx: Context | None = None, **job_kw):
        self.width, self.height = width, height
        self.ctx = ctx or Context()
        self.job_kw = job_kw
        self.scene = None
        self.job = None
        self.camera = None
        self.frame_count = 1.0  # CImage frame count starts at 1 (CDeviceGI.java:325-328)
        self._thread = None
        self._run = threading.Event()
        self._stop = threading.Event()
        self.seed_source = np.random.default_rng()

    # RayDeviceInterface.set(mesh, bvhBuild)
    def set(self, scene: Scene, nodes: np.ndarray | None = None, bounds: np.ndarray | None = None):
        self.scene = scene
        if nodes is not None:
            scene.import_bvh(nodes, bounds)

    # CDeviceGI.setup(w, h)
    def setup(self, width: int, height: int):
        self.width, self.height = width, height
        if self.job:
            self.job.close()
        self.job = Job(self.ctx, self.scene, width, height, **self.job_kw)
        if self.camera is not None:
            self.job.set_camera(self.camera)

    def update_camera(self, camera: np.ndarray):
        cam = camera.copy()
        cam["dimension"] = (self.width, self.height)
        self.camera = cam
        if self.job:
            self.job.set_camera(cam)

    def _seeds(self):
        cfg = self.job.cfg
        if cfg.mode != 0:
            return None
        # allocateState: two random 30-bit primes per call (CDeviceGI.java:364-376); any odd 30-bit
        # values serve the RNG, so odd draws stand in for the primes
        n = 2 * (1 + 2 * cfg.max_depth) * cfg.spp
        return (self.seed_source.integers(2 ** 29, 2 ** 30, size=n) | 1).astype(np.int32)

    def execute(self):
        self.job.render(self._seeds(), self.frame_count)
        self.frame_count += self.job.cfg.spp

    def update_image(self, resolve: bool = True) -> np.ndarray:
        return self.job.film(resolve=resolve)

    def start(self):
        self._stop.clear()
        self._run.set()

        def loop():
            while not self._stop.is_set():
                if not self._run.wait(timeout=0.05):
                    continue
                self.execute()
                self.ctx.finish()

        self._thread = threading.Thread(target=loop, daemon=True)
        self._thread.start()

    def pause(self):
        self._run.clear()

    def resume(self):
        self._run.set()

    def is_paused(self) -> bool:
        return not self._run.is_set()

    def stop(self):
        self._stop.set()
        self._run.set()
        if self._thread:
            self._thread.join()
            self._thread = None


class Server:
    """Served mode: concurrent render requests (mt_job_submit / poll / cancel / wait).
    A request renders `spp` benchmark-semantics passes of one camera; its film lands in
    the float32 array given at submission (kept alive here until the request ends).
    merged=m (m >= 1): the running requests share wavefront queues, their slots split
    over m streams that each run rounds of one merged pass per scene; films are the same
    bit for bit."""

    QUEUED, RUNNING, DONE, CANCELLED, FAILED = range(5)

    def __init__(self, ctx: Context, lanes: int = 8, max_width: int = 1920, max_height: int = 1080,
                 max_spp: int = 64, max_depth: int = 8, rr_depth: int = 3, film_kahan: int = 1,
                 budget_bytes: int = 0, merged: int = 0):
        self.cfg = ServerConfig(lanes, max_width, max_height, max_spp, max_depth, rr_depth, film_kahan,
                                int(merged), budget_bytes)
        h = C.c_void_p()
        check(lib().mt_server_create(ctx.h, C.byref(self.cfg), C.byref(h)))
        self.h = h
        self._films = {}

    def submit(self, scene: Scene, camera: np.ndarray, width: int, height: int, spp: int,
               frame_count: float = 1.0, film: bool = True) -> int:
        cam = np.ascontiguousarray(camera)
        assert cam.dtype == layout.CAMERA
        out = np.zeros((width * height, 4), np.float32) if film else None
        rid = C.c_int64()
        check(lib().mt_job_submit(self.h, scene.h, _p(cam), width, height, spp, float(frame_count), _p(out),
                                  C.byref(rid)))
        self._films[rid.value] = out
        return rid.value

    def poll(self, rid: int):
        st, lat = C.c_int(), C.c_double()
        check(lib().mt_job_poll(self.h, rid, C.byref(st), C.byref(lat)))
        return st.value, lat.value

    def cancel(self, rid: int):
        check(lib().mt_job_cancel(self.h, rid))

    def wait(self, rid: int, timeout_ms: float = -1.0):
        check(lib().mt_job_wait(self.h, rid, float(timeout_ms)))
        return self._films.get(rid)

    def film(self, rid: int):
        return self._films.get(rid)

    def drain(self):
        check(lib().mt_server_drain(self.h))

    def stats(self) -> dict:
        st = ServedStats()
        check(lib().mt_server_stats(self.h, C.byref(st)))
        return {f: (list(getattr(st, f)) if f == "rays" else getattr(st, f)) for f, _ in ServedStats._fields_}

    def close(self):
        if self.h:
            check(lib().mt_server_destroy(self.h))
            self.h = None



TUNING_FIELDS = tuple(f for f, _ in Tuning._fields_)


def get_tuning() -> dict:
    """The process's launch shapes (mt_tuning_get)."""
    t = Tuning()
    check(lib().mt_tuning_get(C.byref(t)))
    return {f: getattr(t, f) for f in TUNING_FIELDS}


def set_tuning(tuning: dict | None = None, **fields):
    """Install launch shapes (mt_tuning_set); fields not given keep their values."""
    cur = get_tuning()
    cur.update(tuning or {})
    cur.update(fields)
    t = Tuning(*(int(cur[f]) for f in TUNING_FIELDS))
    check(lib().mt_tuning_set(C.byref(t)))


def batch_render(ctx: Context, scene: Scene, frames, max_depth: int = 8, rr_depth: int = 3, film_kahan: int = 1):
    """Frames of one scene through one set of wavefront queues (mt_batch_render).
    frames: (camera, width, height, spp, frame_count) each. Returns the films
    (float32 [w * h, 4] each, summed over the frame's passes) and the ray counts."""
    arr = (BatchFrame * len(frames))()
    for f, (cam, w, h, spp, fc) in zip(arr, frames):
        c = np.array(cam, copy=True).reshape(-1)[:1]
        f.width, f.height, f.spp, f.frame_count = int(w), int(h), int(spp), float(fc)
        C.memmove(f.camera, np.frombuffer(c.tobytes(), np.uint8).ctypes.data, 64)
    sizes = [int(w) * int(h) for _, w, h, _, _ in frames]
    out = np.zeros((sum(sizes), 4), np.float32)
    rays = np.zeros(3, np.int64)
    check(lib().mt_batch_render(ctx.h, scene.h, C.cast(arr, C.c_void_p), len(frames), max_depth, rr_depth, film_kahan,
                                _p(out), _p(rays)))
    films, off = [], 0
    for n in sizes:
        films.append(out[off:off + n])
        off += n
    return films, rays
