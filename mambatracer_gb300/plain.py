"""The reference's own host loop over the kernel-by-name API.

`PlainDeviceGI` drives the reference's kernel set (mt_kernel_create / set_arg /
mt_launch_1d) the way its Java host classes do: the buffers of CDeviceGI.createBuffers
(src/cl/device/CDeviceGI.java:130-164), the frame loop of CDeviceGI.loop (:214-271),
CCompact.execute (src/cl/algorithms/CCompact.java:79-89), the light list of
CLightConfiguration.initLights (src/cl/algorithms/CLightConfiguration.java:43-87) with
PrefixSumInteger (src/cl/algorithms/PrefixSumInteger.java), the texture pass with
CTextureApplyPass.process's texel lookup as a device kernel (textureApplyPass) in place
of its copy to the host and back, and CImage.processImage
(src/cl/image/CImage.java:124-136) with PrefixSumFloat. Every buffer has the
reference's layout; every launch is one reference kernel. It is the plain wavefront
that a host keeping its own loop gets from the library, and the comparison point for
the fused path (api.Job).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import check, lib
from .scenes import texture_tables

LOCAL = 100          # CDeviceGI.localWorkSize
SCAN_LOCAL = 128     # PrefixSumInteger / PrefixSumFloat LOCALSIZE
GRID_BYTES = 48 + 3 * 2560000 * 4  # LightGrid struct (LightGrid.cl:9-37)


def global_size(n: int, local: int) -> int:
    """MambaAPIInterface.getGlobal: n rounded up to a multiple of local."""
    return ((n + local - 1) // local) * local


class Buf:
    def __init__(self, ctx, nbytes: int = 0, host: np.ndarray | None = None):
        b = C.c_void_p()
        if host is not None:
            host = np.ascontiguousarray(host)
            check(lib().mt_buf_create_from(ctx.h, host.ctypes.data_as(C.c_void_p), max(host.nbytes, 4), C.byref(b)))
        else:
            check(lib().mt_buf_alloc(ctx.h, max(int(nbytes), 4), C.byref(b)))
        self.h = b

    def write(self, a: np.ndarray, offset: int = 0):
        a = np.ascontiguousarray(a)
        check(lib().mt_buf_write(self.h, offset, a.ctypes.data_as(C.c_void_p), a.nbytes))

    def read(self, like: np.ndarray) -> np.ndarray:
        out = np.zeros_like(like)
        check(lib().mt_buf_read(self.h, 0, out.ctypes.data_as(C.c_void_p), out.nbytes))
        return out

    def int(self) -> int:
        return int(self.read(np.zeros(1, np.int32))[0])

    def free(self):
        if self.h:
            lib().mt_buf_free(self.h)
            self.h = None


class Kernel:
    """OpenCLConfiguration.createKernel(name, args...) and execute1DKernel."""

    def __init__(self, ctx, name: str, *args: Buf):
        h = C.c_void_p()
        check(lib().mt_kernel_create(ctx.h, name.encode(), C.byref(h)))
        self.h = h
        self.name = name
        for i, a in enumerate(args):
            self.put_arg(i, a)

    def put_arg(self, i: int, b: Buf):
        check(lib().mt_kernel_set_arg_buf(self.h, i, b.h))

    def put_local(self, i: int, nbytes: int):
        """CLocalMemory.LOCALINT / LOCALFLOAT: a __local scratch argument."""
        check(lib().mt_kernel_set_arg_local(self.h, i, int(nbytes)))

    def run(self, global_: int, local: int):
        check(lib().mt_launch_1d(self.h, int(global_), int(local)))

    def free(self):
        if self.h:
            lib().mt_kernel_destroy(self.h)
            self.h = None


def int_buf(ctx, v: int) -> Buf:
    return Buf(ctx, host=np.array([v], np.int32))


def float_buf(ctx, v: float) -> Buf:
    return Buf(ctx, host=np.array([v], np.float32))


class PrefixSum:
    """PrefixSumInteger / PrefixSumFloat: local Kogge-Stone scans, a sequential group
    scan, the group prefixes added back, and the total."""

    def __init__(self, ctx, data: Buf, length: int, kind: str = "Integer"):
        self.length = length
        self.G = global_size(length, SCAN_LOCAL)
        ng = self.G // SCAN_LOCAL
        dt = np.int32 if kind == "Integer" else np.float32
        self.dt = dt
        self.clength = int_buf(ctx, length)
        self.prefix = Buf(ctx, 4 * length)
        self.gsum = Buf(ctx, 4 * ng)
        self.gprefix = Buf(ctx, 4 * ng)
        self.gsize = int_buf(ctx, ng)
        self.total = Buf(ctx, host=np.zeros(1, dt))
        local = Kernel(ctx, f"localScan{kind}", data, self.prefix, self.gsum, self.clength)
        local.put_local(4, 4 * SCAN_LOCAL)
        self.k = [local,
                  Kernel(ctx, f"groupScan{kind}", self.gsum, self.gprefix, self.gsize),
                  Kernel(ctx, f"globalScan{kind}", self.prefix, self.gprefix, self.clength),
                  Kernel(ctx, f"globalTotal{kind}", data, self.prefix, self.total, self.clength)]

    def execute(self):
        self.k[0].run(self.G, SCAN_LOCAL)
        self.k[1].run(1, 1)
        self.k[2].run(self.G, SCAN_LOCAL)
        self.k[3].run(1, 1)

    def count(self):
        return self.total.read(np.zeros(1, self.dt))[0]

    def free(self):
        for k in self.k:
            k.free()
        for b in (self.clength, self.prefix, self.gsum, self.gprefix, self.gsize, self.total):
            b.free()


class PlainDeviceGI:
    """CDeviceGI over the kernel-by-name API: reference semantics (seeds per
    allocateState call), `max_depth` bounces per frame."""

    def __init__(self, ctx, scene, nodes: np.ndarray, bounds: np.ndarray, width: int, height: int,
                 max_depth: int = 15, env: tuple | None = None):
        self.ctx, self.W, self.H, self.depth = ctx, width, height, max_depth
        N = self.N = width * height
        self.G = global_size(N, LOCAL)
        sc = scene
        # CMesh.initCLBuffers
        self.points = Buf(ctx, host=np.ascontiguousarray(sc.points, np.float32))
        self.uvs = Buf(ctx, host=np.ascontiguousarray(sc.uvs, np.float32))
        self.normals = Buf(ctx, host=np.ascontiguousarray(sc.normals, np.float32))
        self.faces = Buf(ctx, host=np.ascontiguousarray(sc.faces))
        self.size = int_buf(ctx, sc.ntri)
        self.materials = Buf(ctx, host=np.ascontiguousarray(sc.materials))
        self.nodes = Buf(ctx, host=np.ascontiguousarray(nodes))
        self.bounds = Buf(ctx, host=np.ascontiguousarray(bounds))
        # CEnvironment + the LightGrid struct's header
        grid = np.zeros(48, np.uint8)
        if env is not None:
            rgb, lum, sat, ew, eh = env
            hdr = np.zeros(12, np.int32)
            hdr[0], hdr[2], hdr[3], hdr[4], hdr[5], hdr[6], hdr[7] = 1, ew, eh, 1600, 1600, 16, 32
            grid = hdr.view(np.uint8)
        else:
            rgb, lum, sat = np.zeros((1, 4), np.float32), np.zeros(1, np.float32), np.zeros(1, np.float32)
        self.env_rgb = Buf(ctx, host=np.ascontiguousarray(rgb, np.float32))
        self.env_lum = Buf(ctx, host=np.ascontiguousarray(lum, np.float32))
        self.env_sat = Buf(ctx, host=np.ascontiguousarray(sat, np.float32))
        self.light_grid = Buf(ctx, GRID_BYTES)
        self.light_grid.write(np.zeros(GRID_BYTES, np.uint8))
        self.light_grid.write(grid)
        # CDeviceGI.createBuffers
        self.state = Buf(ctx, 16)
        self.pixels = Buf(ctx, 4 * N)
        self.count = int_buf(ctx, N)
        self.length = int_buf(ctx, N)
        self.rays = Buf(ctx, 80 * N)
        self.occlus = Buf(ctx, 80 * N)
        self.camera = Buf(ctx, 64)
        self.paths = Buf(ctx, 304 * N)
        self.isects = Buf(ctx, 96 * N)
        self.tex = Buf(ctx, 80 * N)
        # the material images CTextureApplyPass.process reads on the host, as a
        # texel pool and a per-material table for the device lookup
        texels, table = texture_tables(sc)
        self.texels = Buf(ctx, host=texels)
        self.tex_ref = Buf(ctx, host=table)
        # CImage
        self.frame_count = float_buf(ctx, 1.0)
        self.accum = Buf(ctx, 16 * N)
        self.frame_buffer = Buf(ctx, 16 * N)
        self.argb = Buf(ctx, 4 * N)
        self.frame_size = int_buf(ctx, N)
        self.loglw = Buf(ctx, 4 * N)
        self.loglw_count = Buf(ctx, 4 * N)
        self.gamma = float_buf(ctx, 2.2)
        self.exposure = float_buf(ctx, 0.18)
        self.lights_init()
        # CCompact.init
        self.temp_isects = Buf(ctx, 96 * N)
        self.temp_pixels = Buf(ctx, 4 * N)
        k = lambda name, *a: Kernel(ctx, name, *a)  # noqa: E731
        self.k_compact = [k("InitIntersection", self.temp_isects, self.length),
                          k("InitIntData", self.temp_pixels, self.length),
                          k("CompactAtomic", self.isects, self.temp_isects, self.pixels, self.temp_pixels, self.count,
                            self.length),
                          k("InitIntersection", self.isects, self.length),
                          k("InitIntData", self.pixels, self.length),
                          k("TransferIntersection", self.isects, self.temp_isects, self.length),
                          k("TransferPixels", self.pixels, self.temp_pixels, self.length)]
        # CDeviceGI.createKernels
        mesh = (self.points, self.uvs, self.normals, self.faces, self.size)
        envb = (self.env_rgb, self.env_lum, self.env_sat, self.light_grid)
        self.k_init = [k("InitCameraRayDataJitter", self.camera, self.rays, self.state, self.length),
                       k("InitPathData", self.paths, self.length),
                       k("InitIntersection", self.isects, self.length),
                       k("InitIntDataToIndex", self.pixels, self.length)]
        self.k_intersect = k("IntersectPrimitives", self.rays, self.isects, self.count, *mesh, self.nodes, self.bounds)
        self.k_setup = k("SetupBSDFPath", self.isects, self.rays, self.paths, self.materials, self.pixels, self.count)
        self.k_lighthit = k("LightHitPass", self.isects, self.rays, self.paths, self.light_count, self.materials, *mesh,
                            self.accum, self.pixels, self.count, *envb)
        self.k_sample = k("SampleBSDFRayDirection", self.isects, self.rays, self.paths, self.materials, self.pixels,
                          self.state, self.count)
        self.k_direct = k("DirectLight", self.paths, self.isects, self.light_info, self.light_count, self.occlus,
                          self.accum, self.pixels, self.count, self.state, self.materials, *mesh, self.nodes,
                          self.bounds, *envb)
        self.k_texpass = k("texturePassGI", self.paths, self.isects, self.tex, self.pixels, self.count)
        self.k_texapply = k("textureApplyPass", self.tex, self.count, self.texels, self.tex_ref)
        self.k_texcolor = k("updateToTextureColorGI", self.paths, self.tex, self.pixels, self.count)
        # CImage.createKernels
        self.k_init_accum = k("InitFloat4DataXYZ", self.accum, self.frame_size)
        self.k_init_argb = k("InitIntDataRGB", self.argb, self.frame_size)
        self.k_average = k("averageAccum", self.accum, self.frame_count, self.frame_buffer, self.loglw,
                           self.loglw_count, self.frame_size)
        self.scan_loglw = PrefixSum(ctx, self.loglw, N, "Float")
        self.scan_count = PrefixSum(ctx, self.loglw_count, N, "Integer")
        self.k_update = k("updateFrameImage", self.frame_buffer, self.argb, self.scan_loglw.total,
                          self.scan_count.total, self.frame_size, self.exposure, self.gamma)
        gi = global_size(N, 128)
        self.k_init_accum.run(gi, 128)
        self.k_init_argb.run(gi, 128)
        self.counts = []

    def lights_init(self):
        """CLightConfiguration.initLights: emissive faces by predicate, prefix sum, LightInfo list."""
        ctx, n = self.ctx, int(self.size.int())
        self.predicate = Buf(ctx, 4 * n)
        g = global_size(n, 100)
        k = Kernel(ctx, "identifyMeshLights", self.faces, self.size, self.materials, self.predicate)
        k.run(g, 100)
        k.free()
        scan = PrefixSum(ctx, self.predicate, n, "Integer")
        scan.execute()
        self.nlights = int(scan.count())
        self.light_count = int_buf(ctx, self.nlights)
        self.light_info = Buf(ctx, 8 * max(self.nlights, 1))
        if self.nlights > 0:
            k = Kernel(ctx, "prepareLightInfo", self.predicate, scan.prefix, self.size, self.light_info)
            k.run(g, 100)
            k.free()
        scan.free()

    def set_camera(self, cam: np.ndarray):
        cam = np.array(cam, copy=True).reshape(-1)[:1]
        cam["dimension"] = (self.W, self.H)
        self.camera.write(np.frombuffer(cam.tobytes(), np.uint8))

    def _state(self, sx: int, sy: int, frame_count: float):
        st = np.zeros(4, np.int32)
        st[0], st[1] = sx, sy
        st[2] = np.array([frame_count], np.float32).view(np.int32)[0]
        self.state.write(st)

    def frame(self, seeds: np.ndarray, frame_count: float, record_counts: bool = False):
        """CDeviceGI.loop with the seeds of its allocateState calls (2 * (1 + 2 * depth) ints)."""
        s = iter(np.asarray(seeds, np.int32).reshape(-1, 2))
        G = self.G
        self._state(*next(s), frame_count)
        for k in self.k_init:
            k.run(G, LOCAL)
        self.count.write(np.array([self.N], np.int32))
        counts = []
        for _ in range(self.depth):
            self.k_intersect.run(G, LOCAL)
            self._state(*next(s), frame_count)
            self.k_setup.run(G, LOCAL)
            self.k_lighthit.run(G, LOCAL)
            self.count.write(np.zeros(1, np.int32))
            for k in self.k_compact:
                k.run(G, LOCAL)
            if record_counts:
                counts.append(self.count.int())
            self.k_texpass.run(G, LOCAL)
            self.k_texapply.run(G, LOCAL)  # CTextureApplyPass.process, on the device
            self.k_texcolor.run(G, LOCAL)
            self._state(*next(s), frame_count)
            self.k_direct.run(G, LOCAL)
            self.k_sample.run(G, LOCAL)
        self.counts = counts
        return counts

    def process_image(self, frame_count: float):
        """CImage.processImage: averageAccum, the log-luminance scans on frames < 3, updateFrameImage."""
        gi = global_size(self.N, 128)
        self.frame_count.write(np.array([frame_count], np.float32))
        self.k_average.run(gi, 128)
        if frame_count < 3:
            self.scan_loglw.execute()
            self.scan_count.execute()
        self.k_update.run(gi, 128)
        return self.argb.read(np.zeros(self.N, np.int32))

    def film(self) -> np.ndarray:
        return self.accum.read(np.zeros((self.N, 4), np.float32))

    def free(self):
        for v in list(vars(self).values()):
            if isinstance(v, (Buf, Kernel, PrefixSum)):
                v.free()
            elif isinstance(v, list):
                for x in v:
                    if isinstance(x, (Buf, Kernel)):
                        x.free()
