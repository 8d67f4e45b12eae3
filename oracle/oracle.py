"""ctypes bindings for the CPU oracle (liboracle.so) and, where it was built,
the reference kernels compiled as C++ (oracle/_ref/libmtref.so).

Test infrastructure only: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py, never by the product.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

HERE = os.path.dirname(os.path.abspath(__file__))
REF_LIB = os.path.join(HERE, "_ref", "libmtref.so")

P = C.c_void_p
I = C.c_int
F = C.c_float


def ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "arrays must be C-contiguous"
    return a.ctypes.data_as(C.c_void_p)


class Oracle:
    """The CPU restatement (oracle/mt_oracle.cpp)."""

    def __init__(self):
        self.lib = C.CDLL(_build.build())
        L = self.lib
        L.or_wanghash.restype = C.c_uint
        L.or_wanghash.argtypes = [I]
        L.or_random.argtypes = [P, F, I, I, P]
        L.or_bvh_build.restype = I
        L.or_bvh_build.argtypes = [P, P, I, P, P, P]
        L.or_intersect.argtypes = [P, P, I, I, P, P, P, P, I, P, P, P]
        L.or_trace_closest.argtypes = [P, I, P, P, I, P, P, P, P, P]
        L.or_occlusion.argtypes = [P, P, I, P, P, I, P, P, P]
        L.or_raygen.argtypes = [P, P, P, F, I, I]
        L.or_stage_seed.argtypes = [I, I, P]
        L.or_light_list.restype = I
        L.or_light_list.argtypes = [P, I, P, P]
        L.or_env_lum_sat.argtypes = [P, I, I, P, P]
        L.or_env_sat_fp64.argtypes = [P, I, I, P]
        L.or_sat_sample.argtypes = [P, P, P, F, F, P, P, P]
        L.or_sat_sample_discrete.argtypes = [P, P, P, F, F, P, P]
        L.or_sat_pdf.restype = F
        L.or_sat_pdf.argtypes = [P, P, P, I, I]
        L.or_env_illuminate.argtypes = [P, P, P, I, I, P, P, P, P]
        L.or_env_radiance.argtypes = [P, P, P, I, I, P, P, P]
        L.or_lightgrid_sat.argtypes = [P, P, I, I, I, I]
        L.or_bsdf_sample.restype = I
        L.or_bsdf_sample.argtypes = [P, P, P, P, P, P, P, P, P, P]
        L.or_bsdf_eval.restype = I
        L.or_bsdf_eval.argtypes = [P, P, P, P, P, P, P, P]
        L.or_render_frame.restype = I
        L.or_render_frame.argtypes = [P, I, I, I, I, I, P, F, P, P, P, P, I, P, P, P, P, P, P, I, I, I, I, P,
                                      P, P]
        L.or_render_frame_grid.restype = I
        L.or_render_frame_grid.argtypes = L.or_render_frame.argtypes + [P, P, P, I, I, I, I, P, I, I]
        L.or_render_frame_subset.restype = I
        L.or_render_frame_subset.argtypes = L.or_render_frame_grid.argtypes + [P, I]
        L.or_grid_init_func.argtypes = [P, P, I, I, I, I, I, I, P]
        L.or_env_grid_illuminate.argtypes = [P, P, P, I, I, P, P, I, I, I, I, P, P, P, P, P, P, P, P]
        L.or_env_grid_radiance.argtypes = [P, P, P, I, I, P, P, I, I, I, I, P, P, P, P, P, P, P]
        L.or_tonemap.argtypes = [P, I, F, F, F, P, P, P]
        L.or_tonemap_with_total.argtypes = [P, I, F, F, F, P, P, P, P]
        L.or_preview.argtypes = [P, I, I, P, P, P, P, I, P, P, P, P, I, I, I, P, P]
        L.or_set_textures.argtypes = [P, P, I]
        L.or_texture_apply.argtypes = [P, I, F, F, P, P, I, P]


class RefOracle:
    """MambaTracer's own kernels compiled as C++ (present only where the
    reference tree was available to build them)."""

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_LIB)

    def __init__(self):
        self.lib = C.CDLL(REF_LIB)
        L = self.lib
        L.ref_sizeof.restype = I
        L.ref_wanghash.restype = C.c_uint
        L.ref_wanghash.argtypes = [I]
        L.ref_intersect.argtypes = [P, P, I, I, P, P, P, P, I, P, P]
        L.ref_occlusion.argtypes = [P, P, I, P, P, P, P, I, P, P]
        L.ref_raygen.argtypes = [P, P, P, F, I]
        L.ref_random.argtypes = [P, F, I, I, P]
        L.ref_light_list.restype = I
        L.ref_light_list.argtypes = [P, I, P, P]
        L.ref_scan_int.restype = I
        L.ref_scan_int.argtypes = [P, I, P, I]
        L.ref_env_lum_sat.argtypes = [P, I, I, P, P]
        L.ref_sat_sample.argtypes = [P, P, P, F, F, P, P, P]
        L.ref_sat_sample_discrete.argtypes = [P, P, P, F, F, P, P]
        L.ref_sat_pdf.restype = F
        L.ref_sat_pdf.argtypes = [P, P, P, I, I]
        L.ref_env_illuminate.argtypes = [P, P, P, I, I, P, P, P, P]
        L.ref_env_radiance.argtypes = [P, P, P, I, I, P, P, P]
        L.ref_lightgrid_sat.argtypes = [P, P, I, I, I, I]
        L.ref_lightgrid_sample.argtypes = [P, P, I, I, I, I, I, F, F, P, P, P]
        L.ref_env_grid_illuminate.argtypes = [P, P, P, I, I, P, P, I, I, I, I, P, P, P, P, P, P, P, P]
        L.ref_env_grid_radiance.argtypes = [P, P, P, I, I, P, P, I, I, I, I, P, P, P, P, P, P, P]
        L.ref_average_accum.argtypes = [P, F, I, P, P, P]
        L.ref_preview.argtypes = [P, I, I, P, P, P, P, I, P, P, P, P, I, I, I, P, P]
        L.ref_set_textures.argtypes = [P, P, I]
        L.ref_texture_apply.argtypes = [P, I, F, F, P, P, I, P]
        L.ref_update_frame_image.argtypes = [P, P, F, I, I, F, F]
        L.ref_lightgrid_global_index.restype = I
        L.ref_lightgrid_global_index.argtypes = [I, I, I, I, I, I, I]
        L.ref_bsdf_sample.restype = I
        L.ref_bsdf_sample.argtypes = [P, P, P, P, P, P, P, P, P, P]
        L.ref_bsdf_eval.restype = I
        L.ref_bsdf_eval.argtypes = [P, P, P, P, P, P, P, P]
        L.ref_render_frame.restype = I
        L.ref_render_frame.argtypes = [P, I, I, I, P, F, P, P, P, P, I, P, P, P, P, P, P, I, I, I, P, P]


def bvh_build(orc: Oracle, scene):
    """CNormalBVH restatement: (nodes int32[2N-1, 7], bounds float32[2N-1, 8], depth, order)."""
    n = scene.ntri
    nodes = np.zeros((2 * n - 1, 7), np.int32)
    bounds = np.zeros((2 * n - 1, 8), np.float32)
    order = np.zeros(n, np.int32)
    depth = orc.lib.or_bvh_build(ptr(scene.points), ptr(scene.faces), n, ptr(nodes), ptr(bounds), ptr(order))
    return nodes, bounds, depth, order
