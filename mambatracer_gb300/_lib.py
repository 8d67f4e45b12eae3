"""ctypes binding of libmambatracer.so (the C-ABI in include/mambatracer.h).

The library is required: importing the package's runtime API without it raises,
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmambatracer.so")

MT_OK = 0
ERRORS = {-1: "MT_ERR_INVALID", -2: "MT_ERR_CUDA", -3: "MT_ERR_NOMEM", -4: "MT_ERR_DEPTH", -5: "MT_ERR_DEVICE",
          -6: "MT_ERR_BUSY"}


class MTError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class RenderConfig(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("max_depth", C.c_int), ("mode", C.c_int),
                ("rr_depth", C.c_int), ("film_kahan", C.c_int), ("spp", C.c_int), ("use_graph", C.c_int),
                ("profile", C.c_int), ("inflight", C.c_int),
                ("grid_updates", C.c_int)]


class BatchFrame(C.Structure):
    """mt_batch_frame"""
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("spp", C.c_int), ("frame_count", C.c_float),
                ("camera", C.c_ubyte * 64)]


class ServerConfig(C.Structure):
    _fields_ = [("lanes", C.c_int), ("max_width", C.c_int), ("max_height", C.c_int), ("max_spp", C.c_int),
                ("max_depth", C.c_int), ("rr_depth", C.c_int), ("film_kahan", C.c_int), ("merged", C.c_int),
                ("budget_bytes", C.c_uint64)]


class Tuning(C.Structure):
    """mt_tuning"""
    _fields_ = [("closest_minb", C.c_int), ("shadow_minb", C.c_int), ("closest_grid", C.c_int),
                ("shadow_grid", C.c_int), ("shade_minb", C.c_int), ("refill_steps", C.c_int),
                ("shadow_stream", C.c_int)]


class ServedStats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("cancelled", C.c_int64), ("failed", C.c_int64), ("queued", C.c_int64),
                ("running", C.c_int64), ("max_queue", C.c_int64), ("rays", C.c_int64 * 3), ("p50_ms", C.c_double),
                ("p95_ms", C.c_double), ("p99_ms", C.c_double), ("max_ms", C.c_double), ("span_ms", C.c_double)]


P = C.c_void_p
I = C.c_int
F = C.c_float
PI = C.POINTER(C.c_int)

# name -> (restype, argtypes)
SIGNATURES = {
    "mt_ctx_create": (I, [I, C.POINTER(P)]),
    "mt_ctx_destroy": (I, [P]),
    "mt_finish": (I, [P]),
    "mt_last_error": (C.c_char_p, []),
    "mt_version": (C.c_char_p, []),
    "mt_buf_alloc": (I, [P, C.c_size_t, C.POINTER(P)]),
    "mt_buf_create_from": (I, [P, P, C.c_size_t, C.POINTER(P)]),
    "mt_buf_write": (I, [P, C.c_size_t, P, C.c_size_t]),
    "mt_buf_read": (I, [P, C.c_size_t, P, C.c_size_t]),
    "mt_buf_fill32": (I, [P, C.c_uint32, C.c_size_t, C.c_size_t]),
    "mt_buf_size": (C.c_size_t, [P]),
    "mt_buf_free": (I, [P]),
    "mt_kernel_create": (I, [P, C.c_char_p, C.POINTER(P)]),
    "mt_kernel_names": (C.c_char_p, []),
    "mt_kernel_set_arg_buf": (I, [P, I, P]),
    "mt_kernel_set_arg_local": (I, [P, I, C.c_size_t]),
    "mt_launch_1d": (I, [P, C.c_size_t, C.c_size_t]),
    "mt_kernel_destroy": (I, [P]),
    "mt_scene_create": (I, [P, P, I, P, I, P, I, P, I, P, I, C.POINTER(P)]),
    "mt_bvh_build": (I, [P, P, P, PI]),
    "mt_bvh_build_host": (I, [P, I, P, I, P, P, PI]),
    "mt_bvh_import": (I, [P, P, P, I]),
    "mt_scene_set_bvh_precision": (I, [P, I]),
    "mt_scene_set_materials": (I, [P, P, I]),
    "mt_scene_light_count": (I, [P]),
    "mt_batch_render": (I, [P, P, P, I, I, I, I, P, P]),
    "mt_obj_parse": (I, [P, C.c_size_t, P, P, P, P, P]),
    "mt_tuning_get": (I, [C.POINTER(Tuning)]),
    "mt_tuning_set": (I, [C.POINTER(Tuning)]),
    "mt_scene_set_texture": (I, [P, I, I, P, I, I]),
    "mt_scene_layout_read": (I, [P, P, P, PI, PI]),
    "mt_scene_destroy": (I, [P]),
    "mt_env_set": (I, [P, P, I, I]),
    "mt_env_set_with_sat": (I, [P, P, P, P, I, I]),
    "mt_env_clear": (I, [P]),
    "mt_env_read": (I, [P, P, P, P]),
    "mt_env_grid_config": (I, [P, I, I, I, I, I]),
    "mt_env_grid_sat": (I, [P, P, P, I, I, I, I, I]),
    "mt_job_create": (I, [P, P, C.POINTER(RenderConfig), C.POINTER(P)]),
    "mt_job_destroy": (I, [P]),
    "mt_job_set_camera": (I, [P, P]),
    "mt_render_frame": (I, [P, P, F]),
    "mt_film_read": (I, [P, P, I]),
    "mt_film_read_async": (I, [P, P, I]),
    "mt_job_grid_read": (I, [P, P, P, P]),
    "mt_image_argb": (I, [P, P, F, F, P]),
    "mt_preview_frame": (I, [P, P, I, I, P, P]),
    "mt_bvh_build_device": (I, [P, P, P, PI]),
    "mt_server_create": (I, [P, C.POINTER(ServerConfig), C.POINTER(P)]),
    "mt_server_destroy": (I, [P]),
    "mt_job_submit": (I, [P, P, P, I, I, I, F, P, C.POINTER(C.c_int64)]),
    "mt_job_poll": (I, [P, C.c_int64, PI, C.POINTER(C.c_double)]),
    "mt_job_cancel": (I, [P, C.c_int64]),
    "mt_job_wait": (I, [P, C.c_int64, C.c_double]),
    "mt_server_drain": (I, [P]),
    "mt_server_stats": (I, [P, C.POINTER(ServedStats)]),
    "mt_film_wait": (I, [P]),
    "mt_film_clear": (I, [P]),
    "mt_job_stats": (I, [P, P, P]),
    "mt_job_last_ms": (I, [P, C.POINTER(C.c_float)]),
    "mt_job_launches": (I, [P, C.POINTER(C.c_int64)]),
    "mt_job_kernel_ms": (I, [P, P]),
    "mt_job_total_rays": (I, [P, P]),
    "mt_ctx_event_record": (I, [P, I]),
    "mt_ctx_event_elapsed": (I, [P, I, I, C.POINTER(C.c_float)]),
    "mt_compact_isects": (I, [P, P, P, I, P, P, P]),
    "mt_buf_device_ptr": (P, [P]),
    "mt_compact_isects_noalloc": (I, [P, P, P, I, P, P, P]),
    "mt_trace_closest": (I, [P, P, I, P, P]),
    "mt_trace_any": (I, [P, P, I, P]),
    "mt_trace_counts": (I, [P, P, I, I, P, P, P]),
    "mt_trace_closest_dev": (I, [P, P, I, P, P, C.POINTER(C.c_float)]),
}

_lib = None


def lib() -> C.CDLL:
    """The loaded library; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with mambatracer_gb300.build.build() "
                              "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code: int) -> None:
    if code != MT_OK:
        raise MTError(code, lib().mt_last_error().decode())
