"""ctypes binding of libgbpt.so (the C ABI in include/gbpt.h).

The library is built in-tree by ``cudapt_gb300.build.build()``.  Loading
fails loudly when it is missing: there is no CPU fallback.
"""
import ctypes
import os
import threading

import numpy as np

from . import build as _build

_lock = threading.Lock()
_lib = None

STATUS = {
    0: "GBPT_OK",
    1: "GBPT_ERR_INVALID_ARG",
    2: "GBPT_ERR_OOM",
    3: "GBPT_ERR_CUDA",
    4: "GBPT_ERR_TIMEOUT",
    5: "GBPT_ERR_BOUNDS",
    6: "GBPT_ERR_STATE",
    7: "GBPT_ERR_NO_DEVICE",
}


class GbptError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class Texture(ctypes.Structure):
    """gbpt_texture: RTTexture (include/raytracer.h:219-226)."""
    _fields_ = [("rgba", ctypes.c_void_p), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [
        ("frame", ctypes.c_uint32),
        ("light_vertices", ctypes.c_uint32),
        ("paths", ctypes.c_uint64),
        ("rays", ctypes.c_uint64),
        ("shadow_rays", ctypes.c_uint64),
        ("nodes", ctypes.c_uint64),
        ("tris", ctypes.c_uint64),
        ("shadow_nodes", ctypes.c_uint64),
        ("shadow_tris", ctypes.c_uint64),
        ("ms_total", ctypes.c_float),
        ("ms_light", ctypes.c_float),
        ("ms_trace", ctypes.c_float),
        ("ms_shade", ctypes.c_float),
        ("ms_shadow", ctypes.c_float),
        ("ms_filter", ctypes.c_float),
        ("ms_adapt", ctypes.c_float),
        ("launches", ctypes.c_uint32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class Request(ctypes.Structure):
    """gbpt_request (80 bytes)."""
    _fields_ = [
        ("scene", ctypes.c_void_p),
        ("camera", ctypes.c_float * 10),
        ("width", ctypes.c_uint32),
        ("height", ctypes.c_uint32),
        ("frames", ctypes.c_uint32),
        ("mode", ctypes.c_int32),
        ("params", ctypes.c_void_p),
        ("out_rgb", ctypes.c_void_p),
    ]


class RequestStatus(ctypes.Structure):
    """gbpt_request_status (56 bytes)."""
    _fields_ = [
        ("id", ctypes.c_uint64),
        ("status", ctypes.c_int32),
        ("done", ctypes.c_uint32),
        ("queued_ms", ctypes.c_double),
        ("run_ms", ctypes.c_double),
        ("latency_ms", ctypes.c_double),
        ("paths", ctypes.c_uint64),
        ("walk_refill", ctypes.c_uint32),
        ("tail_from", ctypes.c_int32),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


assert ctypes.sizeof(Request) == 80 and ctypes.sizeof(RequestStatus) == 56


# every exported entry point of include/gbpt.h with its ctypes signature
vp, u32, i32, f32, f64p = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int32, ctypes.c_float, ctypes.c_void_p
SIGNATURES = {
    "gbpt_last_error_string": (ctypes.c_char_p, []),
    "gbpt_device_check": (i32, [vp]),
    "gbpt_params_default": (i32, [vp]),
    "gbpt_scene_create": (i32, [vp, u32, vp, u32, vp, u32, vp]),
    "gbpt_scene_destroy": (i32, [vp]),
    "gbpt_scene_build_bvh": (i32, [vp, u32, u32, vp]),
    "gbpt_scene_update_materials": (i32, [vp, vp, u32]),
    "gbpt_scene_set_traversal": (i32, [vp, i32]),
    "gbpt_scene_set_textures": (i32, [vp, vp, u32]),
    "gbpt_scene_bvh_info": (i32, [vp, vp, vp, vp]),
    "gbpt_scene_bvh_export": (i32, [vp, vp, vp, vp]),
    "gbpt_trace_rays": (i32, [vp, vp, u32, f32, f32, i32, vp, vp, vp, vp, vp, vp, vp, i32]),
    "gbpt_renderer_create": (i32, [u32, u32, i32, vp, vp]),
    "gbpt_renderer_destroy": (i32, [vp]),
    "gbpt_set_mode": (i32, [vp, i32]),
    "gbpt_renderer_set_window": (i32, [vp, u32, u32, u32, u32]),
    "gbpt_set_params": (i32, [vp, vp]),
    "gbpt_get_params": (i32, [vp, vp]),
    "gbpt_render": (i32, [vp, vp, vp, vp, i32, vp]),
    "gbpt_render_frames": (i32, [vp, vp, vp, u32, vp]),
    "gbpt_result": (ctypes.POINTER(ctypes.c_float), [vp]),
    "gbpt_read_buffer": (i32, [vp, i32, vp, ctypes.c_size_t, i32]),
    "gbpt_host_register": (i32, [vp, ctypes.c_size_t]),
    "gbpt_host_unregister": (i32, [vp]),
    "gbpt_server_create": (i32, [u32, ctypes.c_uint64, vp]),
    "gbpt_server_destroy": (i32, [vp]),
    "gbpt_server_set_policy": (i32, [vp, i32]),
    "gbpt_selftest_wait_timeout": (i32, [vp]),
    "gbpt_test_fail_allocations": (i32, [ctypes.c_int64]),
    "gbpt_renderer_checkpoint_size": (i32, [vp, vp]),
    "gbpt_renderer_checkpoint": (i32, [vp, vp, ctypes.c_size_t]),
    "gbpt_renderer_restore": (i32, [vp, vp, ctypes.c_size_t]),
    "gbpt_server_release": (i32, [vp, ctypes.c_uint64]),
    "gbpt_server_set_graphs": (i32, [vp, i32]),
    "gbpt_renderer_set_graphs": (i32, [vp, i32]),
    "gbpt_server_submit": (i32, [vp, vp, vp]),
    "gbpt_server_wait": (i32, [vp, ctypes.c_uint64, u32, vp]),
    "gbpt_server_tuned": (i32, [vp, i32, u32, u32, u32, vp, vp, vp]),
    "gbpt_server_tuned_params": (i32, [vp, i32, u32, u32, u32, vp, vp]),
    "gbpt_reset": (i32, [vp]),
    "gbpt_clean": (i32, [vp]),
    "gbpt_set_counting": (i32, [vp, i32]),
    "gbpt_attr_count": (i32, [vp, vp]),
    "gbpt_attr_name": (i32, [vp, u32, vp, ctypes.c_size_t]),
    "gbpt_attr_get": (i32, [vp, ctypes.c_char_p, vp]),
    "gbpt_attr_set": (i32, [vp, ctypes.c_char_p, f32]),
    "gbpt_gaussian_table": (i32, [f32, u32, vp]),
    "gbpt_bilateral": (i32, [vp, vp, vp, vp, u32, u32, f32, f32, f32, f32, u32, vp, vp, i32]),
    "gbpt_bilateral_noalloc": (i32, [vp, vp, vp, vp, u32, u32, f32, f32, f32, f32, u32, vp, vp, vp]),
    "gbpt_rmse": (i32, [vp, vp, ctypes.c_uint64, i32, vp]),
    "gbpt_renderer_rmse": (i32, [vp, vp, i32, vp]),
    "gbpt_tonemap_rgba8": (i32, [vp, vp, u32, u32, f32, i32, vp, i32]),
    "gbpt_mlp_param_count": (u32, []),
    "gbpt_mlp_create": (i32, [u32, vp]),
    "gbpt_mlp_destroy": (i32, [vp]),
    "gbpt_mlp_get_params": (i32, [vp, vp]),
    "gbpt_mlp_set_params": (i32, [vp, vp]),
    "gbpt_mlp_forward": (i32, [vp, vp, u32, vp, i32]),
    "gbpt_mlp_gradients": (i32, [vp, vp, vp, u32, i32, vp, vp]),
    "gbpt_mlp_train_step": (i32, [vp, vp, vp, u32, f32, i32, vp]),
    "gbpt_renderer_set_stream": (i32, [vp, vp]),
    "gbpt_renderer_set_mlp": (i32, [vp, vp, i32]),
    "gbpt_renderer_features": (i32, [vp, vp, u32, i32, vp]),
    "gbpt_fmath": (i32, [i32, vp, u32, vp]),
    "gbpt_texture_sample": (i32, [vp, u32, u32, vp, u32, i32, vp]),
    "gbpt_philox": (i32, [vp, u32, u32, u32, vp]),
}


def lib_path():
    return _build.LIB


def load(build_if_missing=False):
    """Load libgbpt.so; raise if it is missing (no fallback path exists)."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = lib_path()
        if not os.path.exists(path):
            if build_if_missing:
                _build.build()
            else:
                raise RuntimeError(f"libgbpt.so not found at {path}; run cudapt_gb300.build.build()")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
        return L


def check(status):
    if status != 0:
        msg = load().gbpt_last_error_string().decode(errors="replace")
        raise GbptError(status, msg)


def ptr(a):
    return None if a is None else a.ctypes.data


def as_c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)
