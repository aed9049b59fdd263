"""ctypes binding of the renderer's C ABI (``include/gvr.h``).

The native library is ``ascent_gb300/_lib/libgvr.so``, built in-tree by
``ascent_gb300/build.py``. There is no fallback: if the library is missing
or does not load, every call raises :class:`GvrError`.
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libgvr.so"

GVR_OK = 0
GVR_ERR_INVALID_ARGUMENT = 1
GVR_ERR_CUDA = 2
GVR_ERR_OUT_OF_MEMORY = 3
GVR_ERR_UNSUPPORTED = 4
GVR_ERR_TIMEOUT = 5
GVR_ERR_NOT_FOUND = 6

MEM_HOST, MEM_DEVICE = 0, 1
DTYPE_FLOAT32, DTYPE_FLOAT64 = 0, 1
ASSOC_VERTEX, ASSOC_ELEMENT = 0, 1
LUT_NEAREST, LUT_LINEAR = 0, 1
UINT8_NONE, UINT8_ROUND, UINT8_TRUNCATE = 0, 1, 2


class GvrError(RuntimeError):
    """A C-ABI call returned a non-zero gvr_status."""

    def __init__(self, code: int, message: str):
        super().__init__(f"gvr error {code}: {message}")
        self.code = code


class Camera(C.Structure):
    _fields_ = [("position", C.c_float * 3), ("look_at", C.c_float * 3), ("up", C.c_float * 3),
                ("fov_y", C.c_float), ("zoom", C.c_float), ("xpan", C.c_float), ("ypan", C.c_float),
                ("near_plane", C.c_float), ("far_plane", C.c_float)]

    def as_dict(self) -> dict:
        return {"position": list(self.position), "look_at": list(self.look_at), "up": list(self.up),
                "fov": self.fov_y, "zoom": self.zoom, "xpan": self.xpan, "ypan": self.ypan,
                "near_plane": self.near_plane, "far_plane": self.far_plane}

    def copy(self) -> "Camera":
        c = Camera()
        C.memmove(C.byref(c), C.byref(self), C.sizeof(Camera))
        return c


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("sample_dist", C.c_float),
                ("scalar_min", C.c_float), ("scalar_max", C.c_float),
                ("lut_rgba", C.POINTER(C.c_float)), ("lut_size", C.c_int), ("lut_filter", C.c_int),
                ("alpha_cull", C.c_float), ("early_term", C.c_float), ("quantize_uint8", C.c_int),
                ("render_bg", C.c_int), ("bg_color", C.c_float * 4), ("clear_depth", C.c_float)]


class ColorTable(C.Structure):
    _fields_ = [("n_rgb", C.c_int), ("rgb_pos", C.POINTER(C.c_double)), ("rgb", C.POINTER(C.c_double)),
                ("n_alpha", C.c_int), ("alpha_pos", C.POINTER(C.c_double)),
                ("alpha", C.POINTER(C.c_double))]


def dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def fptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def make_params(width, height, sample_dist, scalar_range, lut, *, lut_filter=LUT_NEAREST,
                alpha_cull=0.001, early_term=0.99, quantize_uint8=False, render_bg=False,
                bg_color=(0.0, 0.0, 0.0, 1.0), clear_depth=1.0):
    """Build a RenderParams; the LUT array must stay alive while it is used."""
    lut = np.ascontiguousarray(lut, dtype=np.float32).reshape(-1, 4)
    p = RenderParams()
    p.width, p.height = int(width), int(height)
    p.sample_dist = float(sample_dist)
    p.scalar_min, p.scalar_max = float(scalar_range[0]), float(scalar_range[1])
    p.lut_rgba = fptr(lut)
    p.lut_size = lut.shape[0]
    p.lut_filter = int(lut_filter)
    p.alpha_cull = float(alpha_cull)
    p.early_term = float(early_term)
    p.quantize_uint8 = int(bool(quantize_uint8))
    p.render_bg = int(bool(render_bg))
    for i in range(4):
        p.bg_color[i] = float(bg_color[i])
    p.clear_depth = float(clear_depth)
    p._lut_keepalive = lut  # noqa: SLF001 - keep the buffer referenced
    return p


_lib = None
_lock = threading.Lock()

_SIGS = {
    "gvr_last_error": (C.c_char_p, []),
    "gvr_version": (C.c_int, []),
    "gvr_launch_count": (C.c_int, [C.POINTER(C.c_uint64)]),
    "gvr_scratch_trim": (C.c_int, [C.c_int, C.c_uint64, C.POINTER(C.c_uint64)]),
    "gvr_scene_set_staging": (C.c_int, [C.c_void_p, C.c_int]),
    "gvr_scene_set_tile_order": (C.c_int, [C.c_void_p, C.c_int]),
    "gvr_scene_set_brick_cells": (C.c_int, [C.c_void_p, C.c_int]),
    "gvr_scene_staging_failures": (C.c_int, [C.c_void_p, C.POINTER(C.c_uint64)]),
    "gvr_composite_partials_async": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_void_p,
                                               C.c_void_p, C.c_void_p]),
    "gvr_zbuffer_composite": (C.c_int, [C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.c_int,
                                        C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    "gvr_correct_opacity": (C.c_int, [C.POINTER(C.c_double), C.c_int, C.c_int, C.POINTER(C.c_double)]),
    "gvr_sample_distance": (C.c_int, [C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_float)]),
    "gvr_color_table_sample": (C.c_int, [C.POINTER(ColorTable), C.c_int, C.c_int, C.POINTER(C.c_float)]),
    "gvr_camera_reset_to_bounds": (C.c_int, [C.POINTER(Camera), C.POINTER(C.c_double)]),
    "gvr_camera_azimuth": (C.c_int, [C.POINTER(Camera), C.c_double]),
    "gvr_camera_elevation": (C.c_int, [C.POINTER(Camera), C.c_double]),
    "gvr_cinema_cameras": (C.c_int, [C.POINTER(C.c_double), C.POINTER(C.c_float), C.c_int, C.POINTER(Camera)]),
    "gvr_visibility_order": (C.c_int, [C.POINTER(Camera), C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_int)]),
    "gvr_scene_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "gvr_scene_destroy": (C.c_int, [C.c_void_p]),
    "gvr_scene_add_uniform": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.c_void_p, C.c_int, C.c_int64,
                                        C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "gvr_scene_add_rectilinear": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                            C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p,
                                            C.c_int, C.c_int64, C.c_int, C.c_int, C.POINTER(C.c_int)]),
    "gvr_scene_add_hex": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                    C.c_int64, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int,
                                    C.c_int, C.POINTER(C.c_int)]),
    "gvr_scene_hex_bvh": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_void_p, C.c_void_p, C.POINTER(C.c_float)]),
    "gvr_scene_hex_locate": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "gvr_scene_update_field": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_int64, C.c_int]),
    "gvr_scene_num_domains": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "gvr_scene_set_tuning": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    "gvr_diff_workspace": (C.c_int, [C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_float,
                                     C.POINTER(C.c_int)]),
    "gvr_diff_render_forward": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                          C.POINTER(C.c_double), C.c_void_p, C.c_int,
                                          C.POINTER(RenderParams), C.c_void_p, C.c_void_p, C.c_void_p,
                                          C.c_void_p]),
    "gvr_diff_render_backward": (C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                           C.POINTER(C.c_double), C.c_void_p, C.c_int,
                                           C.POINTER(RenderParams), C.c_void_p, C.c_void_p,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "gvr_scene_set_batch_granularity": (C.c_int, [C.c_void_p, C.c_int]),
    "gvr_scene_batch_graph_builds": (C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    "gvr_render_volume_batch": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(RenderParams),
                                          C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                          C.POINTER(C.c_uint64)]),
    "gvr_scene_bounds": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(C.c_double)]),
    "gvr_scene_range": (C.c_int, [C.c_void_p, C.POINTER(C.c_double)]),
    "gvr_render_volume": (C.c_int, [C.c_void_p, C.POINTER(Camera), C.POINTER(RenderParams), C.c_void_p,
                                    C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_uint64)]),
    "gvr_scene_update_fields": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int,
                                          C.c_int64, C.c_int, C.c_void_p]),
    "gvr_scene_hex_neighbors": (C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.POINTER(C.c_float)]),
    "gvr_render_volume_over": (C.c_int, [C.c_void_p, C.POINTER(Camera), C.POINTER(RenderParams),
                                         C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                         C.POINTER(C.c_uint64)]),
    "gvr_canvas_to_rgba8": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_int, C.c_void_p]),
    "gvr_canvas_color_bar": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_float), C.c_int,
                                       C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_int, C.c_void_p]),
    "gvr_composite_partials": (C.c_int, [C.c_void_p, C.c_int64, C.c_void_p, C.POINTER(C.c_int64),
                                         C.c_int, C.c_void_p]),
}


def lib() -> C.CDLL:
    """Load libgvr.so once and declare every entry point's signature."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not LIB_PATH.exists():
            raise GvrError(GVR_ERR_UNSUPPORTED,
                           f"native library {LIB_PATH} is missing; run ascent_gb300.build.build()")
        handle = C.CDLL(str(LIB_PATH))
        for name, (res, args) in _SIGS.items():
            fn = getattr(handle, name)
            fn.restype = res
            fn.argtypes = args
        _lib = handle
    return _lib


def check(rc: int) -> None:
    if rc != GVR_OK:
        msg = lib().gvr_last_error().decode(errors="replace")
        raise GvrError(rc, msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args))


def launch_count() -> int:
    n = C.c_uint64(0)
    call("gvr_launch_count", C.byref(n))
    return int(n.value)


def scratch_trim(device: int = 0, keep_bytes: int = 0) -> int:
    """Return the library's pooled scratch on `device` to the system down to
    keep_bytes (gvr_scratch_trim); the bytes still reserved."""
    r = C.c_uint64(0)
    call("gvr_scratch_trim", int(device), int(keep_bytes), C.byref(r))
    return int(r.value)
