"""ctypes binding of libraymond_cuda.so (include/raymond.h). The library is
required: nothing here falls back to a CPU path."""

from __future__ import annotations

import ctypes
import os
import threading

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libraymond_cuda.so")

OK, EINVAL, ENOMEM, ECUDA, ESTATE, ETIMEOUT, ECAPACITY = 0, -1, -2, -3, -4, -5, -6
FEATURE_VOLUMES, FEATURE_TEXTURES, FEATURE_ENVIRONMENT, FEATURE_DISPERSION = 1, 2, 4, 8
FLAG_CAUSTICS, FLAG_DENOISE, FLAG_MEGAKERNEL, FLAG_WAVEFRONT = 1, 2, 4, 8


class RaymondError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("seed", ctypes.c_uint32), ("path_capacity", ctypes.c_uint64),
                ("reserved", ctypes.c_uint32 * 4)]


class Buffers(ctypes.Structure):
    _fields_ = [("accum", ctypes.c_void_p), ("guide_albedo", ctypes.c_void_p), ("guide_normal", ctypes.c_void_p),
                ("denoised", ctypes.c_void_p), ("display", ctypes.c_void_p), ("width", ctypes.c_uint32),
                ("height", ctypes.c_uint32)]


class Stats(ctypes.Structure):
    _fields_ = [("launches", ctypes.c_uint64), ("rays_primary", ctypes.c_uint64),
                ("rays_extension", ctypes.c_uint64), ("rays_shadow", ctypes.c_uint64),
                ("rays_photon", ctypes.c_uint64), ("paths", ctypes.c_uint64), ("ms_trace", ctypes.c_float),
                ("ms_caustics", ctypes.c_float), ("ms_denoise", ctypes.c_float), ("ms_display", ctypes.c_float),
                ("ms_extend", ctypes.c_float), ("ms_shade", ctypes.c_float), ("ms_shadow", ctypes.c_float),
                ("launches_extend", ctypes.c_uint32), ("launches_shade", ctypes.c_uint32),
                ("launches_shadow", ctypes.c_uint32)]


class Tuning(ctypes.Structure):
    _fields_ = [("path", ctypes.c_uint32), ("steps", ctypes.c_uint32), ("traversal_blocks_per_sm", ctypes.c_uint32),
                ("shade_blocks_per_sm", ctypes.c_uint32)]


PATH_MEGAKERNEL, PATH_WAVEFRONT = 1, 2
BATCH_GRAPH = 1


class Job(ctypes.Structure):
    _fields_ = [("renderer", ctypes.c_void_p), ("params208", ctypes.c_void_p), ("features", ctypes.c_uint32)]


# Every symbol include/raymond.h declares, with its ctypes signature.
_P = ctypes.c_void_p
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_I = ctypes.c_int
SIGNATURES = {
    "raymond_create": (_I, [ctypes.POINTER(_P), ctypes.POINTER(Config)]),
    "raymond_destroy": (None, [_P]),
    "raymond_last_error": (ctypes.c_char_p, [_P]),
    "raymond_upload_scene": (_I, [_P, _P, _U32, _U32, _P, _U32, _P, _U32, _P, _U32, _P, _U32, _U32, _U32]),
    "raymond_upload_textures": (_I, [_P, _I, _P, _U32, _U32, _U32]),
    "raymond_upload_environment": (_I, [_P, _P, _U32, _U32, _P, _U32, _U32]),
    "raymond_set_emitters": (_I, [_P, _P, _U32]),
    "raymond_resize": (_I, [_P, _U32, _U32]),
    "raymond_render": (_I, [_P, _P, _U32, _U32]),
    "raymond_sync": (_I, [_P]),
    "raymond_read_pixels": (_I, [_P, _P, _U64, _I, _U32]),
    "raymond_read_display": (_I, [_P, _P, _U64]),
    "raymond_read_guides": (_I, [_P, _P, _P, _P, _U64]),
    "raymond_trace_primary": (_I, [_P, _P, _U32, _P, _P]),
    "raymond_trace_primary_device": (_I, [_P, _P, _U32, _P, _P]),
    "raymond_bvh_build": (_U32, [_P, _P, _U32, _U32, _P, _P, _I]),
    "raymond_get_buffers": (_I, [_P, ctypes.POINTER(Buffers)]),
    "raymond_get_stats": (_I, [_P, ctypes.POINTER(Stats)]),
    "raymond_get_stream": (_P, [_P]),
    "raymond_denoise_static": (_I, [_P, _P, _P, _U32, _U32, _U32, _P, _P]),
    "raymond_set_tuning": (_I, [_P, ctypes.POINTER(Tuning)]),
    "raymond_set_photons": (_I, [_P, _U32, _U32, ctypes.c_float]),
    "raymond_render_batch": (_I, [_P, ctypes.POINTER(Job), _U32, _U32]),
    "raymond_get_tuning": (_I, [_P, ctypes.POINTER(Tuning)]),
    "raymond_autotune": (_I, [_P, _P, _U32, _U32, ctypes.POINTER(Tuning)]),
}

_lib = None
_lock = threading.Lock()


def lib():
    """The loaded library; raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is None:
            if not os.path.exists(LIB_PATH):
                raise RuntimeError(f"{LIB_PATH} is missing: build it with raymond_gb300.build.build() "
                                   "(the render path has no CPU fallback)")
            handle = ctypes.CDLL(LIB_PATH)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(handle, name)
                fn.restype = res
                fn.argtypes = args
            _lib = handle
    return _lib


def check(rc: int, handle=None):
    if rc != OK:
        msg = lib().raymond_last_error(handle)
        raise RaymondError(rc, msg.decode() if msg else f"raymond error {rc}")


def ptr(a) -> int:
    """Address of a numpy array's data."""
    return a.ctypes.data if a is not None else None
