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
                ("shade_blocks_per_sm", ctypes.c_uint32), ("bvh_width", ctypes.c_uint32)]


PATH_MEGAKERNEL, PATH_WAVEFRONT = 1, 2
BATCH_GRAPH = 1


class Job(ctypes.Structure):
    _fields_ = [("renderer", ctypes.c_void_p), ("params208", ctypes.c_void_p), ("features", ctypes.c_uint32)]


class NetConfig(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("seed", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 6)]


class NetBatch(ctypes.Structure):
    _fields_ = [("accum", ctypes.c_void_p), ("albedo", ctypes.c_void_p), ("normal", ctypes.c_void_p),
                ("target", ctypes.c_void_p), ("samples", ctypes.c_void_p), ("samples_all", ctypes.c_float),
                ("n", ctypes.c_uint32), ("width", ctypes.c_uint32), ("height", ctypes.c_uint32)]


class Conv(ctypes.Structure):
    _fields_ = [("n", ctypes.c_uint32), ("height", ctypes.c_uint32), ("width", ctypes.c_uint32),
                ("cin", ctypes.c_uint32), ("cout", ctypes.c_uint32),
                ("src0", ctypes.c_void_p), ("src0_channels", ctypes.c_uint32), ("src0_stride", ctypes.c_uint32),
                ("src0_shift", ctypes.c_uint32),
                ("src1", ctypes.c_void_p), ("src1_channels", ctypes.c_uint32), ("src1_stride", ctypes.c_uint32),
                ("src1_shift", ctypes.c_uint32),
                ("weight", ctypes.c_void_p), ("bias", ctypes.c_void_p), ("dy", ctypes.c_void_p),
                ("dy_stride", ctypes.c_uint32), ("out", ctypes.c_void_p), ("out_stride", ctypes.c_uint32),
                ("out_f32", ctypes.c_void_p), ("mask", ctypes.c_void_p), ("mask_stride", ctypes.c_uint32),
                ("dweight", ctypes.c_void_p), ("dbias", ctypes.c_void_p), ("activation", ctypes.c_int32),
                ("pixels_per_cta", ctypes.c_uint32), ("status", ctypes.c_void_p), ("kernel", ctypes.c_uint32)]


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
    "raymond_upload_texture_images": (_I, [_P, _I, _P, _P, _P, _U32, _I, _P]),
    "raymond_upload_environment_rgb": (_I, [_P, _P, _U32, _U32, _P, _U32]),
    "raymond_read_textures": (_I, [_P, _I, _P, _U64]),
    "raymond_read_environment": (_I, [_P, _P, _U64, _P, _U64]),
    "raymond_resize": (_I, [_P, _U32, _U32]),
    "raymond_render": (_I, [_P, _P, _U32, _U32]),
    "raymond_sync": (_I, [_P]),
    "raymond_read_pixels": (_I, [_P, _P, _U64, _I, _U32]),
    "raymond_read_display": (_I, [_P, _P, _U64]),
    "raymond_read_guides": (_I, [_P, _P, _P, _P, _U64]),
    "raymond_trace_primary": (_I, [_P, _P, _U32, _P, _P]),
    "raymond_trace_primary_device": (_I, [_P, _P, _U32, _P, _P]),
    "raymond_bvh_build": (_U32, [_P, _P, _U32, _U32, _P, _P, _I]),
    "raymond_sample_streams": (_I, [_P, _P, _U32, _P, _U32, _U32, _U32, _P]),
    "raymond_light_trace": (_I, [_P, _P, _U32, _P, _U64, _P, _U64, _P]),
    "raymond_photon_gather": (_I, [_P, _P, _U32, _P, _U32, _P, _U64]),
    "raymond_get_buffers": (_I, [_P, ctypes.POINTER(Buffers)]),
    "raymond_get_stats": (_I, [_P, ctypes.POINTER(Stats)]),
    "raymond_get_stream": (_P, [_P]),
    "raymond_denoise_static": (_I, [_P, _P, _P, _U32, _U32, _U32, _P, _P]),
    "raymond_set_tuning": (_I, [_P, ctypes.POINTER(Tuning)]),
    "raymond_set_photons": (_I, [_P, _U32, _U32, ctypes.c_float]),
    "raymond_render_batch": (_I, [_P, ctypes.POINTER(Job), _U32, _U32]),
    "raymond_get_tuning": (_I, [_P, ctypes.POINTER(Tuning)]),
    "raymond_autotune": (_I, [_P, _P, _U32, _U32, ctypes.POINTER(Tuning)]),
    "raymond_net_create": (_I, [ctypes.POINTER(_P), ctypes.POINTER(NetConfig)]),
    "raymond_net_destroy": (None, [_P]),
    "raymond_net_last_error": (ctypes.c_char_p, [_P]),
    "raymond_net_param_count": (_U64, [_P]),
    "raymond_net_layout": (_I, [_P, _P, _P, _P, _P, _U32]),
    "raymond_net_set_params": (_I, [_P, _P, _U64]),
    "raymond_net_get_params": (_I, [_P, _P, _U64]),
    "raymond_net_gradients": (_I, [_P, ctypes.POINTER(NetBatch), _P, _U64, _P]),
    "raymond_net_train_step": (_I, [_P, ctypes.POINTER(NetBatch), ctypes.c_float, _P]),
    "raymond_net_sync": (_I, [_P]),
    "raymond_net_set_loss": (_I, [_P, ctypes.c_float, ctypes.c_float, ctypes.c_float]),
    "raymond_net_set_blend": (_I, [_P, ctypes.c_float]),
    "raymond_net_get_blend": (ctypes.c_float, [_P]),
    "raymond_net_infer": (_I, [_P, ctypes.POINTER(NetBatch), _P, _P]),
    "raymond_net_get_stream": (_P, [_P]),
    "raymond_net_set_stream": (_I, [_P, _P]),
    "raymond_denoise_learned": (_I, [_P, _P, _U32, _P]),
    "raymond_conv3x3_forward": (_I, [ctypes.POINTER(Conv), _P]),
    "raymond_conv3x3_backward_data": (_I, [ctypes.POINTER(Conv), _P]),
    "raymond_conv3x3_backward_weight": (_I, [ctypes.POINTER(Conv), _P]),
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


def check_net(rc: int, net):
    if rc != OK:
        msg = lib().raymond_net_last_error(net)
        raise RaymondError(rc, msg.decode() if msg else f"raymond error {rc}")


def ptr(a) -> int:
    """Address of a numpy array's data."""
    return a.ctypes.data if a is not None else None
