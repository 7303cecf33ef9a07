"""ctypes binding of ``libc2g.so`` (the C ABI declared in ``include/c2g.h``).

The library is built in-tree (``crystal2_gb300/build.py``).  There is no CPU fallback: when the
shared library is missing, or a call needs a GPU and none is present, the call raises.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libc2g.so")

C2G_OK = 0
C2G_ERR_INVALID = 1
C2G_ERR_IO = 2
C2G_ERR_PARSE = 3
C2G_ERR_CUDA = 4
C2G_ERR_OOM = 5
C2G_ERR_DEVICE = 6
C2G_ERR_STATE = 7
C2G_ERR_UNSUPPORTED = 8

ACCEL_BVH = 0
ACCEL_BRUTE = 1
TREE_REF_EQUAL_COUNT = 0
TREE_SAH = 1
INTEGRATOR_PATH = 0
INTEGRATOR_DIRECT = 1
INTEGRATOR_GUIDED = 2

STATUS_NAMES = {
    C2G_ERR_INVALID: "invalid argument", C2G_ERR_IO: "i/o error", C2G_ERR_PARSE: "parse error",
    C2G_ERR_CUDA: "CUDA error", C2G_ERR_OOM: "out of device memory", C2G_ERR_DEVICE: "device error",
    C2G_ERR_STATE: "bad state", C2G_ERR_UNSUPPORTED: "unsupported",
}


class C2GError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, 'error')} ({code}): {msg}")
        self.code = code


class DeviceOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("mem_limit_bytes", C.c_size_t), ("verbose", C.c_int)]


class RenderParams(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("spp", C.c_int), ("max_depth", C.c_int),
                ("integrator", C.c_int), ("accel", C.c_int), ("sample_begin", C.c_int), ("sample_count", C.c_int),
                ("wave_paths", C.c_int), ("seed", C.c_uint64)]


K_RAYGEN, K_EXTEND, K_SHADE, K_SHADOW, K_MIS, K_ACCUM, K_FILM, K_GUIDE, K_TRAIN = range(9)
K_KINDS = 10
LEVELS = 64
KERNEL_NAMES = ["raygen", "extend", "shade", "shadow", "mis", "accumulate", "film", "guide", "train", "-"]
COUNT_TRAVERSAL = 1
COUNT_TIMING = 2
COUNT_SERIAL = 4


class Stats(C.Structure):
    _fields_ = [("seconds", C.c_double), ("paths", C.c_double), ("rays", C.c_double * K_KINDS),
                ("nodes", C.c_double * K_KINDS), ("prims", C.c_double * K_KINDS), ("kernel_ms", C.c_double * K_KINDS),
                ("kernel_count", C.c_int * K_KINDS),
                ("kernel_launches", C.c_int), ("waves", C.c_int),
                ("level_ms", C.c_double * LEVELS), ("level_paths", C.c_double * LEVELS), ("levels", C.c_int)]


class BatchStats(C.Structure):
    _fields_ = [("jobs", C.c_int), ("paths", C.c_double), ("seconds", C.c_double), ("mpaths_per_s", C.c_double),
                ("latency_p50_ms", C.c_double), ("latency_p99_ms", C.c_double), ("latency_max_ms", C.c_double),
                ("wave_paths", C.c_int), ("streams", C.c_int), ("graph_launches", C.c_int),
                ("latency_p90_ms", C.c_double), ("latency_mean_ms", C.c_double), ("traversal", C.c_int),
                ("trace_block", C.c_int)]


class BatchSpace(C.Structure):
    _fields_ = [("wave_paths", C.POINTER(C.c_int)), ("n_wave_paths", C.c_int), ("streams", C.POINTER(C.c_int)),
                ("n_streams", C.c_int), ("traversal", C.POINTER(C.c_int)), ("n_traversal", C.c_int),
                ("trace_block", C.POINTER(C.c_int)), ("n_trace_block", C.c_int)]


_P = C.c_void_p
_I = C.c_int
_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int)

# name -> (restype, argtypes); this table is also the list of symbols include/c2g.h declares
SIGNATURES = {
    "c2g_create": (_I, [C.POINTER(_P), C.POINTER(DeviceOpts)]),
    "c2g_destroy": (None, [_P]),
    "c2g_last_error": (C.c_char_p, [_P]),
    "c2g_version": (C.c_char_p, []),
    "c2g_load_json": (_I, [_P, C.c_char_p, C.c_char_p, _I]),
    "c2g_load_json_text": (_I, [_P, C.c_char_p, C.c_char_p, _I]),
    "c2g_bvh_build": (_I, [_P, _I]),
    "c2g_get_render_params": (_I, [_P, C.POINTER(RenderParams)]),
    "c2g_num_objects": (_I, [_P]),
    "c2g_num_lights": (_I, [_P]),
    "c2g_bvh_order": (_I, [_P, _IP, _I]),
    "c2g_bvh_nodes": (_I, [_P, _FP, _IP, _IP, _I]),
    "c2g_render": (_I, [_P, C.POINTER(RenderParams), _P]),
    "c2g_render_noalloc": (_I, [_P, C.POINTER(RenderParams), _P, _P]),
    "c2g_film_clear": (_I, [_P, _P]),
    "c2g_film_download": (_I, [_P, _FP, _FP]),
    "c2g_film_image": (_I, [_P, _FP]),
    "c2g_film_rgb8": (_I, [_P, C.c_float, C.POINTER(C.c_ubyte)]),
    "c2g_film_write_hdr": (_I, [_P, C.c_char_p]),
    "c2g_write_hdr": (_I, [C.c_char_p, _I, _I, _FP]),
    "c2g_register_image": (_I, [_P, C.c_char_p, _I, _I, C.POINTER(C.c_ubyte)]),
    "c2g_film_download_m2": (_I, [_P, _FP]),
    "c2g_get_stats": (_I, [_P, C.POINTER(Stats)]),
    "c2g_set_counting": (_I, [_P, _I]),
    "c2g_set_traversal": (_I, [_P, _I]),
    "c2g_set_trace_block": (_I, [_P, _I]),
    "c2g_probe_l2_read": (_I, [_I, C.c_size_t, _I, C.POINTER(C.c_double)]),
    "c2g_trace_rays": (_I, [_P, _I, _FP, _FP, _FP, _FP, _IP, _I, _IP, _FP]),
    "c2g_trace_rays_dev": (_I, [_P, _I, _P, _P, _P, _P, _P, _I, _P, _P, _P]),
    "c2g_halton": (_I, [_P, _I, _I, _I, _IP, _IP, _IP, _I, _FP]),
    "c2g_camera_rays": (_I, [_P, _I, _FP, _FP, _FP]),
    "c2g_sampler_values": (_I, [_P, _I, _IP, _IP, _IP, _I, _I, _FP]),
    "c2g_guide_reset": (_I, [_P, _FP, _FP, C.c_uint64]),
    "c2g_guide_set_params": (_I, [_P, _FP]),
    "c2g_guide_get_params": (_I, [_P, _FP]),
    "c2g_guide_eval": (_I, [_P, _I, _FP, _FP]),
    "c2g_guide_gradient": (_I, [_P, _I, _FP, _FP, C.POINTER(C.c_double)]),
    "c2g_guide_stats": (_I, [_P, C.POINTER(C.c_double), _IP, _IP]),
    "c2g_guide_config": (_I, [_P, C.c_float, C.c_float, _I, _I]),
    "c2g_guide_levels": (_I, [_P, _I]),
    "c2g_guide_batch": (_I, [_P, _I, _I]),
    "c2g_guide_regularize": (_I, [_P, C.c_float, C.c_float, C.c_float]),
    "c2g_batch_create": (_I, [C.POINTER(_P), _I]),
    "c2g_batch_destroy": (None, [_P]),
    "c2g_batch_last_error": (C.c_char_p, [_P]),
    "c2g_batch_add": (_I, [_P, _P, C.POINTER(RenderParams), _IP]),
    "c2g_batch_tune": (_I, [_P, _I, _I]),
    "c2g_batch_autotune": (_I, [_P, _IP, _I, _IP, _I, _I, C.POINTER(C.c_double)]),
    "c2g_batch_set_trace": (_I, [_P, _I, _I]),
    "c2g_batch_set_lanes": (_I, [_P, _I]),
    "c2g_batch_search": (_I, [_P, C.POINTER(BatchSpace), _I, C.POINTER(C.c_double)]),
    "c2g_batch_run": (_I, [_P, C.POINTER(BatchStats)]),
    "c2g_batch_job_latency": (_I, [_P, _I, C.POINTER(C.c_double)]),
}

GUIDE_PARAMS = 16624
GUIDE_OUTPUTS = 41

_lib = None


def load_library(path: str = LIB_PATH) -> C.CDLL:
    """Load ``libc2g.so`` (raises FileNotFoundError when it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FileNotFoundError(f"{path} is missing: build it with `python crystal2_gb300/build.py`")
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def fptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_FP)


def iptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_IP)
