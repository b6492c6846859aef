"""ctypes binding of libskewengine.so (the C ABI declared in include/skewengine.h).

The library is built in-tree by ``python -m skewengine_gb300.build``.  Loading
fails loudly when it is missing: there is no pure-Python or CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libskewengine.so")

SKE_OK = 0
STATUS_NAMES = {0: "OK", 1: "INVALID", 2: "CUDA", 3: "NO_DEVICE", 4: "STATE", 5: "UNSUPPORTED", 6: "DEVICE"}


class SkeError(RuntimeError):
    """A C ABI call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class Params(C.Structure):
    _fields_ = [("max_sector", C.c_int32), ("povh", C.c_float), ("accum", C.c_int32), ("flags", C.c_int32)]


class SectorGeometry(C.Structure):
    _fields_ = [("angle", C.c_int32), ("sector_type", C.c_int32), ("new_angle", C.c_int32),
                ("dim_i", C.c_int32), ("dim_o", C.c_int32), ("offset", C.c_int32),
                ("skew_height", C.c_int32), ("dim_l", C.c_int32), ("scale", C.c_double),
                ("skewness", C.c_double)]


class SectorView(C.Structure):
    _fields_ = [("geom", SectorGeometry), ("skew_out", C.c_void_p), ("skew_in", C.c_void_p),
                ("first", C.c_void_p), ("last", C.c_void_p), ("target", C.c_void_p),
                ("weight", C.c_void_p), ("povh", C.c_float), ("stream", C.c_void_p)]


OPERATOR_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(SectorView))

# (name, restype, argtypes) of every exported symbol.
SIGNATURES = [
    ("ske_abi_version", C.c_int, []),
    ("ske_last_error", C.c_char_p, []),
    ("ske_params_default", C.c_int, [C.POINTER(Params)]),
    ("ske_device_count", C.c_int, [C.POINTER(C.c_int)]),
    ("ske_geometry", C.c_int, [C.c_int, C.c_int, C.c_int, C.POINTER(SectorGeometry), C.c_void_p, C.c_void_p,
                               C.c_void_p, C.c_void_p]),
    ("ske_create", C.c_int, [C.POINTER(C.c_void_p), C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("ske_destroy", C.c_int, [C.c_void_p]),
    ("ske_stream", C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    ("ske_run", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(Params)]),
    ("ske_run_angles", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p,
                                 C.c_int, C.POINTER(Params)]),
    ("ske_accumulate", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                 C.POINTER(Params), C.c_void_p, C.c_int, C.POINTER(C.c_uint32)]),
    ("ske_run_batch", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                C.c_void_p, C.c_int, C.POINTER(Params)]),
    ("ske_run_batch_angles", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                       C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.POINTER(Params)]),
    ("ske_radon_select", C.c_int, [C.c_int]),
    ("ske_skew_select", C.c_int, [C.c_int]),
    ("ske_sweep_shape", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("ske_set_sweep_shape", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int]),
    ("ske_prepare", C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    ("ske_skew", C.c_int, [C.c_void_p, C.c_int]),
    ("ske_kernel", C.c_int, [C.c_void_p, C.c_int, C.c_float]),
    ("ske_kernel_custom", C.c_int, [C.c_void_p, OPERATOR_FN, C.c_void_p, C.c_float]),
    ("ske_deskew", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("ske_reduce", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int]),
    ("ske_sector", C.c_int, [C.c_void_p, C.POINTER(SectorView)]),
    ("ske_copy_skewed", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]),
    ("ske_sdem_counts", C.c_int, [C.c_void_p, C.c_int, C.c_float, C.c_void_p, C.c_int]),
    ("ske_sdem_sector_noalloc", C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p,
                                          C.c_void_p, C.c_float, C.c_float, C.c_void_p]),
    ("ske_profile_enable", C.c_int, [C.c_void_p, C.c_int]),
    ("ske_profile_get", C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_double), C.POINTER(C.c_int64)]),
    ("ske_launch_count", C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    ("ske_selftest_division", C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                        C.POINTER(C.c_uint32)]),
    ("ske_measure_fp32_peak", C.c_int, [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    ("ske_measure_fp64_peak", C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    ("ske_inject_alloc_failure", C.c_int, [C.c_int64]),
    ("ske_accumulate_resume", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_int,
                                        C.POINTER(Params), C.c_void_p, C.c_void_p, C.c_int,
                                        C.POINTER(C.c_uint32)]),
    ("ske_fold", C.c_int, [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_uint32, C.c_int, C.c_void_p,
                           C.c_int]),
    ("ske_conv3x3_bf16", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("ske_conv3x3_upcat_bf16", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                         C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("ske_conv3x3_wgrad_bf16", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                         C.c_int, C.c_void_p]),
    ("ske_conv_select", C.c_int, [C.c_int]),
    ("ske_conv_stage_channels", C.c_int, [C.c_int]),
    ("ske_conv_wgrad_select", C.c_int, [C.c_int]),
    ("ske_conv3x3_head_bf16", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("ske_maxpool2_bf16", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p]),
    ("ske_surrogate_encode_bf16", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_float,
                                            C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    ("ske_conv_status", C.c_int, [C.POINTER(C.c_int), C.c_void_p]),
    ("ske_read_grid", C.c_int, [C.c_char_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_size_t,
                                C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("ske_png_size", C.c_int, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("ske_png_read_rgba", C.c_int, [C.c_char_p, C.c_void_p, C.c_size_t]),
    ("ske_png_read_image", C.c_int, [C.c_char_p, C.c_void_p, C.c_size_t]),
    ("ske_png_write", C.c_int, [C.c_char_p, C.c_void_p, C.c_int, C.c_int, C.c_int]),
    ("ske_hsv_to_rgb", None, [C.c_float, C.c_float, C.c_float, C.c_void_p]),
    ("ske_render", C.c_int, [C.c_int, C.c_void_p, C.c_int, C.c_int, C.c_void_p]),
    ("ske_render_input", C.c_int, [C.c_void_p, C.c_int, C.c_void_p]),
    ("run", C.c_int, [C.c_int, C.POINTER(C.c_char_p)]),
]

_lib = None


def load(path: str | None = None) -> C.CDLL:
    """Load libskewengine.so once (``path``, else $SKE_LIBRARY, else the in-tree
    build); raises if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("SKE_LIBRARY") or LIB_PATH
    if not os.path.exists(path):
        raise ImportError(f"{path} is missing: build it with `python -m skewengine_gb300.build`")
    lib = C.CDLL(path)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != SKE_OK:
        raise SkeError(status, load().ske_last_error().decode(errors="replace"))
