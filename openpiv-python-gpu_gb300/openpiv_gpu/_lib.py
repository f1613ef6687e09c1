"""ctypes binding of libpiv_gb300.so (the C ABI declared in include/piv_gb300.h).

The library is built in-tree by ``openpiv_gpu._build.build()``. Loading fails
loudly when it is missing: there is no CPU fallback.
"""

import ctypes
import math
import os
import re
import threading
from ctypes import POINTER, c_double, c_int, c_size_t, c_void_p

from . import _build

PIV_OK = 0
PIV_E_ARG = 1
PIV_E_OOM = 2
PIV_E_CUDA = 3
PIV_E_TIMEOUT = 4
PIV_E_UNSUPPORTED = 6

PIXEL = {"u8": 0, "u16": 1, "f32": 2, "f64": 3}
DTYPE = {"float32": 0, "float64": 1}
SUBPIXEL = {"gaussian": 0, "parabolic": 1, "centroid": 2}
S2N = {"peak2peak": 0, "peak2mean": 1, "peak2energy": 2}
REPLACE = {"spring": 0, "median": 1, "mean": 2}
DFT = {"fft": 0, "tensor": 1, "tensor_split": 2, "tensor_refined": 3}
STAGES = ("predictor", "deform", "correlate", "validate", "replace", "smooth")
SMOOTH_S_LOWER, SMOOTH_S_UPPER, SMOOTH_MAX_ITERS = 1, 2, 4

HEADER = os.path.join(os.path.dirname(_build.ROOT), "include", "piv_gb300.h")


class PivIteration(ctypes.Structure):
    _fields_ = [
        ("search_size", c_int), ("window_size", c_int), ("overlap_ratio", c_double), ("fft_size", c_int),
        ("deforming_order", c_int), ("deforming_par", c_double), ("normalize", c_int), ("subpixel_method", c_int),
        ("s2n_method", c_int), ("s2n_size", c_int), ("validation_size", c_int),
        ("s2n_tol", c_double), ("median_tol", c_double), ("mad_tol", c_double), ("mean_tol", c_double),
        ("rms_tol", c_double), ("num_replacing_iters", c_int), ("replacing_method", c_int),
        ("replacing_size", c_int), ("revalidate", c_int), ("smoothing_par", c_double),
    ]


class PivConfig(ctypes.Structure):
    _fields_ = [
        ("height", c_int), ("width", c_int), ("n_iters", c_int), ("iters", POINTER(PivIteration)),
        ("center", c_int), ("dt", c_double), ("scaling_par", c_double), ("dtype", c_int), ("pixel_type", c_int),
        ("max_pairs", c_int), ("mask", c_void_p), ("dft_mode", c_int),
    ]


class PivGeometry(ctypes.Structure):
    _fields_ = [(name, c_int) for name in ("height", "width", "search_size", "window_size", "spacing", "m", "n",
                                           "x_offset", "y_offset")]


class PivIterationView(ctypes.Structure):
    _fields_ = [("m", c_int), ("n", c_int)] + [(name, c_void_p) for name in (
        "u_corr", "v_corr", "up", "vp", "u_rep", "v_rep", "u_out", "v_out", "val0", "smooth_p", "peak_i",
        "peak_j", "s2n", "near_tie", "smooth_flags")]


_SIGNATURES = {
    "piv_plan_create": (c_int, [POINTER(PivConfig), POINTER(c_void_p)]),
    "piv_plan_field_shape": (c_int, [c_void_p, c_int, POINTER(c_int), POINTER(c_int)]),
    "piv_plan_workspace_bytes": (c_int, [c_void_p, POINTER(c_size_t)]),
    "piv_plan_run": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                             c_int, c_void_p]),
    "piv_plan_iteration_view": (c_int, [c_void_p, c_int, POINTER(PivIterationView)]),
    "piv_plan_destroy": (None, [c_void_p]),
    "piv_plan_status": (c_int, [c_void_p, POINTER(c_int), c_void_p]),
    "piv_plan_near_ties": (c_int, [c_void_p, POINTER(c_int), c_int, c_void_p]),
    "piv_plan_autotune": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_int, c_int, c_void_p]),
    "piv_plan_tuning": (c_int, [c_void_p, c_int, POINTER(c_int), POINTER(c_int), POINTER(ctypes.c_float), c_int]),
    "piv_plan_variant_name": (c_int, [c_void_p, c_int, c_int, ctypes.c_char_p, c_size_t]),
    "piv_plan_set_variant": (c_int, [c_void_p, c_int, c_int]),
    "piv_autotune_cache_clear": (None, []),
    "piv_selftest_bounded_wait": (c_int, [ctypes.c_uint, POINTER(c_int), c_void_p]),
    "piv_batch_create": (c_int, [POINTER(PivConfig), c_int, POINTER(c_void_p)]),
    "piv_batch_destroy": (None, [c_void_p]),
    "piv_batch_plan": (c_int, [c_void_p, c_int, POINTER(c_void_p)]),
    "piv_batch_run": (c_int, [c_void_p, POINTER(c_int), POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p),
                              POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p), c_void_p]),
    "piv_batch_graph_capture": (c_int, [c_void_p, POINTER(c_int), POINTER(c_void_p), POINTER(c_void_p),
                                        POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p), POINTER(c_void_p),
                                        POINTER(c_int), c_void_p]),
    "piv_batch_graph_launch": (c_int, [c_void_p, c_void_p]),
    "piv_batch_status": (c_int, [c_void_p, POINTER(c_int), c_void_p]),
    "piv_batch_set_schedule": (c_int, [c_void_p, c_int]),
    "piv_plan_graph_capture": (c_int, [c_void_p, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                       c_void_p, POINTER(c_int), c_void_p]),
    "piv_plan_graph_launch": (c_int, [c_void_p, c_void_p]),
    "piv_plan_set_timing": (c_int, [c_void_p, c_int]),
    "piv_plan_stage_times": (c_int, [c_void_p, POINTER(ctypes.c_float), c_int, POINTER(c_int)]),
    "piv_last_error": (c_int, [ctypes.c_char_p, c_size_t]),
    "piv_bounds_check": (c_int, [POINTER(c_int), POINTER(c_int)]),
    "piv_memcpy": (c_int, [c_void_p, c_void_p, c_size_t, c_int, c_void_p]),
    "piv_field_geometry": (c_int, [c_int, c_int, c_int, c_int, c_double, c_int, POINTER(PivGeometry)]),
    "piv_correlate": (c_int, [POINTER(PivGeometry), c_int, c_void_p, c_void_p, c_int, c_int, c_int, c_int, c_int,
                              c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_void_p, c_int,
                              c_void_p]),
    "piv_correlate_maps": (c_int, [POINTER(PivGeometry), c_int, c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                                   c_void_p, c_void_p, c_int, c_void_p]),
    "piv_regrid": (c_int, [POINTER(PivGeometry), POINTER(PivGeometry), c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                           c_void_p]),
    "piv_deform": (c_int, [POINTER(PivGeometry), c_int, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_double,
                           c_int, c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_void_p]),
    "piv_spline_prefilter": (c_int, [c_int, c_int, c_int, c_void_p, c_int, c_void_p, c_void_p]),
    "piv_validate": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_int, c_int, c_double, c_double,
                             c_double, c_double, c_double, c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    "piv_replace": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_void_p, c_int, c_int, c_int, c_int,
                            c_void_p, c_int, c_int, c_double, c_double, c_double, c_double, c_double, c_int, c_int,
                            c_void_p]),
    "piv_smoothn": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p]),
    "piv_smoothn_flags": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double, c_void_p, c_void_p,
                                  c_void_p]),
    "piv_smoothn_noalloc": (c_int, [c_int, c_int, c_int, c_void_p, c_void_p, c_void_p, c_double, c_void_p,
                                    c_void_p]),
}

_lock = threading.Lock()
_lib = None


class PIVError(RuntimeError):
    def __init__(self, code, message):
        super().__init__(f"[{code}] {message}")
        self.code = code


def header_functions():
    """Names of the functions declared in include/piv_gb300.h."""
    with open(HEADER) as fh:
        text = fh.read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|void)\s+\**\s*(piv_\w+)\s*\(", text, flags=re.M)))


def load(path=None):
    """Loads (without building) the shared library and declares its signatures."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = path or _build.LIB_PATH
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with openpiv_gpu._build.build() "
                               "(the GPU path has no fallback)")
        lib = ctypes.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
        return lib


def lib():
    return _lib if _lib is not None else load()


def load_checked():
    """Loads the checked build (``_build.build(checked=True)``) as a separate
    library with the same signatures; it shares no state with ``lib()``."""
    path = _build.CHECKED_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with openpiv_gpu._build.build(checked=True)")
    checked = ctypes.CDLL(path)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(checked, name)
        fn.restype = res
        fn.argtypes = args
    return checked


def last_error():
    buf = ctypes.create_string_buffer(512)
    lib().piv_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc):
    if rc != PIV_OK:
        raise PIVError(rc, last_error())
    return rc


def opt(value):
    """None -> NaN for optional tolerances / smoothing parameters."""
    return math.nan if value is None else float(value)
