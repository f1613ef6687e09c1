"""Multi-pass PIV on a GB300: the drop-in for openpiv_gpu.gpu_process.

``piv_gpu`` and ``PIVGPU`` keep the reference's constructor arguments, defaults,
argument checks and results (openpiv_gpu/gpu_process.py:41-867). The whole
multi-pass pipeline runs in libpiv_gb300.so: one plan per instance, one
launch sequence per call with no host synchronisation until results are read.
Device arrays are torch CUDA tensors where the reference returns CuPy arrays.
"""

import ctypes
import logging
import math
from math import ceil, log2, prod

import numpy as np

from . import DTYPE_f, DTYPE_i
from . import _lib
from . import gpu_smoothn
from .gpu_smoothn import SMOOTHING_PAR
from .gpu_validation import (ALLOWED_REPLACING_METHODS, MAD_TOL, MEAN_TOL, MEDIAN_TOL, REPLACING_METHOD,
                             REPLACING_SIZE, RMS_TOL, S2N_TOL, VALIDATION_SIZE)

# Default settings (gpu_process.py:19-35).
SEARCH_SIZE_ITERS = 1
OVERLAP_RATIO = 0.5
SHRINK_RATIO = 1
CENTER = True
DEFORMING_ORDER = 1
NORMALIZE = True
SUBPIXEL_METHOD = "gaussian"
N_FFT = 2
DEFORMING_PAR = 0.5
BATCH_SIZE = "full"
S2N_METHOD = "peak2peak"
S2N_SIZE = 2
NUM_REPLACING_ITERS = 1
REVALIDATE = False
SMOOTH = True
BLOCK_SIZE = 8

# Allowed settings (gpu_process.py:38-39).
ALLOWED_SUBPIXEL_METHODS = {"gaussian", "parabolic", "centroid"}
ALLOWED_S2N_METHODS = {"peak2peak", "peak2mean", "peak2energy"}

# Names accepted as aliases of the reference's arguments.
_ALIASES = {"window_size_iters": "search_size_iters", "min_window_size": "min_search_size"}


def _torch():
    import torch

    return torch


def _apply_aliases(kwargs):
    for alias, name in _ALIASES.items():
        if alias in kwargs:
            value = kwargs.pop(alias)
            if name != "min_search_size":
                kwargs.setdefault(name, value)
            else:
                kwargs["_min_search_size"] = value
    return kwargs


def _is_real(x):
    return isinstance(x, int) or isinstance(x, float)


class piv_gpu:
    """Wrapper of PIVGPU with the reference's input checks and host results
    (gpu_process.py:41-352).

    Parameters
    ----------
    frame_shape : tuple
        Shape of the images in pixels.
    min_search_size : int
        Width of the square search window in pixels (multiple of 8, power of 2).
    **kwargs
        PIV settings, see PIVGPU. ``window_size_iters`` and ``min_window_size``
        are accepted as aliases of ``search_size_iters`` and ``min_search_size``.
    """

    def __init__(self, frame_shape, min_search_size=None, **kwargs):
        kwargs = _apply_aliases(dict(kwargs))
        if min_search_size is None:
            min_search_size = kwargs.pop("_min_search_size", None)
        kwargs.pop("_min_search_size", None)
        g = lambda name, default: kwargs[name] if name in kwargs else default
        search_size_iters = g("search_size_iters", SEARCH_SIZE_ITERS)
        overlap_ratio = g("overlap_ratio", OVERLAP_RATIO)
        shrink_ratio = g("shrink_ratio", SHRINK_RATIO)
        center = g("center", CENTER)
        normalize = g("normalize", NORMALIZE)
        subpixel_method = g("subpixel_method", SUBPIXEL_METHOD)
        n_fft = g("n_fft", N_FFT)
        deforming_par = g("deforming_par", DEFORMING_PAR)
        batch_size = g("batch_size", BATCH_SIZE)
        s2n_method = g("s2n_method", S2N_METHOD)
        s2n_size = g("s2n_size", S2N_SIZE)
        validation_size = g("validation_size", VALIDATION_SIZE)
        s2n_tol = g("s2n_tol", S2N_TOL)
        median_tol = g("median_tol", MEDIAN_TOL)
        mad_tol = g("mad_tol", MAD_TOL)
        mean_tol = g("mean_tol", MEAN_TOL)
        rms_tol = g("rms_tol", RMS_TOL)
        num_replacing_iters = g("num_replacing_iters", NUM_REPLACING_ITERS)
        replacing_method = g("replacing_method", REPLACING_METHOD)
        replacing_size = g("replacing_size", REPLACING_SIZE)
        revalidate = g("revalidate", REVALIDATE)
        smooth = g("smooth", SMOOTH)
        smoothing_par = g("smoothing_par", SMOOTHING_PAR)
        dt = g("dt", 1)
        scaling_par = g("scaling_par", 1)
        mask = g("mask", None)
        dtype_f = g("dtype_f", "float32")

        # Geometry settings (gpu_process.py:96-133).
        self.min_search_size = min_search_size
        assert isinstance(self.min_search_size, int) and self.min_search_size >= 8, \
            "{} must be an {} number greater than 8.".format("min_search_size", "int")
        self.search_size_iters = (search_size_iters,) if isinstance(search_size_iters, int) else search_size_iters
        assert isinstance(self.search_size_iters, tuple) and len(self.search_size_iters) > 0 and \
            all(isinstance(item, int) for item in self.search_size_iters) and \
            all(item > 0 for item in self.search_size_iters), \
            "{} must be a tuple of positive {} numbers.".format("search_size_iters", "int")
        self.num_passes = len(self.search_size_iters)
        self.max_search_size = 2 ** (self.num_passes - 1) * self.min_search_size
        self.frame_shape = frame_shape
        assert isinstance(self.frame_shape, tuple) and len(self.frame_shape) == 2 and \
            all(isinstance(item, int) for item in self.frame_shape) and \
            all(item >= self.max_search_size for item in self.frame_shape), \
            "{} must be a tuple of {} values greater than {} of {}.".format(
                "frame_shape", "int", "max_search_size", self.max_search_size)
        n = self.num_passes
        self.overlap_ratio = (overlap_ratio,) * n if overlap_ratio == 0 or isinstance(overlap_ratio, float) \
            else overlap_ratio
        assert isinstance(self.overlap_ratio, tuple) and len(self.overlap_ratio) >= n and \
            all(item == 0 or isinstance(item, float) for item in self.overlap_ratio) and \
            all(0 <= item < 1 for item in self.overlap_ratio), \
            "{} must be a tuple of {} values between 0 and 1, defined for all passes.".format("overlap_ratio", "real")
        self.shrink_ratio = shrink_ratio
        assert shrink_ratio == 1 or isinstance(self.shrink_ratio, float) and 0 < self.shrink_ratio <= 1, \
            "{} must be a {} number between 0 and 1.".format("shrink_ratio", "real")
        self.center = center
        assert isinstance(self.center, bool), "{} must have a {} value.".format("center", "bool")

        # Correlation settings (gpu_process.py:135-166).
        self.normalize = self._tuple(normalize, bool)
        assert isinstance(self.normalize, tuple) and len(self.normalize) >= n and \
            all(isinstance(item, bool) for item in self.normalize), \
            "{} must be a tuple of {} values, defined for all passes.".format("normalize", "bool")
        self.subpixel_method = self._tuple(subpixel_method, str)
        assert isinstance(self.subpixel_method, tuple) and len(self.subpixel_method) >= n and \
            all(item in ALLOWED_SUBPIXEL_METHODS for item in self.subpixel_method), \
            "{} for every pass must be one of {}.".format("subpixel_method", ALLOWED_SUBPIXEL_METHODS)
        self.n_fft = self._tuple(n_fft, int)
        assert isinstance(self.n_fft, tuple) and len(self.n_fft) >= n and \
            all(_is_real(item) for item in self.n_fft) and all(item >= 1 for item in self.n_fft), \
            "{} must be a tuple of {} numbers greater than 1, defined for all passes.".format("n_fft", "real")
        self.deforming_par = (deforming_par,) * n if deforming_par == 0 or deforming_par == 1 or \
            isinstance(deforming_par, float) else deforming_par
        assert isinstance(self.deforming_par, tuple) and len(self.deforming_par) >= n and \
            all(item == 0 or item == 1 or isinstance(item, float) for item in self.deforming_par) and \
            all(0 <= item <= 1 for item in self.deforming_par), \
            "{} must be a tuple of {} values between 0 and 1, defined for all passes.".format("deforming_par", "real")
        self.batch_size = (batch_size,) * n if isinstance(batch_size, int) or batch_size == "full" else batch_size
        assert isinstance(self.batch_size, tuple) and len(self.batch_size) >= n and \
            all(isinstance(item, int) or item == "full" for item in self.batch_size), \
            "{} must be a tuple of positive {} numbers or 'full', defined for all passes.".format("batch_size", "int")

        # Validation settings (gpu_process.py:168-222).
        self.s2n_method = self._tuple(s2n_method, str)
        assert isinstance(self.s2n_method, tuple) and len(self.s2n_method) >= n and \
            all(item in ALLOWED_S2N_METHODS for item in self.s2n_method), \
            "{} for every pass must be one of {}.".format("s2n_method", ALLOWED_S2N_METHODS)
        for name, value in (("s2n_size", s2n_size), ("validation_size", validation_size)):
            t = self._tuple(value, int)
            assert isinstance(t, tuple) and len(t) >= n and all(isinstance(item, int) for item in t) and \
                all(item > 0 for item in t), \
                "{} must be a tuple of positive {} numbers, defined for all passes.".format(name, "int")
            setattr(self, name, t)
        for name, value in (("s2n_tol", s2n_tol), ("median_tol", median_tol), ("mad_tol", mad_tol),
                            ("mean_tol", mean_tol), ("rms_tol", rms_tol)):
            t = (value,) * n if value is None or _is_real(value) else value
            assert isinstance(t, tuple) and len(t) >= n and all(item is None or _is_real(item) for item in t), \
                "{} must be a tuple of {} or None values, defined for all passes.".format(name, "real")
            setattr(self, name, t)

        # Replacement settings (gpu_process.py:224-250).
        self.num_replacing_iters = self._tuple(num_replacing_iters, int)
        assert isinstance(self.num_replacing_iters, tuple) and len(self.num_replacing_iters) >= n and \
            all(isinstance(item, int) for item in self.num_replacing_iters) and \
            all(item >= 0 for item in self.num_replacing_iters), \
            "{} must be a tuple of positive {} numbers, defined for all passes.".format("num_replacing_iters", "int")
        self.replacing_method = self._tuple(replacing_method, str)
        assert isinstance(self.replacing_method, tuple) and len(self.replacing_method) >= n and \
            all(item in ALLOWED_REPLACING_METHODS for item in self.replacing_method), \
            "{} for every pass must be one of {}.".format("replacing_method", ALLOWED_REPLACING_METHODS)
        self.replacing_size = self._tuple(replacing_size, int)
        assert isinstance(self.replacing_size, tuple) and len(self.replacing_size) >= n and \
            all(isinstance(item, int) for item in self.replacing_size) and \
            all(item > 0 for item in self.replacing_size), \
            "{} must be a tuple of positive {} values, defined for all passes.".format("replacing_size", "int")
        self.revalidate = self._tuple(revalidate, bool)
        assert isinstance(self.revalidate, tuple) and len(self.revalidate) >= n and \
            all(isinstance(item, bool) for item in self.revalidate), \
            "{} must be a tuple of {} values, defined for all passes.".format("revalidate", "bool")

        # Smoothing settings (gpu_process.py:252-266).
        self.smooth = self._tuple(smooth, bool)
        assert isinstance(self.smooth, tuple) and len(self.smooth) >= n and \
            all(isinstance(item, bool) for item in self.smooth), \
            "{} must be a tuple of {} values, defined for all passes.".format("smooth", "bool")
        self.smoothing_par = (smoothing_par,) * n if smoothing_par is None or _is_real(smoothing_par) \
            else smoothing_par
        assert isinstance(self.smoothing_par, tuple) and len(self.smoothing_par) >= n and \
            all(item is None or _is_real(item) for item in self.smoothing_par) and \
            all(item > 0 if item is not None else True for item in self.smoothing_par), \
            "{} must be a tuple of positive {} or None values, defined for all passes.".format("smoothing_par", "real")

        # Scaling and masking settings (gpu_process.py:268-286).
        self.dt = dt
        assert isinstance(self.dt, int) or isinstance(self.dt, float) and self.dt > 0, \
            "{} must be a {} number greater than 0.".format("dt", "real")
        self.scaling_par = scaling_par
        assert isinstance(self.scaling_par, int) or isinstance(self.scaling_par, float) and self.scaling_par > 0, \
            "{} must be a {} number greater than 0.".format("scaling_par", "real")
        self.mask = mask
        assert self.mask is None or (isinstance(self.mask, np.ndarray) and self.mask.shape == self.frame_shape and
                                     (np.issubdtype(self.mask.dtype, np.number) or mask.dtype == bool)), \
            "{} must be an ndarray of {} values with shape {}.".format("mask", "real", self.frame_shape)
        self.mask = mask.astype(bool) if mask is not None else None
        self.frame_mask = self.mask if self.mask is not None else np.full(self.frame_shape, False, dtype=bool)
        self.dtype_f = DTYPE_f if dtype_f == "float64" else np.float32

        self.gpu_process = PIVGPU(frame_shape, min_search_size, **kwargs)

    def _tuple(self, value, kind):
        return (value,) * self.num_passes if isinstance(value, kind) else value

    def __call__(self, frame_a, frame_b):
        """Computes the velocity field of an image pair; returns host arrays (u, v)."""
        frames = [frame_a, frame_b]
        assert all(isinstance(frame, np.ndarray) for frame in frames) and \
            all(frame.shape == self.frame_shape for frame in frames) and \
            all(np.issubdtype(frame.dtype, np.number) for frame in frames) and \
            all(not np.iscomplex(frame).any() for frame in frames), \
            "Both frames must be an ndarray of {} values with shape {}.".format("real", self.frame_shape)
        u, v = self.gpu_process(frame_a, frame_b)
        return u.cpu().numpy(), v.cpu().numpy()

    @property
    def field_shape(self):
        return self.gpu_process.piv_fields[-1].field_shape

    @property
    def coords(self):
        x, y = self.gpu_process.coords
        return x.cpu().numpy(), y.cpu().numpy()

    @property
    def field_mask(self):
        if self.mask is not None:
            return self.gpu_process.field_mask.cpu().numpy()
        x, y = self.coords
        return self.frame_mask[y.astype(int), x.astype(int)]

    @property
    def val_locations(self):
        if self.gpu_process.init_val_locations is not None:
            return self.gpu_process.init_val_locations.cpu().numpy()
        return np.full(self.gpu_process.piv_fields[-1].field_shape, False, dtype=bool)

    @property
    def outliers(self):
        if self.gpu_process.val_locations is not None:
            return self.gpu_process.val_locations.cpu().numpy()
        return np.full(self.gpu_process.piv_fields[-1].field_shape, False, dtype=bool)


def _per_pass(value, n, kind):
    if value is None or isinstance(value, kind):
        return (value,) * n
    return tuple(value)


def _pixel_type(arr):
    dt = np.dtype(arr.dtype) if isinstance(arr, np.ndarray) else None
    if dt is None:
        torch = _torch()
        dt = {torch.uint8: np.dtype(np.uint8), torch.int16: np.dtype(np.int16), torch.float32: np.dtype(np.float32),
              torch.float64: np.dtype(np.float64)}.get(arr.dtype, np.dtype(np.float64))
    if dt == np.uint8:
        return _lib.PIXEL["u8"]
    if dt == np.uint16:
        return _lib.PIXEL["u16"]
    return None


class PIVGPU:
    """Iterative multigrid PIV (gpu_process.py:354-867) on the GB300 kernels.

    Same constructor arguments and defaults as the reference (dtype_f defaults
    to float64 there and here). ``deforming_order`` 3 selects cubic B-spline
    deformation; any other order is the reference's bilinear deformation.
    ``batch_size`` is accepted and has no effect (every window of a pass runs
    in one launch). ``dft`` selects the correlation engine: "fft" (plain
    float FFT), "tensor" (tcgen05 DFT on fp16 operands where available) or
    "tensor_split" (tcgen05 DFT on fp16 hi/lo operand pairs, three products
    per stage, for 16 and 32 px passes; the FFT elsewhere) or
    "tensor_refined" (the "tensor" maps give each window's integer peak, and
    the five values of the subpixel fit are recomputed in float32 by direct
    sums from the frames: the float32 FFT form's fit at nearly the fp16
    form's cost). With
    ``autotune=True`` the first run of each plan times every launch variant
    of each pass's correlation engine on that run's frames (radix split and
    tile shape of the FFT engine, CTAs per SM and staging of the tensor
    engines) and keeps the fastest; ``tuning()`` reports the choices.
    """

    def __init__(self, frame_shape, min_search_size, search_size_iters=SEARCH_SIZE_ITERS,
                 overlap_ratio=OVERLAP_RATIO, shrink_ratio=SHRINK_RATIO, center=CENTER,
                 deforming_order=DEFORMING_ORDER, normalize=NORMALIZE, subpixel_method=SUBPIXEL_METHOD, n_fft=N_FFT,
                 deforming_par=DEFORMING_PAR, batch_size=BATCH_SIZE, s2n_method=S2N_METHOD, s2n_size=S2N_SIZE,
                 validation_size=VALIDATION_SIZE, s2n_tol=S2N_TOL, median_tol=MEDIAN_TOL, mad_tol=MAD_TOL,
                 mean_tol=MEAN_TOL, rms_tol=RMS_TOL, num_replacing_iters=NUM_REPLACING_ITERS,
                 replacing_method=REPLACING_METHOD, replacing_size=REPLACING_SIZE, revalidate=REVALIDATE,
                 smooth=SMOOTH, smoothing_par=SMOOTHING_PAR, dt=1, scaling_par=1, mask=None, dtype_f=DTYPE_f,
                 dft="fft", autotune=False, **aliases):
        aliases = _apply_aliases(dict(aliases))
        if "search_size_iters" in aliases:
            search_size_iters = aliases.pop("search_size_iters")
        aliases.pop("_min_search_size", None)
        if aliases:
            raise TypeError(f"unexpected arguments: {sorted(aliases)}")
        self.min_search_size = min_search_size
        self.ss_iters = (search_size_iters,) if isinstance(search_size_iters, int) else tuple(search_size_iters)
        self.n_passes = len(self.ss_iters)
        self.frame_shape = tuple(frame_shape)
        n = self.n_passes
        self.overlap_ratio = (overlap_ratio,) * n if overlap_ratio == 0 or isinstance(overlap_ratio, float) \
            else overlap_ratio
        self.shrink_ratio = shrink_ratio
        self.center = center
        self.deforming_order = _per_pass(deforming_order, n, int)
        self.is_normalized = _per_pass(normalize, n, bool)
        self.subpixel_method = _per_pass(subpixel_method, n, str)
        self.n_fft = _per_pass(n_fft, n, (int, float))
        self.deforming_par = (deforming_par,) * n if deforming_par == 0 or deforming_par == 1 or \
            isinstance(deforming_par, float) else deforming_par
        self.batch_size = (batch_size,) * n if isinstance(batch_size, int) or batch_size == "full" else batch_size
        self.s2n_method = _per_pass(s2n_method, n, str)
        self.s2n_size = _per_pass(s2n_size, n, int)
        self.validation_size = _per_pass(validation_size, n, int)
        self.s2n_tol = _per_pass(s2n_tol, n, (int, float))
        self.median_tol = _per_pass(median_tol, n, (int, float))
        self.mad_tol = _per_pass(mad_tol, n, (int, float))
        self.mean_tol = _per_pass(mean_tol, n, (int, float))
        self.rms_tol = _per_pass(rms_tol, n, (int, float))
        self.num_replacing_iters = _per_pass(num_replacing_iters, n, int)
        self.replacing_method = _per_pass(replacing_method, n, str)
        self.replacing_size = _per_pass(replacing_size, n, int)
        self.is_revalidated = _per_pass(revalidate, n, bool)
        self.is_smoothed = _per_pass(smooth, n, bool)
        self.smoothing_par = _per_pass(smoothing_par, n, (int, float))
        self.dt = dt
        self.scaling_par = scaling_par
        self.mask = np.asarray(mask).astype(bool) if mask is not None else None
        self.dtype_f = np.float32 if dtype_f == "float32" else DTYPE_f
        if dft not in _lib.DFT:
            raise ValueError(f"dft must be one of {sorted(_lib.DFT)}, not {dft!r}")
        self.dft = dft
        self.init_val_locations = self.val_locations = None
        self.piv_fields = None
        self.init_piv_fields()
        self._iterations = self._build_iterations()
        self._plans = {}
        self._last = None
        self.autotune = bool(autotune)
        self._tuned = set()

    # -- geometry -------------------------------------------------------------
    def get_geom_settings(self):
        """Search size and overlap of every iteration (gpu_process.py:675-680)."""
        for i, n_it in enumerate(self.ss_iters):
            for _ in range(n_it):
                yield (2 ** (len(self.ss_iters) - i - 1)) * self.min_search_size, self.overlap_ratio[i]

    def init_piv_fields(self):
        """One PIVFieldGPU per iteration (gpu_process.py:649-673)."""
        self.piv_fields = []
        for k, (ss, ov) in enumerate(self.get_geom_settings()):
            ws = ss
            if k == 0 and self.shrink_ratio != 1:
                ws = int(ss * self.shrink_ratio)
                ws = ws if ws % 2 == 0 else ws + 1
                ws = max(ws, 8)
            self.piv_fields.append(PIVFieldGPU(self.frame_shape, ws, search_size=ss, overlap_ratio=ov,
                                               center=self.center, mask=self.mask, dtype_f=self.dtype_f))

    @property
    def max_iters(self):
        return sum(self.ss_iters)

    def _build_iterations(self):
        its = []
        k = 0
        for i, n_it in enumerate(self.ss_iters):
            for _ in range(n_it):
                f = self.piv_fields[k]
                n_fft = self.n_fft[i]
                it = _lib.PivIteration()
                it.search_size = f.search_size
                it.window_size = f.window_size
                it.overlap_ratio = float(self.overlap_ratio[i])
                it.fft_size = 2 ** ceil(log2(f.search_size * n_fft))
                it.deforming_order = int(self.deforming_order[i])
                it.deforming_par = float(self.deforming_par[i])
                it.normalize = int(bool(self.is_normalized[i]))
                it.subpixel_method = _lib.SUBPIXEL[self.subpixel_method[i]]
                it.s2n_method = _lib.S2N[self.s2n_method[i]]
                it.s2n_size = int(self.s2n_size[i])
                it.validation_size = int(self.validation_size[i])
                it.s2n_tol = _lib.opt(self.s2n_tol[i])
                it.median_tol = _lib.opt(self.median_tol[i])
                it.mad_tol = _lib.opt(self.mad_tol[i])
                it.mean_tol = _lib.opt(self.mean_tol[i])
                it.rms_tol = _lib.opt(self.rms_tol[i])
                it.num_replacing_iters = int(self.num_replacing_iters[i])
                it.replacing_method = _lib.REPLACE[self.replacing_method[i]]
                it.replacing_size = int(self.replacing_size[i])
                it.revalidate = int(bool(self.is_revalidated[i]))
                # Smoothing runs after every non-final iteration: the reference
                # tests the whole `is_smoothed` tuple (gpu_process.py:839-841).
                it.smoothing_par = _lib.opt(self.smoothing_par[i])
                its.append(it)
                k += 1
        return its

    # -- execution ------------------------------------------------------------
    def _config(self, pixel_type, n_pairs):
        """(piv_config, objects it points to) for this instance's settings."""
        arr = (_lib.PivIteration * len(self._iterations))(*self._iterations)
        cfg = _lib.PivConfig()
        cfg.height, cfg.width = self.frame_shape
        cfg.n_iters = len(self._iterations)
        cfg.iters = arr
        cfg.center = int(bool(self.center))
        cfg.dt = float(self.dt)
        cfg.scaling_par = float(self.scaling_par)
        cfg.dtype = _lib.DTYPE["float32" if self.dtype_f == np.float32 else "float64"]
        cfg.pixel_type = pixel_type
        cfg.max_pairs = int(n_pairs)
        mask_buf = None
        if self.mask is not None:
            mask_buf = np.ascontiguousarray(self.mask, dtype=np.uint8)
            cfg.mask = mask_buf.ctypes.data
        cfg.dft_mode = _lib.DFT[self.dft]
        return cfg, (arr, mask_buf)

    def _plan(self, pixel_type, n_pairs, slot=0):
        key = (pixel_type, slot)
        entry = self._plans.get(key)
        if entry is not None and entry[1] >= n_pairs:
            return entry[0]
        if entry is not None:
            _lib.lib().piv_plan_destroy(entry[0])
        cfg, _keep = self._config(pixel_type, n_pairs)
        plan = ctypes.c_void_p()
        _lib.check(_lib.lib().piv_plan_create(ctypes.byref(cfg), ctypes.byref(plan)))
        self._plans[key] = (plan, int(n_pairs))
        return plan

    def __del__(self):
        try:
            for plan, _ in self._plans.values():
                _lib.lib().piv_plan_destroy(plan)
        except Exception:
            pass

    def _frames(self, frames):
        """Returns (pointer-holder, pixel_type, on_host) for a frame batch."""
        torch = _torch()
        if isinstance(frames, torch.Tensor):
            if not frames.is_cuda:
                frames = frames.numpy()
            else:
                pt = _pixel_type(frames)
                if pt is None:
                    frames = frames.to(torch.float32 if self.dtype_f == np.float32 else torch.float64)
                    pt = _lib.PIXEL["f32" if self.dtype_f == np.float32 else "f64"]
                return frames.contiguous(), pt, 0
        frames = np.asarray(frames)
        pt = _pixel_type(frames)
        if pt is None:
            frames = frames.astype(self.dtype_f)
            pt = _lib.PIXEL["f32" if self.dtype_f == np.float32 else "f64"]
        return np.ascontiguousarray(frames), pt, 1

    def run_batch(self, frames_a, frames_b, host_out=False):
        """Processes a batch of equally sized pairs [B, H, W] in one plan run.

        Frames may be host arrays (pinned or pageable) or CUDA tensors. Returns
        (u, v) as torch CUDA tensors [B, m, n] in the reference's result dtype
        and keeps val_locations / outliers of the batch; with ``host_out`` the
        results are copied into pinned host memory before the call returns and
        come back as NumPy arrays.
        """
        torch = _torch()
        fa, pt_a, host_a = self._frames(frames_a)
        fb, pt_b, host_b = self._frames(frames_b)
        if pt_a != pt_b or host_a != host_b:
            target = self.dtype_f
            fa, pt_a, host_a = self._frames(np.asarray(frames_a, dtype=target))
            fb, pt_b, host_b = self._frames(np.asarray(frames_b, dtype=target))
        B = fa.shape[0]
        assert tuple(fa.shape[1:]) == self.frame_shape and tuple(fb.shape) == tuple(fa.shape)
        plan = self._plan(pt_a, B)
        m, n = self.piv_fields[-1].field_shape
        if host_out:
            key = (B, m, n)
            if getattr(self, "_host_out", (None,))[0] != key:
                self._host_out = (key,) + tuple(torch.empty((B, m, n), dtype=dt, pin_memory=True)
                                                for dt in (torch.float64, torch.float64, torch.uint8, torch.uint8))
            u, v, val, out = self._host_out[1:]
        else:
            dev = torch.device("cuda", torch.cuda.current_device())
            u = torch.empty((B, m, n), dtype=torch.float64, device=dev)
            v = torch.empty_like(u)
            val = torch.empty((B, m, n), dtype=torch.uint8, device=dev)
            out = torch.empty_like(val)
        pa = fa.ctypes.data if host_a else fa.data_ptr()
        pb = fb.ctypes.data if host_b else fb.data_ptr()
        stream = torch.cuda.current_stream().cuda_stream
        self._maybe_tune(plan, B, pa, pb, host_a, stream)
        _lib.check(_lib.lib().piv_plan_run(plan, B, pa, pb, host_a, u.data_ptr(), v.data_ptr(), val.data_ptr(),
                                           out.data_ptr(), int(bool(host_out)), stream))
        self._last = (plan, B, fa, fb)
        self.init_val_locations = val.bool()
        self.val_locations = out.bool()
        self._log_smoothing(plan, B)
        if host_out:
            u, v = u.numpy(), v.numpy()
            self.init_val_locations = self.init_val_locations.numpy()
            self.val_locations = self.val_locations.numpy()
            if self.max_iters == 1 and self.dtype_f == np.float32:
                u, v = u.astype(np.float32), v.astype(np.float32)
            return u, v
        if self.max_iters == 1 and self.dtype_f == np.float32:
            u, v = u.float(), v.float()
        return u, v

    def run_batches(self, batches):
        """Pipelined run over an iterable of (frames_a, frames_b) batches of
        host frames [B, H, W] (pinned memory gives the overlap): two plans on
        two streams, so that one batch's upload and download overlap the
        other's kernels. Yields (u, v) NumPy arrays per batch, in order; they
        are views of pinned buffers that stay valid until two more batches
        have been yielded (copy them to keep them longer).
        """
        torch = _torch()
        lib = _lib.lib()
        streams = [torch.cuda.Stream(), torch.cuda.Stream()]
        bufs = [None, None]
        pending = [None, None]
        m, n = self.piv_fields[-1].field_shape

        def finish(slot):
            B = pending[slot][0]  # the batch's frames stay referenced until its copies are done
            streams[slot].synchronize()
            pending[slot] = None
            u, v, val, out = (t[:B] for t in bufs[slot][1:])
            self.init_val_locations, self.val_locations = val.numpy().astype(bool), out.numpy().astype(bool)
            u, v = u.numpy(), v.numpy()
            if self.max_iters == 1 and self.dtype_f == np.float32:
                u, v = u.astype(np.float32), v.astype(np.float32)
            return u, v

        k = 0
        for frames_a, frames_b in batches:
            slot = k % 2
            if pending[slot] is not None:
                yield finish(slot)
            fa, pt_a, host_a = self._frames(frames_a)
            fb, pt_b, host_b = self._frames(frames_b)
            assert pt_a == pt_b and host_a == host_b, "both frames of a batch need the same type and location"
            B = fa.shape[0]
            assert tuple(fa.shape[1:]) == self.frame_shape and tuple(fb.shape) == tuple(fa.shape)
            plan = self._plan(pt_a, B, slot)
            if bufs[slot] is None or bufs[slot][0] < B:
                bufs[slot] = (B,) + tuple(torch.empty((B, m, n), dtype=dt, pin_memory=True)
                                          for dt in (torch.float64, torch.float64, torch.uint8, torch.uint8))
            u, v, val, out = bufs[slot][1:]
            pa = fa.ctypes.data if host_a else fa.data_ptr()
            pb = fb.ctypes.data if host_b else fb.data_ptr()
            self._maybe_tune(plan, B, pa, pb, host_a, streams[slot].cuda_stream)
            _lib.check(lib.piv_plan_run(plan, B, pa, pb, host_a, u.data_ptr(), v.data_ptr(), val.data_ptr(),
                                        out.data_ptr(), 2, streams[slot].cuda_stream))
            pending[slot] = (B, fa, fb)
            k += 1
        for j in range(k, k + 2):
            if pending[j % 2] is not None:
                yield finish(j % 2)

    def _maybe_tune(self, plan, n_pairs, pa, pb, on_host, stream):
        if self.autotune and plan.value not in self._tuned:
            _lib.check(_lib.lib().piv_plan_autotune(plan, n_pairs, pa, pb, on_host, 5, stream))
            self._tuned.add(plan.value)

    def tune(self, frames_a, frames_b, reps=5):
        """Autotunes the plan for batches like (frames_a, frames_b) [B, H, W]
        now (see ``autotune``); returns ``tuning()``."""
        torch = _torch()
        fa, pt, host = self._frames(frames_a)
        fb, _, _ = self._frames(frames_b)
        plan = self._plan(pt, fa.shape[0])
        pa = fa.ctypes.data if host else fa.data_ptr()
        pb = fb.ctypes.data if host else fb.data_ptr()
        _lib.check(_lib.lib().piv_plan_autotune(plan, fa.shape[0], pa, pb, host, int(reps),
                                                torch.cuda.current_stream().cuda_stream))
        self._tuned.add(plan.value)
        return self.tuning(plan)

    def tuning(self, plan=None):
        """Per pass of a plan (the last one run by default): the chosen
        correlation variant, its description, and the autotuner's time of every
        variant in ms (None where it was not timed)."""
        if plan is None:
            if self._last is None:
                return []
            plan = self._last[0]
        lib = _lib.lib()
        out = []
        for k in range(len(self._iterations)):
            var, nv = ctypes.c_int(0), ctypes.c_int(0)
            ms = (ctypes.c_float * 64)()
            _lib.check(lib.piv_plan_tuning(plan, k, ctypes.byref(var), ctypes.byref(nv), ms, 64))
            names = []
            for j in range(nv.value):
                buf = ctypes.create_string_buffer(128)
                _lib.check(lib.piv_plan_variant_name(plan, k, j, buf, 128))
                names.append(buf.value.decode())
            times = [None if ms[j] < 0 else float(ms[j]) for j in range(min(nv.value, 64))]
            out.append({"variant": var.value, "name": names[var.value] if names else None, "variants": names,
                        "ms": times})
        return out

    def status(self):
        """PIV_OK, or PIV_E_TIMEOUT when a bounded device-side wait of the
        cached plans gave up since the last call (see piv_plan_status)."""
        torch = _torch()
        worst = 0
        for plan, _ in self._plans.values():
            st = ctypes.c_int(0)
            _lib.check(_lib.lib().piv_plan_status(plan, ctypes.byref(st), torch.cuda.current_stream().cuda_stream))
            worst = worst or st.value
        return worst

    def _log_smoothing(self, plan, n_pairs):
        """SmoothnGPU's log messages for every smoothing of the run (the
        PIV_SMOOTH_* flags of each pair); read only when INFO is enabled."""
        if not gpu_smoothn._log.isEnabledFor(logging.INFO):
            return
        lib = _lib.lib()
        for k in range(len(self._iterations) - 1):
            view = _lib.PivIterationView()
            _lib.check(lib.piv_plan_iteration_view(plan, k, ctypes.byref(view)))
            flags = (ctypes.c_int * n_pairs)()
            _lib.check(lib.piv_memcpy(ctypes.addressof(flags), view.smooth_flags, 4 * n_pairs, 0, None))
            for f in flags:
                gpu_smoothn.log_flags(int(f), (view.m, view.n))

    def near_ties(self):
        """Near-tie windows of the last run per iteration (summed over its
        pairs): windows whose two largest correlation values are within the
        engine's map accuracy, so that their integer peak may differ from the
        reference's first argmax (see piv_plan_near_ties)."""
        if self._last is None:
            return []
        plan = self._last[0]
        n = len(self._iterations)
        counts = (ctypes.c_int * n)()
        _lib.check(_lib.lib().piv_plan_near_ties(plan, counts, n, _torch().cuda.current_stream().cuda_stream))
        return [int(c) for c in counts]

    def plan_handle(self, frames, n_pairs):
        """The C plan used for frames like ``frames`` and up to n_pairs pairs."""
        _, pt, _ = self._frames(frames)
        return self._plan(pt, n_pairs)

    def __call__(self, frame_a, frame_b):
        """Computes the velocity field from an image pair (gpu_process.py:564-647).

        Returns (u, v) as torch CUDA tensors.
        """
        if isinstance(frame_a, np.ndarray):
            fa, fb = frame_a[None], frame_b[None]
        else:
            fa, fb = frame_a.unsqueeze(0), frame_b.unsqueeze(0)
        u, v = self.run_batch(fa, fb)
        self.init_val_locations = self.init_val_locations[0]
        self.val_locations = self.val_locations[0]
        return u[0], v[0]

    def iteration_outputs(self, pair=0):
        """Per-iteration intermediates of the last run, as host NumPy arrays."""
        if self._last is None:
            return []
        plan, B, _, _ = self._last
        lib = _lib.lib()
        out = []
        ft = np.float32 if self.dtype_f == np.float32 else np.float64
        for k in range(len(self._iterations)):
            view = _lib.PivIterationView()
            _lib.check(lib.piv_plan_iteration_view(plan, k, ctypes.byref(view)))
            m, n = view.m, view.n
            mn = m * n

            def fetch(ptr, dtype, count=mn, offset=pair * mn):
                if not ptr:
                    return None
                arr = np.empty(count, dtype=dtype)
                _lib.check(lib.piv_memcpy(arr.ctypes.data, ptr + offset * np.dtype(dtype).itemsize, arr.nbytes, 0,
                                          None))
                return arr

            d = {
                "u_corr": fetch(view.u_corr, ft).reshape(m, n), "v_corr": fetch(view.v_corr, ft).reshape(m, n),
                "u_rep": fetch(view.u_rep, np.float64).reshape(m, n),
                "v_rep": fetch(view.v_rep, np.float64).reshape(m, n),
                "u_out": fetch(view.u_out, np.float64).reshape(m, n),
                "v_out": fetch(view.v_out, np.float64).reshape(m, n),
                "val0": fetch(view.val0, np.uint8).reshape(m, n).astype(bool),
                "i_peak": fetch(view.peak_i, np.int32), "j_peak": fetch(view.peak_j, np.int32),
                "p": float(fetch(view.smooth_p, np.float64, 1, pair)[0]),
            }
            if view.up:
                d["up"] = fetch(view.up, np.float64).reshape(m, n)
                d["vp"] = fetch(view.vp, np.float64).reshape(m, n)
            if view.s2n:
                d["s2n"] = fetch(view.s2n, ft).reshape(m, n)
            if view.near_tie:
                d["near_tie"] = fetch(view.near_tie, np.uint8).reshape(m, n).astype(bool)
            out.append(d)
        return out

    @property
    def coords(self):
        torch = _torch()
        x, y = self.piv_fields[-1].coords
        return torch.as_tensor(x * self.scaling_par).cuda(), torch.as_tensor(y * self.scaling_par).cuda()

    @property
    def field_mask(self):
        fm = self.piv_fields[-1].field_mask
        return None if fm is None else _torch().as_tensor(fm).cuda()


class PIVFieldGPU:
    """Geometry of a PIV field (gpu_process.py:869-961); host arrays."""

    def __init__(self, frame_shape, window_size, search_size=None, overlap_ratio=OVERLAP_RATIO, center=CENTER,
                 mask=None, dtype_f=DTYPE_f):
        self.frame_shape = tuple(frame_shape)
        self.window_size = window_size
        self.search_size = search_size if search_size is not None else window_size
        geom = _geometry(self.frame_shape, self.window_size, self.search_size, overlap_ratio, center)
        self.geometry = geom
        self.overlap = int(overlap_ratio * self.search_size)
        self.pad_ht = self.pad_wd = (self.search_size - self.window_size) // 2
        self.pad_shape = (self.pad_ht, self.pad_wd)
        self.spacing = geom.spacing
        self.field_shape = (geom.m, geom.n)
        self.n_wins = prod(self.field_shape)
        self.dtype_f = dtype_f
        self.center = center
        self.offset = (geom.x_offset, geom.y_offset)
        xg = np.arange(geom.n) * self.spacing + self.search_size / 2.0 + geom.x_offset
        yg = np.arange(geom.m) * self.spacing + self.search_size / 2.0 + geom.y_offset
        x, y = np.meshgrid(xg, yg)
        self.x, self.y = x.astype(dtype_f), y.astype(dtype_f)
        self.x_grid, self.y_grid = self.x[0, :], self.y[:, 0]
        self.mask = mask
        self.field_mask = mask[self.y.astype(int), self.x.astype(int)] if mask is not None else None

    @property
    def coords(self):
        return self.x, self.y

    @property
    def grid_coords(self):
        return self.x_grid, self.y_grid


def _geometry(frame_shape, window_size, search_size, overlap_ratio, center):
    """Field geometry computed by the library (piv_field_geometry)."""
    g = _lib.PivGeometry()
    ht, wd = frame_shape
    _lib.check(_lib.lib().piv_field_geometry(int(ht), int(wd), int(window_size), int(search_size),
                                             float(overlap_ratio), int(bool(center)), ctypes.byref(g)))
    return g


class CorrelationGPU:
    """Correlation of the window pairs of one pass (gpu_process.py:963-1376).

    ``frame_a``/``frame_b`` are device tensors (or host arrays, uploaded once).
    ``modules`` is accepted for signature compatibility and unused.
    """

    def __init__(self, frame_a, frame_b, modules=None, deforming_order=DEFORMING_ORDER, normalize=NORMALIZE,
                 subpixel_method=SUBPIXEL_METHOD, s2n_method=S2N_METHOD, s2n_size=S2N_SIZE, dtype_f=DTYPE_f,
                 dft="fft"):
        torch = _torch()
        self.dtype_f = np.float32 if dtype_f in ("float32", np.float32) else np.float64
        tdt = torch.float32 if self.dtype_f == np.float32 else torch.float64
        self.frame_a = torch.as_tensor(np.asarray(frame_a, dtype=self.dtype_f) if isinstance(frame_a, np.ndarray)
                                       else frame_a.to(tdt)).cuda().contiguous()
        self.frame_b = torch.as_tensor(np.asarray(frame_b, dtype=self.dtype_f) if isinstance(frame_b, np.ndarray)
                                       else frame_b.to(tdt)).cuda().contiguous()
        self.deforming_order = deforming_order
        self.is_normalized = normalize
        self.subpixel_method = subpixel_method
        self.s2n_method = s2n_method
        self.s2n_size = s2n_size
        if dft not in _lib.DFT:
            raise ValueError(f"dft must be one of {sorted(_lib.DFT)}, not {dft!r}")
        self.dft = dft
        self.sig2noise = None
        self._args = None

    def __call__(self, piv_field, shift=None, n_fft=N_FFT, dt=DEFORMING_PAR, batch_size=BATCH_SIZE):
        torch = _torch()
        self.piv_field = piv_field
        self.sig2noise = None
        fa, fb = self.frame_a, self.frame_b
        g = piv_field.geometry
        pt = _lib.PIXEL["f32" if self.dtype_f == np.float32 else "f64"]
        stream = torch.cuda.current_stream().cuda_stream
        if shift is not None:
            up, vp = (torch.as_tensor(np.asarray(a) if not isinstance(a, torch.Tensor) else a)
                      .to(device="cuda", dtype=torch.float64).contiguous() for a in shift)
            da, db = torch.empty_like(fa), torch.empty_like(fb)
            _lib.check(_lib.lib().piv_deform(ctypes.byref(g), 1, fa.data_ptr(), fb.data_ptr(), pt, up.data_ptr(),
                                             vp.data_ptr(), float(dt), 1, None, None, None,
                                             _lib.DTYPE["float32" if self.dtype_f == np.float32 else "float64"],
                                             da.data_ptr(), db.data_ptr(), stream))
            fa, fb = da, db
        m, n = piv_field.field_shape
        tdt = torch.float32 if self.dtype_f == np.float32 else torch.float64
        self.fft_size = 2 ** ceil(log2(piv_field.search_size * n_fft))
        u = torch.empty((m, n), dtype=tdt, device="cuda")
        v = torch.empty_like(u)
        pi = torch.empty((m, n), dtype=torch.int32, device="cuda")
        pj = torch.empty_like(pi)
        self._args = (g, fa, fb, pt)
        _lib.check(_lib.lib().piv_correlate(ctypes.byref(g), 1, fa.data_ptr(), fb.data_ptr(), pt,
                                            _lib.DTYPE["float32" if self.dtype_f == np.float32 else "float64"],
                                            self.fft_size, int(bool(self.is_normalized)),
                                            _lib.SUBPIXEL[self.subpixel_method], None, u.data_ptr(), v.data_ptr(),
                                            pi.data_ptr(), pj.data_ptr(), _lib.S2N[self.s2n_method],
                                            int(self.s2n_size), None, _lib.DFT[self.dft], stream))
        self.u, self.v, self.i_peak1, self.j_peak1 = u, v, pi, pj
        return u, v

    def get_s2n_ratio(self):
        torch = _torch()
        g, fa, fb, pt = self._args
        m, n = self.piv_field.field_shape
        tdt = torch.float32 if self.dtype_f == np.float32 else torch.float64
        u = torch.empty((m, n), dtype=tdt, device="cuda")
        v = torch.empty_like(u)
        s2n = torch.empty_like(u)
        _lib.check(_lib.lib().piv_correlate(ctypes.byref(g), 1, fa.data_ptr(), fb.data_ptr(), pt,
                                            _lib.DTYPE["float32" if self.dtype_f == np.float32 else "float64"],
                                            self.fft_size, int(bool(self.is_normalized)),
                                            _lib.SUBPIXEL[self.subpixel_method], None, u.data_ptr(), v.data_ptr(),
                                            None, None, _lib.S2N[self.s2n_method], int(self.s2n_size),
                                            s2n.data_ptr(), _lib.DFT[self.dft],
                                            torch.cuda.current_stream().cuda_stream))
        self.sig2noise = s2n
        return s2n

    @property
    def s2n_ratio(self):
        if self.sig2noise is None:
            return self.get_s2n_ratio()
        return self.sig2noise


def gpu_piv(frame_a, frame_b, **kwargs):
    """Convenience call: returns (x, y, u, v, val_locations, s2n) for one pair."""
    frame_a = np.asarray(frame_a)
    frame_b = np.asarray(frame_b)
    if "min_search_size" not in kwargs and "min_window_size" not in kwargs:
        kwargs["min_search_size"] = 16
    proc = piv_gpu(tuple(int(s) for s in frame_a.shape), **kwargs)
    u, v = proc(frame_a, frame_b)
    x, y = proc.coords
    return x, y, u, v, proc.val_locations, None
