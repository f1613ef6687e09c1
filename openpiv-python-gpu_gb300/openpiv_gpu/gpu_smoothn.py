"""smoothn of PIV fields on the GB300 kernels.

Mirrors openpiv_gpu.gpu_smoothn.SmoothnGPU (gpu_smoothn.py:37-439) for the
way PIVGPU uses it: order 2, non-robust, equal weights, two fields sharing
one smoothing parameter chosen by GCV when ``s`` is None.
"""

import logging
from math import log10, sqrt

import numpy as np

from . import DTYPE_f
from . import _lib

_log = logging.getLogger(__name__)

# Default settings (gpu_smoothn.py:16-35).
SMOOTHING_WEIGHTS = None
INIT_GUESS = None
SPACING = None
SMOOTHING_PAR = None
SMOOTHING_ORDER = 2
MAX_ROBUST_STEPS = 3
MAX_SMOOTHING_ITERS = 100
TOL = 1e-3
ROBUST = False
WEIGHTING_METHOD = "bisquare"


def _torch():
    import torch

    return torch


def p_bounds(shape):
    """Bounds of p = log10(s) for order 2 (gpu_smoothn.py:320-338)."""
    h_min = 1e-3
    h_max = 1 - h_min
    rank = sum(1 for d in shape if d != 1)
    a_max, a_min = h_max ** (2 / rank), h_min ** (2 / rank)
    p_min = log10((((1 + sqrt(1 + 8 * a_max)) / 4 / a_max) ** 2 - 1) / 16)
    p_max = log10((((1 + sqrt(1 + 8 * a_min)) / 4 / a_min) ** 2 - 1) / 16)
    return p_min, p_max


def log_flags(flags, shape, max_iters=MAX_SMOOTHING_ITERS):
    """Logs SmoothnGPU's messages (gpu_smoothn.py:218-222, 429-439) for the
    PIV_SMOOTH_* flag word of one smoothing."""
    if flags & (_lib.SMOOTH_S_LOWER | _lib.SMOOTH_S_UPPER):
        p_min, p_max = p_bounds(shape)
        if flags & _lib.SMOOTH_S_LOWER:
            _log.info('The lower bound for s ({:.3f}) has been reached. '
                      'Put s as an input variable if required.'.format(10 ** p_min))
        else:
            _log.info('The upper bound for s ({:.3f}) has been reached. '
                      'Put s as an input variable if required.'.format(10 ** p_max))
    if flags & _lib.SMOOTH_MAX_ITERS:
        _log.info('The maximum number of iterations ({:d}) has been exceeded. '
                  'Increase max_iters option or decrease tol_z value.'.format(max_iters))


class SmoothnGPU:
    """Discretised smoothing spline (Garcia 2010) by DCT, GCV choice of s."""

    def __init__(self, f_shape, mask=None, w=SMOOTHING_WEIGHTS, z0=INIT_GUESS, spacing=SPACING, s=SMOOTHING_PAR,
                 smoothing_order=SMOOTHING_ORDER, max_steps=MAX_ROBUST_STEPS, max_iters=MAX_SMOOTHING_ITERS,
                 tol_z=TOL, robust=ROBUST, weighting_method=WEIGHTING_METHOD, dtype_f=DTYPE_f):
        if w is not None or z0 is not None or spacing is not None or smoothing_order != 2 or robust:
            raise NotImplementedError("only the PIVGPU configuration of smoothn is implemented "
                                      "(order 2, non-robust, no weights, unit spacing)")
        self.f_shape = tuple(f_shape)
        self.mask = mask
        self.s = s
        self.is_auto = s is None
        self.p = None

    def __call__(self, *f):
        torch = _torch()
        fields = list(f)
        if len(fields) not in (1, 2):
            raise NotImplementedError("smoothn of one or two fields")
        m, n = self.f_shape
        u = (fields[0] if isinstance(fields[0], torch.Tensor) else torch.as_tensor(np.asarray(fields[0])))
        u = u.to(device="cuda", dtype=torch.float64).contiguous().clone()
        v = u.clone() if len(fields) == 1 else (fields[1] if isinstance(fields[1], torch.Tensor) else
                                                torch.as_tensor(np.asarray(fields[1]))).to(
            device="cuda", dtype=torch.float64).contiguous().clone()
        mask_ptr = None
        if self.mask is not None:
            self._mask = torch.as_tensor(np.asarray(self.mask)).to(device="cuda", dtype=torch.uint8).contiguous()
            mask_ptr = self._mask.data_ptr()
        p = torch.empty(1, dtype=torch.float64, device="cuda")
        flags = torch.zeros(1, dtype=torch.int32, device="cuda")
        s = float("nan") if self.s is None else float(self.s)
        _lib.check(_lib.lib().piv_smoothn_flags(m, n, 1, u.data_ptr(), v.data_ptr(), mask_ptr, s, p.data_ptr(),
                                                flags.data_ptr(), torch.cuda.current_stream().cuda_stream))
        self.p = float(p.item())
        self.flags = int(flags.item())
        log_flags(self.flags, self.f_shape)
        if self.s is None:
            self.s = float(10.0 ** self.p)
        return [u] if len(fields) == 1 else [u, v]

    @property
    def smoothing_par(self):
        return self.s
