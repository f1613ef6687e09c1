"""Validation and replacement of PIV fields on the GB300 kernels.

Mirrors openpiv_gpu.gpu_validation (ValidationGPU, gpu_validation.py:25-243;
ReplacementGPU, gpu_validation.py:245-415). Fields are torch CUDA tensors or
host arrays; results are torch CUDA tensors.
"""

import numpy as np

from . import DTYPE_f
from . import _lib

# Default validation settings (gpu_validation.py:10-16).
VALIDATION_SIZE = 1
S2N_TOL = None
MEDIAN_TOL = 2
MAD_TOL = None
MEAN_TOL = None
RMS_TOL = None

# Default replacement settings (gpu_validation.py:18-23).
REPLACING_METHOD = "spring"
REPLACING_SIZE = 1
ALLOWED_REPLACING_METHODS = {"spring", "median", "mean"}


def _torch():
    import torch

    return torch


def _dev64(f):
    torch = _torch()
    t = f if isinstance(f, torch.Tensor) else torch.as_tensor(np.asarray(f))
    return t.to(device="cuda", dtype=torch.float64).contiguous()


def _is_fp32(f):
    torch = _torch()
    if isinstance(f, torch.Tensor):
        return f.dtype == torch.float32
    return np.asarray(f).dtype == np.float32


class ValidationGPU:
    """Outlier detection by S2N, local median, MAD, local mean and global RMS
    tests, OR-ed and cleared inside the mask (gpu_validation.py:80-121).
    Sizes 1..3 are supported."""

    def __init__(self, f_shape, s2n_ratio=None, size=VALIDATION_SIZE, s2n_tol=S2N_TOL, median_tol=MEDIAN_TOL,
                 mad_tol=MAD_TOL, mean_tol=MEAN_TOL, rms_tol=RMS_TOL, dtype_f=DTYPE_f):
        self.f_shape = tuple(f_shape)
        self.s2n_ratio = s2n_ratio
        self.validation_tols = {"s2n": s2n_tol, "median": median_tol, "mad": mad_tol, "mean": mean_tol,
                                "rms": rms_tol}
        self.size = size
        assert all(self.size <= item for item in self.f_shape), "size cannot exceed field_shape."
        self.dtype_f = dtype_f
        self.val_locations = None

    def __call__(self, *f, mask=None):
        torch = _torch()
        if all(t is None for t in self.validation_tols.values()):
            self.val_locations = None
            return None
        fields = list(f)
        fp32 = int(all(_is_fp32(x) for x in fields))
        m, n = self.f_shape
        stream = torch.cuda.current_stream().cuda_stream
        s2n_ptr, s2n_dt = None, 0
        if self.s2n_ratio is not None and self.validation_tols["s2n"] is not None:
            s2n = self.s2n_ratio if isinstance(self.s2n_ratio, torch.Tensor) else torch.as_tensor(self.s2n_ratio)
            s2n = s2n.cuda().contiguous()
            s2n_dt = 1 if s2n.dtype == torch.float64 else 0
            if s2n.dtype not in (torch.float32, torch.float64):
                s2n = s2n.double()
                s2n_dt = 1
            self._s2n = s2n
            s2n_ptr = s2n.data_ptr()
        excl = None
        if mask is not None:
            excl = (mask if isinstance(mask, torch.Tensor) else torch.as_tensor(np.asarray(mask)))
            excl = excl.to(device="cuda", dtype=torch.uint8).contiguous()
        if len(fields) == 1:
            fields = fields * 2
        out = None
        for k in range(0, len(fields), 2):
            u = _dev64(fields[k])
            v = _dev64(fields[k + 1] if k + 1 < len(fields) else fields[k])
            val = torch.empty((m, n), dtype=torch.uint8, device="cuda")
            t = self.validation_tols
            _lib.check(_lib.lib().piv_validate(m, n, 1, u.data_ptr(), v.data_ptr(), s2n_ptr, s2n_dt, int(self.size),
                                               _lib.opt(t["s2n"]), _lib.opt(t["median"]), _lib.opt(t["mad"]),
                                               _lib.opt(t["mean"]), _lib.opt(t["rms"]), None,
                                               excl.data_ptr() if excl is not None else None, fp32,
                                               val.data_ptr(), stream))
            out = val.bool() if out is None else (out | val.bool())
        self.val_locations = out
        return out


class ReplacementGPU:
    """Replacement of outliers by spring, local median or local mean
    (gpu_validation.py:245-334). One call replaces once; points that stay
    unresolved (no usable neighbour, singular spring system) keep their input
    values."""

    def __init__(self, f_shape, method=REPLACING_METHOD, size=REPLACING_SIZE, dtype_f=DTYPE_f):
        self.f_shape = tuple(f_shape)
        self.method = method
        self.size = size
        assert all(self.size <= item for item in self.f_shape), "size cannot exceed field_shape."
        self.dtype_f = dtype_f

    def __call__(self, *f, val_locations, n_vals=None, fill_value=None):
        torch = _torch()
        fields = list(f)
        if len(fields) == 1:
            fields = fields * 2
        fp32 = int(all(_is_fp32(x) for x in fields))
        m, n = self.f_shape
        dtype = _lib.DTYPE["float32" if self.dtype_f in ("float32", np.float32) else "float64"]
        stream = torch.cuda.current_stream().cuda_stream
        results = []
        for k in range(0, len(fields), 2):
            u = _dev64(fields[k]).clone()
            v = _dev64(fields[k + 1] if k + 1 < len(fields) else fields[k]).clone()
            val = (val_locations if isinstance(val_locations, torch.Tensor) else
                   torch.as_tensor(np.asarray(val_locations))).to(device="cuda", dtype=torch.uint8).contiguous().clone()
            nan = float("nan")
            _lib.check(_lib.lib().piv_replace(m, n, 1, u.data_ptr(), v.data_ptr(), val.data_ptr(), None, 1,
                                              _lib.REPLACE[self.method], int(self.size), 0, None, 0, 1, nan, nan,
                                              nan, nan, nan, fp32, dtype, stream))
            results += [u, v]
        results = results[:len(f)]
        if fp32:
            results = [r.float() for r in results]
        return results if len(results) > 1 else results[0]
