"""CuPy -> NumPy/SciPy import shim: runs the unmodified reference package on the CPU.

Test infrastructure only. ``make_golden.py`` calls :func:`install` before it
imports the reference's ``openpiv_gpu`` package from a source checkout, so that
the reference's own code path produces the golden vectors under this folder.
Nothing in the product imports this module.

What the shim supplies (each item is a name the reference imports):

* ``cupy``: NumPy's namespace, with every array result viewed as an ``ndarray``
  subclass that has ``.get()`` and keeps 0-d results as arrays (the reference
  calls ``.get()`` on ``count_nonzero`` results, ``gpu_misc.py:19``, and on GCV
  scores, ``gpu_smoothn.py:372``); the constants ``Inf``/``NINF`` that NumPy 2
  removed (used at ``gpu_process.py:1336,1353``); ``cupy.fft``; ``cupy.linalg``;
  ``cupy.lib.stride_tricks.as_strided``; ``RawModule``.
* ``cupy.RawModule``: ``get_function(name)`` returns a NumPy restatement of the
  reference's four CUDA C kernels (``gpu_process.py:1387-1547``), computed in the
  kernel's own float type.
* ``cupyx.scipy.{interpolate.RegularGridInterpolator, sparse.csr_matrix,
  sparse.linalg.spsolve, fft.dct, fft.idct}`` mapped to SciPy.
"""

import sys
import types

import numpy as np
import scipy.fft
import scipy.interpolate
import scipy.sparse
import scipy.sparse.linalg


class ndarray(np.ndarray):
    """NumPy array that answers ``.get()`` like a CuPy device array."""

    def get(self):
        return np.asarray(self)

    def __array_wrap__(self, arr, context=None, return_scalar=False):
        if isinstance(arr, np.ndarray):
            return arr.view(ndarray)
        return arr


def _wrap_value(obj):
    if isinstance(obj, ndarray):
        return obj
    if isinstance(obj, np.ndarray):
        return obj.view(ndarray)
    if isinstance(obj, (np.generic, bool, int, float)) and not isinstance(obj, (np.str_, np.bytes_)):
        return np.asarray(obj).view(ndarray)
    if isinstance(obj, tuple):
        return tuple(_wrap_value(o) for o in obj)
    if isinstance(obj, list):
        return [_wrap_value(o) for o in obj]
    return obj


def _wrap_fn(fn):
    def wrapped(*args, **kwargs):
        return _wrap_value(fn(*args, **kwargs))

    wrapped.__name__ = getattr(fn, "__name__", "wrapped")
    wrapped.__doc__ = getattr(fn, "__doc__", None)
    return wrapped


def _namespace(mod_name, source):
    mod = types.ModuleType(mod_name)
    for name in dir(source):
        if name.startswith("__"):
            continue
        obj = getattr(source, name)
        if isinstance(obj, np.ufunc) or isinstance(obj, type) or isinstance(obj, types.ModuleType):
            setattr(mod, name, obj)
        elif callable(obj):
            setattr(mod, name, _wrap_fn(obj))
        else:
            setattr(mod, name, obj)
    return mod


# ----------------------------------------------------------------------------
# NumPy restatements of the reference's RawModule kernels.
# ----------------------------------------------------------------------------
def _k_get_stack(grid, block, args):
    # gpu_process.py:1420-1449
    fo, f, ws, sp, j_off, i_off, n, wd, ht = args
    ws, sp, j_off, i_off, n, wd, ht = (int(a) for a in (ws, sp, j_off, i_off, n, wd, ht))
    n_wins = int(grid[0])
    fo3 = np.asarray(fo).reshape(-1)
    f2 = np.asarray(f)
    k = np.arange(n_wins)
    jj = (k % n)[:, None, None] * sp + j_off + np.arange(ws)[None, None, :]
    ii = (k // n)[:, None, None] * sp + i_off + np.arange(ws)[None, :, None]
    jj, ii = np.broadcast_arrays(jj, ii)
    inside = (jj >= 0) & (jj < wd) & (ii >= 0) & (ii < ht)
    out = fo3.reshape(n_wins, ws, ws)
    out[inside] = f2.reshape(-1)[(ii * wd + jj)[inside]]


def _k_get_masked_stack(grid, block, args):
    # gpu_process.py:1387-1418
    fo, f, ws, sp, k_offset, j_off, i_off, n, wd, ht, mask = args
    ws, sp, j_off, i_off, n, wd, ht = (int(a) for a in (ws, sp, j_off, i_off, n, wd, ht))
    n_wins = int(grid[0])
    f2 = np.asarray(f).reshape(-1)
    k_offset = np.asarray(k_offset).reshape(-1)
    mask = np.asarray(mask).reshape(-1)
    out = np.asarray(fo).reshape(-1, ws, ws)
    for k in range(n_wins):
        if mask[k]:
            continue
        jj = (k % n) * sp + j_off + np.arange(ws)[None, :]
        ii = (k // n) * sp + i_off + np.arange(ws)[:, None]
        jj, ii = np.broadcast_arrays(jj, ii)
        inside = (jj >= 0) & (jj < wd) & (ii >= 0) & (ii < ht)
        dst = out[k - int(k_offset[k])]
        dst[inside] = f2[(ii * wd + jj)[inside]]


def _interp_core(f, x, y, up, vp, dt, wd, ht):
    # gpu_process.py:1528-1546, evaluated in the kernel's float type.
    ft = np.asarray(f).dtype.type
    x, y, up, vp = (np.asarray(a) for a in (x, y, up, vp))
    dt = ft(dt)
    xi = (x + up * dt).astype(ft)
    yi = (y + vp * dt).astype(ft)
    xl = np.floor(xi.astype(np.float32)).astype(np.int64)
    yu = np.floor(yi.astype(np.float32)).astype(np.int64)
    yu = np.clip(yu, 0, ht - 2)
    xl = np.clip(xl, 0, wd - 2)
    yd = yu + 1
    xr = xl + 1
    f1 = np.asarray(f).reshape(-1)
    ful = f1[yu * wd + xl]
    fur = f1[yu * wd + xr]
    fdl = f1[yd * wd + xl]
    fdr = f1[yd * wd + xr]
    yuf, ydf, xlf, xrf = (a.astype(ft) for a in (yu, yd, xl, xr))
    return ((yi - yuf) * (xrf - xi) * fdl + (yi - yuf) * (xi - xlf) * fdr
            + (ydf - yi) * (xrf - xi) * ful + (ydf - yi) * (xi - xlf) * fur).astype(ft)


def _k_interpolate_frame(grid, block, args):
    fi, f, x, y, up, vp, dt, wd, ht = args
    out = np.asarray(fi)
    out[...] = _interp_core(f, x, y, up, vp, dt, int(wd), int(ht))


def _k_interpolate_masked_frame(grid, block, args):
    # gpu_process.py:1461-1506
    fi, f, x, y, up, vp, dt, wd, ht, mask = args
    out = np.asarray(fi)
    val = _interp_core(f, x, y, up, vp, dt, int(wd), int(ht))
    keep = ~np.asarray(mask, dtype=bool)
    out[keep] = val[keep]


_KERNELS = {
    "cuda_get_stack": _k_get_stack,
    "cuda_get_masked_stack": _k_get_masked_stack,
    "cuda_interpolate_frame": _k_interpolate_frame,
    "cuda_interpolate_masked_frame": _k_interpolate_masked_frame,
}


class RawModule:
    def __init__(self, code=None, options=()):
        self.code = code
        self.options = options

    def get_function(self, name):
        fn = _KERNELS[name]

        def launch(grid, block, args):
            fn(grid, block, args)

        return launch


def _count_nonzero(a, *args, **kwargs):
    return np.asarray(np.count_nonzero(a, *args, **kwargs)).view(ndarray)


def install():
    """Registers the shim modules in ``sys.modules`` (idempotent)."""
    if "cupy" in sys.modules and getattr(sys.modules["cupy"], "_IS_SHIM", False):
        return
    cp = _namespace("cupy", np)
    cp._IS_SHIM = True
    cp.ndarray = ndarray
    cp.Inf = np.inf
    cp.NINF = -np.inf
    cp.newaxis = None
    cp.count_nonzero = _count_nonzero
    cp.RawModule = RawModule
    cp.fft = _namespace("cupy.fft", np.fft)
    cp.linalg = _namespace("cupy.linalg", np.linalg)
    lib = types.ModuleType("cupy.lib")
    st = types.ModuleType("cupy.lib.stride_tricks")
    st.as_strided = _wrap_fn(np.lib.stride_tricks.as_strided)
    lib.stride_tricks = st
    cp.lib = lib

    cupyx = types.ModuleType("cupyx")
    cx_scipy = types.ModuleType("cupyx.scipy")
    cx_interp = types.ModuleType("cupyx.scipy.interpolate")

    class RegularGridInterpolator(scipy.interpolate.RegularGridInterpolator):
        def __init__(self, points, values, **kwargs):
            points = tuple(np.asarray(p) for p in points)
            super().__init__(points, np.asarray(values), **kwargs)

        def __call__(self, xi, **kwargs):
            if isinstance(xi, tuple):
                xi = tuple(np.asarray(a) for a in xi)
            return _wrap_value(super().__call__(xi, **kwargs))

    cx_interp.RegularGridInterpolator = RegularGridInterpolator
    cx_sparse = types.ModuleType("cupyx.scipy.sparse")
    cx_sparse.csr_matrix = lambda a, *args, **kw: scipy.sparse.csr_matrix(np.asarray(a), *args, **kw)
    cx_sparse_linalg = types.ModuleType("cupyx.scipy.sparse.linalg")
    cx_sparse_linalg.spsolve = lambda A, b, *args, **kw: _wrap_value(
        scipy.sparse.linalg.spsolve(A, np.asarray(b), *args, **kw))
    cx_sparse.linalg = cx_sparse_linalg
    cx_fft = types.ModuleType("cupyx.scipy.fft")
    cx_fft.dct = _wrap_fn(scipy.fft.dct)
    cx_fft.idct = _wrap_fn(scipy.fft.idct)
    cx_scipy.interpolate = cx_interp
    cx_scipy.sparse = cx_sparse
    cx_scipy.fft = cx_fft
    cupyx.scipy = cx_scipy

    sys.modules.update({
        "cupy": cp,
        "cupy.fft": cp.fft,
        "cupy.linalg": cp.linalg,
        "cupy.lib": lib,
        "cupy.lib.stride_tricks": st,
        "cupyx": cupyx,
        "cupyx.scipy": cx_scipy,
        "cupyx.scipy.interpolate": cx_interp,
        "cupyx.scipy.sparse": cx_sparse,
        "cupyx.scipy.sparse.linalg": cx_sparse_linalg,
        "cupyx.scipy.fft": cx_fft,
    })
