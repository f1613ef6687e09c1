"""CPU oracle for the multi-pass PIV hot path (TEST INFRASTRUCTURE ONLY).

A NumPy/SciPy restatement of the reference's ``PIVGPU.__call__`` path
(``openpiv_gpu/gpu_process.py``, ``gpu_validation.py``, ``gpu_smoothn.py``,
``gpu_misc.py``). It is the checker: only ``tests/``, ``__graft_entry__.smoke()``
and ``bench.py``'s CPU-baseline leg use it. The GPU product never calls it.

Pinning: ``tests/golden/make_golden.py`` runs the unmodified reference through a
CuPy->NumPy import shim and stores its outputs under ``tests/golden/``;
``tests/test_oracle_golden.py`` checks this restatement against them.

Numerics follow the reference's dtype flow exactly:

* ``dtype_f`` (float32 or float64) for frames, window stacks, FFT correlation,
  the subpixel fit and the correlation output (``gpu_process.py:582,1127,1213``);
* smoothn always runs in float64 (``SmoothnGPU`` is built without ``dtype_f``,
  ``gpu_process.py:842``, default ``gpu_smoothn.py:103``), so from the first
  smoothed pass onward ``u + up`` (``gpu_process.py:632``), validation and
  replacement run in float64;
* smoothing runs after every non-final iteration regardless of ``smooth`` because
  the reference tests the tuple ``self.is_smoothed`` instead of the per-pass flag
  (``gpu_process.py:839-841``).

``deforming_order`` is inert in the reference (``gpu_process.py:403``; the only
deformation kernel is bilinear). Order 3 here is this project's definition of
cubic deformation: ``scipy.ndimage.map_coordinates(frame, (clip(y), clip(x)),
order=3, mode='mirror')`` with the sample coordinates clamped into the frame.
Order 1 (and any other value) is the reference's bilinear kernel.
"""

from math import ceil, log2, log10, prod, sqrt

import numpy as np
import scipy.fft
import scipy.ndimage
import scipy.optimize
import scipy.sparse
import scipy.sparse.linalg

# Defaults: gpu_process.py:19-35, gpu_validation.py:10-20, gpu_smoothn.py:16-35.
DEFAULTS = dict(
    search_size_iters=1, overlap_ratio=0.5, shrink_ratio=1, center=True, deforming_order=1, normalize=True,
    subpixel_method="gaussian", n_fft=2, deforming_par=0.5, batch_size="full", s2n_method="peak2peak",
    s2n_size=2, validation_size=1, s2n_tol=None, median_tol=2, mad_tol=None, mean_tol=None, rms_tol=None,
    num_replacing_iters=1, replacing_method="spring", replacing_size=1, revalidate=False, smooth=True,
    smoothing_par=None, dt=1, scaling_par=1, mask=None, dtype_f="float64",
)
EPS = 1e-7  # gpu_process.py:1011


def _per_pass(value, n, scalar_types):
    """Scalar -> tuple broadcast used by every per-pass setting (gpu_process.py:497-546)."""
    if value is None or isinstance(value, scalar_types):
        return (value,) * n
    return tuple(value)


def expand_settings(min_search_size, **kw):
    """Returns the per-iteration settings list (gpu_process.py:497-546, 675-728)."""
    s = dict(DEFAULTS)
    s.update(kw)
    ss_iters = (s["search_size_iters"],) if isinstance(s["search_size_iters"], int) else tuple(s["search_size_iters"])
    n_passes = len(ss_iters)
    ov = s["overlap_ratio"]
    ov = (ov,) * n_passes if ov == 0 or isinstance(ov, float) else tuple(ov)
    dp = s["deforming_par"]
    dp = (dp,) * n_passes if dp == 0 or dp == 1 or isinstance(dp, float) else tuple(dp)
    per = dict(
        deforming_order=_per_pass(s["deforming_order"], n_passes, int),
        normalize=_per_pass(s["normalize"], n_passes, bool),
        subpixel_method=_per_pass(s["subpixel_method"], n_passes, str),
        n_fft=_per_pass(s["n_fft"], n_passes, int),
        batch_size=_per_pass(s["batch_size"], n_passes, (int, str)),
        s2n_method=_per_pass(s["s2n_method"], n_passes, str),
        s2n_size=_per_pass(s["s2n_size"], n_passes, int),
        validation_size=_per_pass(s["validation_size"], n_passes, int),
        s2n_tol=_per_pass(s["s2n_tol"], n_passes, (int, float)),
        median_tol=_per_pass(s["median_tol"], n_passes, (int, float)),
        mad_tol=_per_pass(s["mad_tol"], n_passes, (int, float)),
        mean_tol=_per_pass(s["mean_tol"], n_passes, (int, float)),
        rms_tol=_per_pass(s["rms_tol"], n_passes, (int, float)),
        num_replacing_iters=_per_pass(s["num_replacing_iters"], n_passes, int),
        replacing_method=_per_pass(s["replacing_method"], n_passes, str),
        replacing_size=_per_pass(s["replacing_size"], n_passes, int),
        revalidate=_per_pass(s["revalidate"], n_passes, bool),
        smooth=_per_pass(s["smooth"], n_passes, bool),
        smoothing_par=_per_pass(s["smoothing_par"], n_passes, (int, float)),
    )
    iters = []
    for i, n_it in enumerate(ss_iters):
        for _ in range(n_it):
            it = {k: v[i] for k, v in per.items()}
            it["search_size"] = 2 ** (n_passes - i - 1) * min_search_size  # gpu_process.py:679
            it["overlap_ratio"] = ov[i]
            it["deforming_par"] = dp[i]
            iters.append(it)
    return s, iters


class Field:
    """Field geometry (gpu_process.py:897-961)."""

    def __init__(self, frame_shape, window_size, search_size, overlap_ratio, center, mask, dtype_f):
        self.frame_shape = frame_shape
        self.window_size = window_size
        self.search_size = search_size
        self.overlap = int(overlap_ratio * search_size)
        self.pad = (search_size - window_size) // 2
        self.spacing = search_size - self.overlap
        ht, wd = frame_shape
        m = (ht - search_size) // self.spacing + 1
        n = (wd - search_size) // self.spacing + 1
        self.field_shape = (m, n)
        self.n_wins = m * n
        if center:
            self.x_offset = (wd - (self.spacing * (n - 1) + search_size)) // 2 + search_size % 2
            self.y_offset = (ht - (self.spacing * (m - 1) + search_size)) // 2 + search_size % 2
        else:
            self.x_offset = self.y_offset = 0
        xg = np.arange(n) * self.spacing + search_size / 2.0 + self.x_offset
        yg = np.arange(m) * self.spacing + search_size / 2.0 + self.y_offset
        x, y = np.meshgrid(xg, yg)
        self.x, self.y = x.astype(dtype_f), y.astype(dtype_f)
        self.x_grid, self.y_grid = self.x[0, :], self.y[:, 0]
        self.field_mask = mask[self.y.astype(int), self.x.astype(int)] if mask is not None else None


def grid_interp(yg, xg, values, yq, xq):
    """Linear interpolation on a rectilinear grid with linear extrapolation outside it.

    Restates ``RegularGridInterpolator(..., bounds_error=False, fill_value=None)``
    as used at gpu_process.py:737-740 and 1159-1162: interval index clamped to
    ``[0, n-2]``, weights from the unclamped normalised distance. Evaluated in
    float64.
    """
    yg = np.asarray(yg, dtype=np.float64)
    xg = np.asarray(xg, dtype=np.float64)
    yq = np.asarray(yq, dtype=np.float64)
    xq = np.asarray(xq, dtype=np.float64)
    v = np.asarray(values, dtype=np.float64)
    iy = np.clip(np.searchsorted(yg, yq, side="right") - 1, 0, len(yg) - 2)
    ix = np.clip(np.searchsorted(xg, xq, side="right") - 1, 0, len(xg) - 2)
    ty = (yq - yg[iy]) / (yg[iy + 1] - yg[iy])
    tx = (xq - xg[ix]) / (xg[ix + 1] - xg[ix])
    v00, v01 = v[iy, ix], v[iy, ix + 1]
    v10, v11 = v[iy + 1, ix], v[iy + 1, ix + 1]
    return (v00 * (1 - ty) * (1 - tx) + v01 * (1 - ty) * tx + v10 * ty * (1 - tx) + v11 * ty * tx)


def bilinear_frame(f, x, y, up, vp, dt, mask=None):
    """The reference's frame-deformation kernel (gpu_process.py:1461-1547) in the
    frame's float type: clamped base index, unclamped weights (linear
    extrapolation at the borders)."""
    ft = f.dtype.type
    ht, wd = f.shape
    dt = ft(dt)
    xi = (x + up * dt).astype(ft)
    yi = (y + vp * dt).astype(ft)
    xl = np.clip(np.floor(xi.astype(np.float32)).astype(np.int64), 0, wd - 2)
    yu = np.clip(np.floor(yi.astype(np.float32)).astype(np.int64), 0, ht - 2)
    yd, xr = yu + 1, xl + 1
    f1 = f.reshape(-1)
    ful, fur = f1[yu * wd + xl], f1[yu * wd + xr]
    fdl, fdr = f1[yd * wd + xl], f1[yd * wd + xr]
    yuf, ydf, xlf, xrf = (a.astype(ft) for a in (yu, yd, xl, xr))
    out = ((yi - yuf) * (xrf - xi) * fdl + (yi - yuf) * (xi - xlf) * fdr
           + (ydf - yi) * (xrf - xi) * ful + (ydf - yi) * (xi - xlf) * fur).astype(ft)
    if mask is not None:
        out = np.where(mask, ft(0), out)
    return out


def cubic_frame(f, x, y, up, vp, dt, mask=None, coeffs=None):
    """Cubic B-spline deformation (this project's definition of deforming_order=3):
    ``map_coordinates(f, (clip(yi), clip(xi)), order=3, mode='mirror')`` where
    ``xi = x + up*dt`` is formed in the frame's float type like the bilinear kernel."""
    ft = f.dtype.type
    ht, wd = f.shape
    dt = ft(dt)
    xi = np.clip((x + up * dt).astype(ft), 0, wd - 1).astype(np.float64)
    yi = np.clip((y + vp * dt).astype(ft), 0, ht - 1).astype(np.float64)
    if coeffs is None:
        coeffs = scipy.ndimage.spline_filter(f.astype(np.float64), order=3, mode="mirror")
    out = scipy.ndimage.map_coordinates(coeffs, (yi, xi), order=3, mode="mirror", prefilter=False).astype(ft)
    if mask is not None:
        out = np.where(mask, ft(0), out)
    return out


def get_stack(f, field):
    """Gathers the (n_wins, ss, ss) window stack (gpu_process.py:1122-1147, 1420-1449)."""
    ss, sp = field.search_size, field.spacing
    m, n = field.field_shape
    iy = (np.arange(m) * sp + field.y_offset)[:, None] + np.arange(ss)[None, :]
    ix = (np.arange(n) * sp + field.x_offset)[:, None] + np.arange(ss)[None, :]
    st = f[iy[:, None, :, None], ix[None, :, None, :]]
    return st.reshape(m * n, ss, ss)


def fft_size(search_size, n_fft):
    """N = 2**ceil(log2(ss * n_fft)) (gpu_process.py:1099-1109)."""
    return 2 ** ceil(log2(search_size * n_fft))


def correlate(win_a, win_b, N, normalize, dtype_f, chunk=8192):
    """Mean removal, centred zero-pad, irfft2(conj(rfft2(a)) * rfft2(b)), fftshift
    (gpu_process.py:1065, 1077-1086, 1201-1246). Returns (n_wins, N, N)."""
    n_wins, ss, _ = win_a.shape
    pad = (N - ss) // 2
    if pad != 0:
        normalize = True  # gpu_process.py:1065
    win_a = win_a.astype(dtype_f, copy=True)
    win_b = win_b.astype(dtype_f, copy=True)
    if normalize:
        win_a -= np.mean(win_a, axis=(1, 2), keepdims=True)
        win_b -= np.mean(win_b, axis=(1, 2), keepdims=True)
    corr = np.empty((n_wins, N, N), dtype=dtype_f)
    for s in range(0, n_wins, chunk):
        a = win_a[s:s + chunk]
        b = win_b[s:s + chunk]
        if pad != 0:
            pa = np.zeros((a.shape[0], N, N), dtype=dtype_f)
            pb = np.zeros_like(pa)
            pa[:, pad:-pad, pad:-pad] = a
            pb[:, pad:-pad, pad:-pad] = b
            a, b = pa, pb
        fa = np.fft.rfft2(a, axes=(1, 2))
        fb = np.fft.rfft2(b, axes=(1, 2))
        corr[s:s + chunk] = np.fft.irfft2(np.conj(fa) * fb, s=(N, N), axes=(1, 2))
    return np.fft.fftshift(corr, axes=(1, 2))


def first_peak(corr):
    """First-occurrence argmax over the row-major map (gpu_process.py:1248-1254)."""
    n, N, _ = corr.shape
    idx = np.argmax(corr.reshape(n, -1), axis=1)
    return idx // N, idx % N


def peak_gap(corr, i_peak, j_peak):
    """Relative gap between the highest and second-highest value of each map, a
    near-tie measure for argmax parity (0 means an exact tie)."""
    n = corr.shape[0]
    flat = corr.reshape(n, -1)
    top2 = -np.partition(-flat, 1, axis=1)[:, :2]
    denom = np.maximum(np.abs(top2[:, 0]), np.finfo(np.float32).tiny)
    return (top2[:, 0] - top2[:, 1]) / denom


def fragile_windows(corr, i_peak, j_peak, method, search_size, tie_tol=1e-5):
    """Windows whose integer peak or subpixel fit depends on floating-point
    rounding noise: a near tie between the two largest map values, or (for the
    Gaussian fit, which requires all five stencil values > 0) a stencil value
    on a lag without window overlap (|lag| >= search size), whose exact value
    is zero and whose computed value is rounding noise of either sign."""
    n, N, _ = corr.shape
    frag = peak_gap(corr, i_peak, j_peak) < tie_tol
    if method == "gaussian":
        lo = N // 2 - search_size  # shifted index of lag -ss
        hi = N // 2 + search_size  # shifted index of lag +ss
        for di, dj in ((0, 0), (-1, 0), (1, 0), (0, -1), (0, 1)):
            ii, jj = i_peak + di, j_peak + dj
            frag |= (ii <= lo) | (ii >= hi) | (jj <= lo) | (jj >= hi)
        inside = (i_peak > 0) & (i_peak < N - 1) & (j_peak > 0) & (j_peak < N - 1)
        frag &= inside | (peak_gap(corr, i_peak, j_peak) < tie_tol)
    return frag


def subpixel(corr, i_peak, j_peak, method, dtype_f):
    """Subpixel peak position (gpu_process.py:1256-1294)."""
    n, N, _ = corr.shape
    ft = np.dtype(dtype_f).type
    i_sp, j_sp = i_peak.astype(dtype_f), j_peak.astype(dtype_f)
    ok = (i_peak > 0) & (i_peak < N - 1) & (j_peak > 0) & (j_peak < N - 1)
    k = np.nonzero(ok)[0]
    ic, jc = i_peak[k], j_peak[k]
    c = corr[k, ic, jc]
    cd = corr[k, ic - 1, jc]
    cu = corr[k, ic + 1, jc]
    cl = corr[k, ic, jc - 1]
    cr = corr[k, ic, jc + 1]
    eps = ft(EPS)
    if method == "gaussian":
        pos = (c > 0) & (cd > 0) & (cu > 0) & (cl > 0) & (cr > 0)
        k, ic, jc = k[pos], ic[pos], jc[pos]
        c, cd, cu, cl, cr = (np.log(a[pos]) for a in (c, cd, cu, cl, cr))
        i_sp[k] = ic + ft(0.5) * (cd - cu) / (cd - ft(2.0) * c + cu + eps)
        j_sp[k] = jc + ft(0.5) * (cl - cr) / (cl - ft(2.0) * c + cr + eps)
    elif method == "parabolic":
        i_sp[k] = ic + ft(0.5) * (cd - cu) / (cd - ft(2.0) * c + cu + eps)
        j_sp[k] = jc + ft(0.5) * (cl - cr) / (cl - ft(2.0) * c + cr + eps)
    elif method == "centroid":
        i_sp[k] = ic + (cu - cd) / (cd + c + cu + eps)
        j_sp[k] = jc + (cr - cl) / (cl + c + cr + eps)
    return i_sp, j_sp


def s2n_ratio(corr, i_peak, j_peak, method, size, dtype_f):
    """Signal-to-noise ratio (gpu_process.py:1312-1365). ``corr`` is not modified
    here; the reference's peak2peak mutates its map in place, which only matters
    for a second call on the same map."""
    n, N, _ = corr.shape
    k = np.arange(n)
    p1 = corr[k, i_peak, j_peak]
    if method == "peak2peak":
        c2 = corr.copy()
        off = np.arange(-size, size + 1)
        ii = i_peak[:, None, None] + off[None, :, None]
        jj = j_peak[:, None, None] + off[None, None, :]
        ii, jj = np.broadcast_arrays(ii, jj)
        kk = np.broadcast_to(k[:, None, None], ii.shape)
        # fill_kernel (gpu_misc.py:52-85): negative indices wrap, out-of-range raise in NumPy;
        # CuPy wraps both. Indices are taken modulo N to match the device behaviour.
        c2[kk, ii % N, jj % N] = -np.inf
        i2, j2 = first_peak(c2)
        p2 = corr[k, i2, j2]
    elif method == "peak2mean":
        c2 = np.where(corr > 0.5 * p1[:, None, None], np.nan, corr)
        c2 = np.where(c2 <= 0, np.nan, c2)
        with np.errstate(invalid="ignore"):
            p2 = np.nanmean(c2, axis=(1, 2))
    else:
        c2 = np.where(corr <= 0, np.nan, corr)
        with np.errstate(invalid="ignore"):
            p2 = np.nanmean(c2, axis=(1, 2))
    s2n = np.zeros(n, dtype=dtype_f)
    with np.errstate(divide="ignore", invalid="ignore"):
        s2n = np.where(p1 > 0, p1 / p2, s2n)
    s2n = np.where(np.logical_and(p2 <= 0, p1 > 0), np.inf, s2n)
    return s2n.astype(dtype_f)


# ----------------------------------------------------------------------------
# Validation (gpu_validation.py:25-243).
# ----------------------------------------------------------------------------
def _neighbour_stack(f, size):
    """(m*n, 2s+1, 2s+1) NaN-padded neighbourhoods (gpu_validation.py:194-205)."""
    m, n = f.shape
    fp = np.pad(f, size, mode="constant", constant_values=np.nan)
    k = 2 * size + 1
    iy = np.arange(m)[:, None] + np.arange(k)[None, :]
    ix = np.arange(n)[:, None] + np.arange(k)[None, :]
    st = fp[iy[:, None, :, None], ix[None, :, None, :]].reshape(m * n, k, k)
    return st


def neighbour_stats(f, size, method, field_mask=None):
    """Local median/mean/MAD over the neighbourhood without its centre
    (gpu_validation.py:166-205)."""
    st = _neighbour_stack(f, size)
    st[:, size, size] = np.nan
    out = np.full(f.shape, np.nan, dtype=f.dtype)
    sel = np.ones(f.size, dtype=bool) if field_mask is None else ~field_mask.reshape(-1)
    with np.errstate(invalid="ignore"):
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore", RuntimeWarning)
            if method == "median":
                val = np.nanmedian(st[sel], axis=(1, 2))
            elif method == "mean":
                val = np.nanmean(st[sel], axis=(1, 2))
            else:
                med = np.nanmedian(st[sel], axis=(1, 2), keepdims=True)
                val = np.nanmedian(np.abs(st[sel] - med), axis=(1, 2))
    out.reshape(-1)[sel] = val
    return out


def validate(fields, size=1, s2n=None, s2n_tol=None, median_tol=2, mad_tol=None, mean_tol=None, rms_tol=None,
             mask=None):
    """Outlier test: OR of the selected tests, then AND with ~mask (gpu_validation.py:80-121)."""
    locs = []
    with np.errstate(invalid="ignore"):
        if s2n_tol is not None and s2n is not None:
            locs.append(s2n < s2n_tol)
        med = None
        if median_tol is not None:
            med = [neighbour_stats(f, size, "median", mask) for f in fields]
            locs.append(np.any([np.abs(f - md) > median_tol for f, md in zip(fields, med)], axis=0))
        if mad_tol is not None:
            med = med or [neighbour_stats(f, size, "median", mask) for f in fields]
            mad = [neighbour_stats(f, size, "mad", mask) for f in fields]
            locs.append(np.any([np.abs(f - md) > mad_tol * ma for f, md, ma in zip(fields, med, mad)], axis=0))
        if mean_tol is not None:
            mean = [neighbour_stats(f, size, "mean", mask) for f in fields]
            locs.append(np.any([np.abs(f - mn) > mean_tol for f, mn in zip(fields, mean)], axis=0))
        if rms_tol is not None:
            locs.append(np.any([np.abs(f - np.nanmean(f)) > rms_tol * np.nanstd(f) for f in fields], axis=0))
    if not locs:
        return None
    val = np.any(np.stack(locs, axis=0), axis=0)
    if mask is not None:
        val = np.logical_and(val, ~mask)
    return val


# ----------------------------------------------------------------------------
# Replacement (gpu_validation.py:245-415, gpu_process.py:788-834).
# ----------------------------------------------------------------------------
def _cross_mean(f, val, size, fill_value):
    """Mean of the 4 linked neighbours at distance ``size`` (NaN padding excluded)
    with outliers counted as ``fill_value`` (gpu_validation.py:381-394)."""
    src = np.where(val, fill_value, f) if fill_value is not None else f
    st = _neighbour_stack(src, size)[val.reshape(-1)]
    k = 2 * size + 1
    km = np.full((k, k), True)
    km[[size, size, k - 1, 0], [0, k - 1, size, size]] = False
    st = np.where(km, np.nan, st)
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        return np.nanmean(st, axis=(1, 2))


def _kernel_stat(f, val, size, method, fill_value):
    """Median/mean over the (2s+1)^2 neighbourhood without its centre
    (gpu_validation.py:373-394)."""
    src = np.where(val, fill_value, f) if fill_value is not None else f
    st = _neighbour_stack(src, size)[val.reshape(-1)]
    st[:, size, size] = np.nan
    import warnings
    with warnings.catch_warnings():
        warnings.simplefilter("ignore", RuntimeWarning)
        return np.nanmedian(st, axis=(1, 2)) if method == "median" else np.nanmean(st, axis=(1, 2))


def spring_coef(shape, size, dtype_f):
    """Link coefficients -1/4 interior, -1/3 edge, -1/2 corner (gpu_validation.py:365-371)."""
    coef = np.full(shape, -1 / 3, dtype=dtype_f)
    coef[size:-size, size:-size] = -1 / 4
    coef[:size, :size] = coef[:size, -size:] = coef[-size:, :size] = coef[-size:, -size:] = -1 / 2
    return coef


def replace_once(fields, val, method, size, fill_value, dtype_f):
    """One ReplacementGPU call (gpu_validation.py:295-334). Returns new fields."""
    out = [f.copy() for f in fields]
    n_vals = int(np.count_nonzero(val))
    if method == "spring":
        coef = spring_coef(val.shape, size, dtype_f)[val]
        iv, jv = np.nonzero(val)
        index = -np.ones(val.shape, dtype=np.int64)
        index[iv, jv] = np.arange(n_vals)
        rows, cols, data = [np.arange(n_vals)], [np.arange(n_vals)], [np.ones(n_vals, dtype=dtype_f)]
        m, n = val.shape
        for di, dj in ((0, -size), (0, size), (size, 0), (-size, 0)):
            ii, jj = iv + di, jv + dj
            ok = (ii >= 0) & (ii < m) & (jj >= 0) & (jj < n)
            nb = np.full(n_vals, -1)
            nb[ok] = index[ii[ok], jj[ok]]
            link = nb >= 0
            rows.append(np.arange(n_vals)[link])
            cols.append(nb[link])
            data.append(coef[link])
        A = scipy.sparse.csr_matrix((np.concatenate(data), (np.concatenate(rows), np.concatenate(cols))),
                                    shape=(n_vals, n_vals), dtype=dtype_f)
        for k, f in enumerate(fields):
            rhs = _cross_mean(f, val, size, 0)
            import warnings
            with warnings.catch_warnings():
                warnings.simplefilter("ignore")
                x = scipy.sparse.linalg.spsolve(A, rhs)
            out[k][val] = x
    else:
        for k, f in enumerate(fields):
            out[k][val] = _kernel_stat(f, val, size, method, fill_value)
    return out


def replace_outliers(fields, val, field_mask, n_iters, method, size, revalidate, vkw, dtype_f):
    """The replacement loop (gpu_process.py:788-834). Returns (fields, val)."""
    if val is None or np.count_nonzero(val) == 0 or n_iters == 0:
        return fields, val
    f_init = [f.copy() for f in fields]
    fill_value = np.nan
    cur = fields
    for _ in range(n_iters):
        if np.count_nonzero(val) == 0:
            break
        cur = replace_once(cur, val, method, size, fill_value, dtype_f)
        unresolved = np.logical_and(np.any([np.isnan(f) for f in cur], axis=0), val)
        if revalidate:
            mask = ~val if field_mask is None else np.logical_or(field_mask, ~val)
            cur = [np.where(unresolved, fi, f) for fi, f in zip(f_init, cur)]
            v2 = validate(cur, mask=mask, **vkw)
            val = np.logical_or(v2, unresolved) if v2 is not None else unresolved
        else:
            fill_value = None
    if not revalidate:
        unresolved = np.logical_and(np.any([np.isnan(f) for f in cur], axis=0), val)
        cur = [np.where(unresolved, fi, f) for fi, f in zip(f_init, cur)]
    return cur, val


# ----------------------------------------------------------------------------
# smoothn (gpu_smoothn.py:123-372), non-robust as PIVGPU uses it.
# ----------------------------------------------------------------------------
def dct2(z):
    return scipy.fft.dct(scipy.fft.dct(z, norm="ortho", type=2).T, norm="ortho", type=2).T


def idct2(z):
    return scipy.fft.idct(scipy.fft.idct(z, norm="ortho", type=2).T, norm="ortho", type=2).T


def p_bounds(shape, order=2):
    """Bounds of p = log10(s) (gpu_smoothn.py:320-338)."""
    h_min = 1e-3
    h_max = 1 - h_min
    rank = int(np.sum(np.array(shape) != 1))
    if order == 0:
        return log10(1 / h_max ** (1 / rank) - 1), log10(1 / h_min ** (1 / rank) - 1)
    if order == 1:
        return log10((1 / (h_max ** (2 / rank)) - 1) / 4), log10((1 / (h_min ** (2 / rank)) - 1) / 4)
    p_min = log10((((1 + sqrt(1 + 8 * h_max ** (2 / rank))) / 4 / h_max ** (2 / rank)) ** 2 - 1) / 16)
    p_max = log10((((1 + sqrt(1 + 8 * h_min ** (2 / rank))) / 4 / h_min ** (2 / rank)) ** 2 - 1) / 16)
    return p_min, p_max


def smoothn_lambda(shape):
    """Eigenvalues 2(2 - cos(pi i/m) - cos(pi j/n)) (gpu_smoothn.py:340-351), before ** order."""
    m, n = shape
    lam = np.cos(np.pi * np.arange(m) / m)[:, None] + np.cos(np.pi * np.arange(n) / n)[None, :]
    return 2 * (2 - lam)


def gcv_score(p, f_dct, lam2, n_finite, f_size, n_fields, w=None, f=None, is_finite=None):
    """GCV score (gpu_smoothn.py:353-372); ``w is None`` selects the w_mean > 0.9 branch."""
    gamma = 1 / (1 + 10 ** np.asarray(p, dtype=np.float64) * lam2)
    rss = 0.0
    if w is None:
        for fd in f_dct:
            rss += np.linalg.norm(fd * (gamma - 1)) ** 2
    else:
        for fd, fi in zip(f_dct, f):
            f_hat = idct2(gamma * fd)
            rss += np.linalg.norm(np.sqrt(w[is_finite]) * (fi[is_finite] - f_hat[is_finite])) ** 2
    tr_h = np.sum(gamma)
    return rss / n_finite / (1 - tr_h / f_size) ** 2 / n_fields


def smoothn(fields, mask=None, s=None, order=2, max_iters=100, tol_z=1e-3, trace=None):
    """Garcia's DCT-based penalised least squares (gpu_smoothn.py:123-231), GCV
    choice of s by a 10-point scan then L-BFGS-B (gpu_smoothn.py:179-193).
    Returns float64 fields."""
    shape = fields[0].shape
    f_size = prod(shape)
    if f_size < 2:
        return list(fields)
    f = [np.asarray(a, dtype=np.float64).copy() if a.dtype != np.float64 else a.copy() for a in fields]
    f = [a for a in f]
    n_fields = len(f)
    is_finite = np.ones(shape, dtype=bool)
    for a in f:
        is_finite &= np.isfinite(a)
    n_finite = int(np.sum(is_finite))
    missing = ~is_finite
    if np.any(missing):
        # replace_non_finite (gpu_smoothn.py:233-251): nearest finite neighbour by EDT.
        idx = scipy.ndimage.distance_transform_edt(missing, return_distances=False, return_indices=True)
        for a in f:
            a[missing] = a[tuple(idx)][missing]
    w = np.ones(shape, dtype=np.float64) * is_finite
    if mask is not None:
        w = np.where(mask, 0, w)
    is_weighted = bool(np.any(w != 1))
    if is_weighted:
        # get_init_z (gpu_smoothn.py:284-297): keep the lowest tenth of DCT coefficients.
        z = []
        for a in f:
            zd = dct2(a)
            n_dct = np.ceil(np.array(zd.shape) / 10).astype(int) + 1
            zd[n_dct[0]:, n_dct[1]:] = 0  # one trailing block (gpu_smoothn.py:291-293)
            z.append(idct2(zd))
    else:
        z = [np.zeros(shape, dtype=np.float64) for _ in range(n_fields)]
    is_auto = s is None
    if is_auto:
        p_min, p_max = p_bounds(shape, order)
        p = None
    else:
        p = log10(s)
    rf = 1 + 0.75 * is_weighted
    lam2 = smoothn_lambda(shape) ** order
    w_mean = float(np.mean(w))
    for k in range(max_iters):
        z0 = z
        f_dct = [dct2(w * (fi - zi) + zi) for fi, zi in zip(f, z)]
        if is_auto and not np.remainder(log2(k + 1), 1):
            args = (f_dct, lam2, n_finite, f_size, n_fields) + (() if w_mean > 0.9 else (w, f, is_finite))
            if not p:
                p_span = np.arange(10) * (1 / 9) * (p_max - p_min) + p_min
                g = np.array([gcv_score(pi, *args) for pi in p_span])
                p = p_span[np.argmin(g)]
            res = scipy.optimize.fmin_l_bfgs_b(lambda q, *a: float(gcv_score(q, *a)), np.array([p]), fprime=None,
                                               factr=10, approx_grad=True, bounds=[(p_min, p_max)], args=args)
            p = res[0][0]
        s_val = np.power(10, p)  # gpu_smoothn.py:196
        gamma = 1 / (1 + s_val * lam2)
        z = [rf * idct2(gamma * fd) + (1 - rf) * zi for fd, zi in zip(f_dct, z)]
        if is_weighted:
            num = np.linalg.norm(np.concatenate([a - b for a, b in zip(z0, z)]))
            tol = num / (np.linalg.norm(np.concatenate(z)) + 1e-6)
        else:
            tol = 0
        if tol <= tol_z:
            break
    if trace is not None:
        trace["p"] = p
        trace["smoothn_iters"] = k + 1
    if mask is not None:
        z = [np.where(mask, 0, zi) for zi in z]
    return z


# ----------------------------------------------------------------------------
# The multi-pass driver (gpu_process.py:564-647).
# ----------------------------------------------------------------------------
class OraclePIV:
    """Restatement of ``PIVGPU(frame_shape, min_search_size, **settings)``.

    ``__call__(frame_a, frame_b)`` returns ``(u, v)`` as NumPy arrays; after a
    call, ``trace`` holds one dict of intermediates per iteration.
    """

    def __init__(self, frame_shape, min_search_size, **kw):
        self.frame_shape = tuple(frame_shape)
        self.min_search_size = min_search_size
        self.settings, self.iters = expand_settings(min_search_size, **kw)
        self.dtype_f = np.float32 if self.settings["dtype_f"] == "float32" else np.float64
        mask = self.settings["mask"]
        self.mask = np.asarray(mask).astype(bool) if mask is not None else None
        shrink = self.settings["shrink_ratio"]
        self.fields = []
        for k, it in enumerate(self.iters):
            ss = it["search_size"]
            ws = ss
            if k == 0 and shrink != 1:
                ws = int(ss * shrink)
                ws = ws if ws % 2 == 0 else ws + 1
                ws = max(ws, 8)
            self.fields.append(Field(self.frame_shape, ws, ss, it["overlap_ratio"], self.settings["center"],
                                     self.mask, self.dtype_f))
        self.trace = []
        self.val_locations = None
        self.outliers = None
        self.s2n = None

    @property
    def coords(self):
        sp = self.settings["scaling_par"]
        return self.fields[-1].x * sp, self.fields[-1].y * sp

    @property
    def field_mask(self):
        return self.fields[-1].field_mask

    def __call__(self, frame_a, frame_b):
        ft = self.dtype_f
        fa = np.asarray(frame_a).astype(ft)
        fb = np.asarray(frame_b).astype(ft)
        if self.mask is not None:  # mask_frames (gpu_process.py:682-688)
            fa[self.mask] = 0
            fb[self.mask] = 0
        n_it = len(self.iters)
        self.trace = []
        u = v = None
        spline = {}
        for k, it in enumerate(self.iters):
            fld = self.fields[k]
            tr = {}
            up = vp = None
            if k > 0:
                up, vp = u, v
                prev = self.fields[k - 1]
                if prev.search_size != fld.search_size:  # interpolate_displacement (gpu_process.py:730-742)
                    up = grid_interp(prev.y_grid, prev.x_grid, up, fld.y, fld.x)
                    vp = grid_interp(prev.y_grid, prev.x_grid, vp, fld.y, fld.x)
                tr["up"], tr["vp"] = up, vp
            # Deformation (gpu_process.py:1111-1120, 1149-1192).
            da, db = fa, fb
            if up is not None:
                ht, wd = self.frame_shape
                x, y = np.meshgrid(np.arange(wd), np.arange(ht))
                x, y = x.astype(ft), y.astype(ft)
                upx = grid_interp(fld.y_grid, fld.x_grid, up, y, x).astype(ft)
                vpx = grid_interp(fld.y_grid, fld.x_grid, vp, y, x).astype(ft)
                dp = it["deforming_par"]
                if it["deforming_order"] == 3:
                    if not spline:
                        spline["a"] = scipy.ndimage.spline_filter(fa.astype(np.float64), order=3, mode="mirror")
                        spline["b"] = scipy.ndimage.spline_filter(fb.astype(np.float64), order=3, mode="mirror")
                    interp = lambda f, c, t: cubic_frame(f, x, y, upx, vpx, t, self.mask, coeffs=spline[c])
                else:
                    interp = lambda f, c, t: bilinear_frame(f, x, y, upx, vpx, t, self.mask)
                if 0 < dp < 1:
                    da, db = interp(fa, "a", dp - 1), interp(fb, "b", dp)
                elif dp == 1:
                    db = interp(fb, "b", 1)
                else:
                    da = interp(fa, "a", -1)
            N = fft_size(fld.search_size, it["n_fft"])
            wa, wb = get_stack(da, fld), get_stack(db, fld)
            sel = None
            if fld.field_mask is not None:
                sel = ~fld.field_mask.reshape(-1)
                wa, wb = wa[sel], wb[sel]
            if fld.pad != 0:  # shrink_ratio: zero the first stack outside the window (gpu_process.py:1072-1081)
                p = fld.pad
                z = np.zeros_like(wa)
                z[:, p:-p, p:-p] = wa[:, p:-p, p:-p]
                wa = z
                norm = True if (N - fld.search_size) // 2 != 0 else it["normalize"]
                if norm:
                    inner = wa[:, p:-p, p:-p].astype(ft)
                    wa = wa.astype(ft)
                    wa[:, p:-p, p:-p] = inner - np.mean(inner, axis=(1, 2), keepdims=True)
                    wb = wb.astype(ft) - np.mean(wb.astype(ft), axis=(1, 2), keepdims=True)
                corr = correlate(wa, wb, N, False, ft)
            else:
                corr = correlate(wa, wb, N, it["normalize"], ft)
            i1, j1 = first_peak(corr)
            i_sp, j_sp = subpixel(corr, i1, j1, it["subpixel_method"], ft)
            tr["i_peak"], tr["j_peak"] = i1, j1
            tr["peak_gap"] = peak_gap(corr, i1, j1)
            tr["fragile"] = fragile_windows(corr, i1, j1, it["subpixel_method"], fld.search_size)
            # The Gaussian-stencil rule alone (no tie rule): a fit that reads a lag without overlap.
            tr["stencil"] = fragile_windows(corr, i1, j1, it["subpixel_method"], fld.search_size, tie_tol=0.0)
            uc_flat = j_sp - N // 2
            vc_flat = i_sp - N // 2
            if sel is not None:
                uc = np.full(fld.field_shape, np.nan, dtype=ft)
                vc = np.full(fld.field_shape, np.nan, dtype=ft)
                uc.reshape(-1)[sel] = uc_flat
                vc.reshape(-1)[sel] = vc_flat
            else:
                uc, vc = uc_flat.reshape(fld.field_shape), vc_flat.reshape(fld.field_shape)
            tr["u_corr"], tr["v_corr"] = uc, vc
            s2n = None
            if it["s2n_tol"] is not None:
                s2n_flat = s2n_ratio(corr, i1, j1, it["s2n_method"], it["s2n_size"], ft)
                if sel is not None:
                    s2n = np.zeros(fld.field_shape, dtype=ft)
                    s2n.reshape(-1)[sel] = s2n_flat
                else:
                    s2n = s2n_flat.reshape(fld.field_shape)
                tr["s2n"] = s2n
                self.s2n = s2n
            del corr
            if k > 0:
                u, v = uc + up, vc + vp
            else:
                u, v = uc, vc
            tr["u_sum"], tr["v_sum"] = u, v
            vkw = dict(size=it["validation_size"], s2n=s2n, s2n_tol=it["s2n_tol"], median_tol=it["median_tol"],
                       mad_tol=it["mad_tol"], mean_tol=it["mean_tol"], rms_tol=it["rms_tol"])
            val = validate([u, v], mask=fld.field_mask, **vkw)
            tr["val0"] = val
            if k == n_it - 1:
                self.val_locations = val
            (u, v), val = replace_outliers([u, v], val, fld.field_mask, it["num_replacing_iters"],
                                           it["replacing_method"], it["replacing_size"], it["revalidate"], vkw, ft)
            tr["u_rep"], tr["v_rep"] = u, v
            if k == n_it - 1:
                self.outliers = validate([u, v], mask=fld.field_mask, **vkw)
            if k != n_it - 1:
                st = {}
                u, v = smoothn([u, v], mask=fld.field_mask, s=it["smoothing_par"], trace=st)
                tr.update(st)
                tr["u_smooth"], tr["v_smooth"] = u, v
            self.trace.append(tr)
        dt, sc = self.settings["dt"], self.settings["scaling_par"]
        if dt != 1 or sc != 1:  # scale_fields (gpu_process.py:847-849)
            u, v = u * sc / dt, v * sc / dt
        return u, v
