"""Stage-level GPU parity through the C ABI against the CPU oracle on seeded
random inputs: correlation (every FFT size, both float types, every subpixel
and S2N method), predictor regrid, frame deformation (bilinear and cubic),
validation, replacement and smoothn.

Tolerances: displacements 1e-4 px for the correlation alone; predictor regrid
bit-exact; deformed pixels within 1e-2 grey levels (the per-pixel predictor
is float32 on the device, float64 in the reference; cubic also has float32
spline coefficients);
validation masks identical; replacement 1e-5 px; smoothed fields 1e-6 px at a
fixed smoothing parameter.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

from oracle import piv_oracle as po  # noqa: E402


@pytest.fixture(scope="module")
def env():
    import torch

    from openpiv_gpu import _build, _lib

    _build.build()
    torch.cuda.set_device(0)
    return torch, _lib, _lib.load()


def _geom(_lib, lib, shape, ss, ov, center=True, ws=None):
    g = _lib.PivGeometry()
    _lib.check(lib.piv_field_geometry(shape[0], shape[1], ws or ss, ss, ov, int(center), ctypes.byref(g)))
    return g


def _frames(seed, shape, n_pairs=1, shift=(1.3, -0.6)):
    from openpiv_gpu import synthetic as syn

    a, b = [], []
    for k in range(n_pairs):
        fa, fb = syn.render_pair(shape, syn.uniform_field(*shift), seed + k, density=0.03)
        a.append(fa)
        b.append(fb)
    return np.stack(a), np.stack(b)


def _stream(torch):
    return torch.cuda.current_stream().cuda_stream


CORR_CASES = [
    # (ss, n_fft, dtype, subpixel, normalize)
    (8, 1, "float32", "gaussian", True), (8, 2, "float32", "gaussian", True),
    (16, 1, "float32", "parabolic", False), (16, 2, "float32", "gaussian", True),
    (32, 2, "float32", "centroid", True), (64, 2, "float32", "gaussian", True),
    (128, 2, "float32", "gaussian", True), (16, 2, "float64", "gaussian", True),
    (32, 2, "float64", "parabolic", True), (64, 2, "float64", "gaussian", True),
    (8, 2, "float64", "gaussian", True), (32, 1, "float32", "gaussian", True),
]


@pytest.mark.parametrize("ss,n_fft,dtype,subpix,norm", CORR_CASES)
def test_correlation_matches_oracle(env, ss, n_fft, dtype, subpix, norm):
    torch, _lib, lib = env
    shape = (max(4 * ss, 96), max(5 * ss, 112))
    fa, fb = _frames(100 + ss, shape, n_pairs=2)
    g = _geom(_lib, lib, shape, ss, 0.5)
    N = po.fft_size(ss, n_fft)
    ft = np.float32 if dtype == "float32" else np.float64
    tdt = torch.float32 if dtype == "float32" else torch.float64
    da, db = torch.as_tensor(fa).cuda(), torch.as_tensor(fb).cuda()
    u = torch.empty((2, g.m, g.n), dtype=tdt, device="cuda")
    v = torch.empty_like(u)
    pi = torch.empty((2, g.m, g.n), dtype=torch.int32, device="cuda")
    pj = torch.empty_like(pi)
    _lib.check(lib.piv_correlate(ctypes.byref(g), 2, da.data_ptr(), db.data_ptr(), _lib.PIXEL["u8"],
                                 _lib.DTYPE[dtype], N, int(norm), _lib.SUBPIXEL[subpix], None, u.data_ptr(),
                                 v.data_ptr(), pi.data_ptr(), pj.data_ptr(), 0, 2, None, 0, _stream(torch)))
    field = po.Field(shape, ss, ss, 0.5, True, None, ft)
    for k in range(2):
        wa, wb = po.get_stack(fa[k].astype(ft), field), po.get_stack(fb[k].astype(ft), field)
        corr = po.correlate(wa, wb, N, norm, ft)
        i1, j1 = po.first_peak(corr)
        frag = po.fragile_windows(corr, i1, j1, subpix, ss)
        isp, jsp = po.subpixel(corr, i1, j1, subpix, ft)
        gi, gj = pi[k].cpu().numpy().ravel(), pj[k].cpu().numpy().ravel()
        mism = (gi != i1) | (gj != j1)
        assert not (mism & ~frag).any(), f"pair {k}: {int(mism.sum())} peaks differ"
        ok = ~mism & ~frag
        du = np.abs(u[k].cpu().numpy().ravel() - (jsp - N // 2))[ok]
        dv = np.abs(v[k].cpu().numpy().ravel() - (isp - N // 2))[ok]
        assert max(du.max(), dv.max()) < 1e-4, f"pair {k}: max displacement error {max(du.max(), dv.max()):.3e}"


@pytest.mark.parametrize("method", ["peak2peak", "peak2mean", "peak2energy"])
@pytest.mark.parametrize("n_fft", [1, 2])
def test_s2n_matches_oracle(env, method, n_fft):
    torch, _lib, lib = env
    shape, ss = (160, 192), 32
    fa, fb = _frames(7, shape)
    g = _geom(_lib, lib, shape, ss, 0.5)
    N = po.fft_size(ss, n_fft)
    da, db = torch.as_tensor(fa).cuda(), torch.as_tensor(fb).cuda()
    u = torch.empty((1, g.m, g.n), dtype=torch.float32, device="cuda")
    v, s2n = torch.empty_like(u), torch.empty_like(u)
    _lib.check(lib.piv_correlate(ctypes.byref(g), 1, da.data_ptr(), db.data_ptr(), _lib.PIXEL["u8"], 0, N, 1, 0,
                                 None, u.data_ptr(), v.data_ptr(), None, None, _lib.S2N[method], 2, s2n.data_ptr(),
                                 0, _stream(torch)))
    field = po.Field(shape, ss, ss, 0.5, True, None, np.float32)
    corr = po.correlate(po.get_stack(fa[0].astype(np.float32), field), po.get_stack(fb[0].astype(np.float32), field),
                        N, True, np.float32)
    i1, j1 = po.first_peak(corr)
    ref = po.s2n_ratio(corr, i1, j1, method, 2, np.float32)
    got = s2n.cpu().numpy().ravel()
    # peak2mean / peak2energy average the positive map values; with zero
    # padding (n_fft=2) the lag -ss row and column are zero in exact arithmetic
    # and hold rounding noise of either sign in any FFT, so the count of
    # positive values (and the ratio) differs by up to a few percent between
    # FFT implementations, the reference's own GPU and CPU paths included.
    rtol = 1e-4 if (method == "peak2peak" or n_fft == 1) else 5e-2
    np.testing.assert_allclose(got, ref, rtol=rtol)


def test_regrid_and_deform_bilinear_match_oracle(env):
    torch, _lib, lib = env
    shape = (200, 232)
    fa, fb = _frames(11, shape, n_pairs=2)
    g1 = _geom(_lib, lib, shape, 32, 0.5)
    g2 = _geom(_lib, lib, shape, 16, 0.5)
    rng = np.random.default_rng(3)
    up1 = rng.normal(0, 2, (2, g1.m, g1.n))
    vp1 = rng.normal(0, 2, (2, g1.m, g1.n))
    dup, dvp = torch.as_tensor(up1).cuda(), torch.as_tensor(vp1).cuda()
    up2 = torch.empty((2, g2.m, g2.n), dtype=torch.float64, device="cuda")
    vp2 = torch.empty_like(up2)
    _lib.check(lib.piv_regrid(ctypes.byref(g1), ctypes.byref(g2), 2, dup.data_ptr(), dvp.data_ptr(),
                              up2.data_ptr(), vp2.data_ptr(), _stream(torch)))
    f1 = po.Field(shape, 32, 32, 0.5, True, None, np.float32)
    f2 = po.Field(shape, 16, 16, 0.5, True, None, np.float32)
    for k in range(2):
        ref = po.grid_interp(f1.y_grid, f1.x_grid, up1[k], f2.y, f2.x)
        np.testing.assert_array_equal(up2[k].cpu().numpy(), ref)
    da, db = torch.as_tensor(fa).cuda(), torch.as_tensor(fb).cuda()
    for dp in (0.5, 1.0, 0.0, 0.3):
        oa = torch.empty((2,) + shape, dtype=torch.float32, device="cuda")
        ob = torch.empty_like(oa)
        _lib.check(lib.piv_deform(ctypes.byref(g2), 2, da.data_ptr(), db.data_ptr(), _lib.PIXEL["u8"],
                                  up2.data_ptr(), vp2.data_ptr(), dp, 1, None, None, None, 0, oa.data_ptr(),
                                  ob.data_ptr(), _stream(torch)))
        y, x = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
        x, y = x.astype(np.float32), y.astype(np.float32)
        for k in range(2):
            upx = po.grid_interp(f2.y_grid, f2.x_grid, up2[k].cpu().numpy(), y, x).astype(np.float32)
            vpx = po.grid_interp(f2.y_grid, f2.x_grid, vp2[k].cpu().numpy(), y, x).astype(np.float32)
            ra, rb = fa[k].astype(np.float32), fb[k].astype(np.float32)
            if 0 < dp < 1:
                ra = po.bilinear_frame(ra, x, y, upx, vpx, dp - 1)
                rb = po.bilinear_frame(rb, x, y, upx, vpx, dp)
            elif dp == 1:
                rb = po.bilinear_frame(rb, x, y, upx, vpx, 1)
            else:
                ra = po.bilinear_frame(ra, x, y, upx, vpx, -1)
            np.testing.assert_allclose(oa[k].cpu().numpy(), ra, atol=1e-2, rtol=1e-5)
            np.testing.assert_allclose(ob[k].cpu().numpy(), rb, atol=1e-2, rtol=1e-5)


def test_deform_cubic_matches_oracle(env):
    torch, _lib, lib = env
    import scipy.ndimage

    shape = (150, 170)
    fa, fb = _frames(12, shape, n_pairs=1)
    g = _geom(_lib, lib, shape, 16, 0.5)
    rng = np.random.default_rng(4)
    up = rng.normal(0, 3, (1, g.m, g.n))
    vp = rng.normal(0, 3, (1, g.m, g.n))
    da, db = torch.as_tensor(fa).cuda(), torch.as_tensor(fb).cuda()
    coef = torch.empty((2,) + shape, dtype=torch.float32, device="cuda")
    _lib.check(lib.piv_spline_prefilter(shape[0], shape[1], 1, da.data_ptr(), 0, coef[0].data_ptr(), _stream(torch)))
    _lib.check(lib.piv_spline_prefilter(shape[0], shape[1], 1, db.data_ptr(), 0, coef[1].data_ptr(), _stream(torch)))
    ref_c = scipy.ndimage.spline_filter(fa[0].astype(np.float64), order=3, mode="mirror")
    np.testing.assert_allclose(coef[0].cpu().numpy(), ref_c, atol=2e-3, rtol=1e-5)
    dup, dvp = torch.as_tensor(up).cuda(), torch.as_tensor(vp).cuda()
    oa = torch.empty((1,) + shape, dtype=torch.float32, device="cuda")
    ob = torch.empty_like(oa)
    _lib.check(lib.piv_deform(ctypes.byref(g), 1, da.data_ptr(), db.data_ptr(), 0, dup.data_ptr(), dvp.data_ptr(),
                              0.5, 3, coef[0].data_ptr(), coef[1].data_ptr(), None, 0, oa.data_ptr(), ob.data_ptr(),
                              _stream(torch)))
    f = po.Field(shape, 16, 16, 0.5, True, None, np.float32)
    y, x = np.meshgrid(np.arange(shape[0]), np.arange(shape[1]), indexing="ij")
    x, y = x.astype(np.float32), y.astype(np.float32)
    upx = po.grid_interp(f.y_grid, f.x_grid, up[0], y, x).astype(np.float32)
    vpx = po.grid_interp(f.y_grid, f.x_grid, vp[0], y, x).astype(np.float32)
    ra = po.cubic_frame(fa[0].astype(np.float32), x, y, upx, vpx, -0.5)
    rb = po.cubic_frame(fb[0].astype(np.float32), x, y, upx, vpx, 0.5)
    np.testing.assert_allclose(oa[0].cpu().numpy(), ra, atol=1e-2)
    np.testing.assert_allclose(ob[0].cpu().numpy(), rb, atol=1e-2)


@pytest.mark.parametrize("shape,pixel", [((7, 5), "u8"), ((1, 40), "f32"), ((13, 3), "u16"), ((70, 150), "f64"),
                                         ((33, 65), "u8")])
def test_spline_prefilter_matches_scipy(env, shape, pixel):
    """Prefilter against scipy's mirror-mode cubic spline_filter, frames smaller
    than the filter support and tiles that straddle the frame edge included."""
    torch, _lib, lib = env
    import scipy.ndimage

    rng = np.random.default_rng(sum(shape))
    dt = {"u8": np.uint8, "u16": np.uint16, "f32": np.float32, "f64": np.float64}[pixel]
    hi = {"u8": 255, "u16": 4000, "f32": 1.0, "f64": 50.0}[pixel]
    frames = (rng.random((2,) + shape) * hi).astype(dt)
    d = torch.as_tensor(frames).cuda()
    coef = torch.empty((2,) + shape, dtype=torch.float32, device="cuda")
    _lib.check(lib.piv_spline_prefilter(shape[0], shape[1], 2, d.data_ptr(), _lib.PIXEL[pixel],
                                        coef.data_ptr(), _stream(torch)))
    for k in range(2):
        ref = scipy.ndimage.spline_filter(frames[k].astype(np.float64), order=3, mode="mirror")
        np.testing.assert_allclose(coef[k].cpu().numpy(), ref, atol=2e-6 * hi, rtol=1e-5)


def _fields(seed, shape, n_out, fp32):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:shape[0], 0:shape[1]]
    u = 3 * np.sin(x / 5.0) + rng.normal(0, 0.2, shape)
    v = 2 * np.cos(y / 7.0) + rng.normal(0, 0.2, shape)
    idx = rng.choice(u.size, n_out, replace=False)
    u.ravel()[idx] += rng.normal(0, 6, n_out)
    v.ravel()[idx[: n_out // 2]] -= rng.normal(0, 6, n_out // 2)
    if fp32:
        u, v = u.astype(np.float32), v.astype(np.float32)
    return u, v


VAL_CASES = [
    dict(median_tol=2), dict(median_tol=1.0, mad_tol=3.0), dict(mean_tol=1.5), dict(rms_tol=2.0),
    dict(median_tol=0.8, size=2), dict(median_tol=1.2, mean_tol=2.0, mad_tol=2.5, size=1),
]


@pytest.mark.parametrize("fp32", [True, False])
@pytest.mark.parametrize("kw", VAL_CASES)
def test_validation_matches_oracle(env, kw, fp32):
    torch, _lib, lib = env
    shape = (23, 31)
    u, v = _fields(5, shape, 25, fp32)
    kw = dict(kw)
    size = kw.pop("size", 1)
    excl = np.zeros(shape, bool)
    excl[3:6, 4:9] = True
    for exclude in (None, excl):
        ref = po.validate([u, v], size=size, mask=exclude, **{**dict(median_tol=None), **kw})
        du, dv = torch.as_tensor(u.astype(np.float64)).cuda(), torch.as_tensor(v.astype(np.float64)).cuda()
        val = torch.empty(shape, dtype=torch.uint8, device="cuda")
        ex = torch.as_tensor(exclude.astype(np.uint8)).cuda() if exclude is not None else None
        t = lambda name: _lib.opt(kw.get(name))
        _lib.check(lib.piv_validate(shape[0], shape[1], 1, du.data_ptr(), dv.data_ptr(), None, 0, size, t("s2n_tol"),
                                    t("median_tol"), t("mad_tol"), t("mean_tol"), t("rms_tol"), None,
                                    ex.data_ptr() if ex is not None else None, int(fp32), val.data_ptr(),
                                    _stream(torch)))
        got = val.cpu().numpy().astype(bool)
        if "rms_tol" in kw:
            # global mean/std use a different summation order: allow points within rounding of the threshold
            f = [u, v]
            margin = [np.abs(np.abs(ff - np.nanmean(ff)) - kw["rms_tol"] * np.nanstd(ff)) for ff in f]
            near = (margin[0] < 1e-5) | (margin[1] < 1e-5)
            assert not ((got != ref) & ~near).any()
        else:
            np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("fp32", [True, False])
@pytest.mark.parametrize("method,n_iters,revalidate,size", [
    ("spring", 1, False, 1), ("spring", 2, True, 1), ("median", 1, False, 1), ("median", 3, False, 1),
    ("mean", 2, True, 1), ("median", 2, True, 2), ("spring", 1, False, 2), ("mean", 1, False, 1),
])
def test_replacement_matches_oracle(env, method, n_iters, revalidate, size, fp32):
    torch, _lib, lib = env
    shape = (19, 27)
    u, v = _fields(9, shape, 60, fp32)
    vkw = dict(size=1, s2n=None, s2n_tol=None, median_tol=1.0, mad_tol=None, mean_tol=None, rms_tol=None)
    val = po.validate([u, v], **vkw)
    ft = np.float32 if fp32 else np.float64
    (ru, rv), rval = po.replace_outliers([u.copy(), v.copy()], val.copy(), None, n_iters, method, size, revalidate,
                                         vkw, np.float32)
    du, dv = torch.as_tensor(u.astype(np.float64)).cuda(), torch.as_tensor(v.astype(np.float64)).cuda()
    dval = torch.as_tensor(val.astype(np.uint8)).cuda()
    nan = float("nan")
    _lib.check(lib.piv_replace(shape[0], shape[1], 1, du.data_ptr(), dv.data_ptr(), dval.data_ptr(), None, n_iters,
                               _lib.REPLACE[method], size, int(revalidate), None, 0, 1, nan, 1.0, nan, nan, nan,
                               int(fp32), 0, _stream(torch)))
    gu, gv = du.cpu().numpy(), dv.cpu().numpy()
    tol = 2e-4 if fp32 else 1e-6
    np.testing.assert_allclose(gu, ru.astype(np.float64), atol=tol)
    np.testing.assert_allclose(gv, rv.astype(np.float64), atol=tol)
    np.testing.assert_array_equal(dval.cpu().numpy().astype(bool), rval)
    assert ft  # float type of the reference fields


def test_replacement_all_outliers_gives_zero(env):
    torch, _lib, lib = env
    shape = (3, 4)
    u, v = _fields(1, shape, 0, False)
    du, dv = torch.as_tensor(u).cuda(), torch.as_tensor(v).cuda()
    dval = torch.ones(shape, dtype=torch.uint8, device="cuda")
    nan = float("nan")
    _lib.check(lib.piv_replace(3, 4, 1, du.data_ptr(), dv.data_ptr(), dval.data_ptr(), None, 1, 0, 1, 0, None, 0, 1,
                               nan, 0.3, nan, nan, nan, 0, 0, _stream(torch)))
    np.testing.assert_array_equal(du.cpu().numpy(), np.zeros(shape))


@pytest.mark.parametrize("shape", [(31, 31), (63, 63), (15, 23), (127, 127), (20, 32), (64, 90)])
@pytest.mark.parametrize("s", [0.8, None])
def test_smoothn_matches_oracle(env, shape, s):
    torch, _lib, lib = env
    u, v = _fields(13, shape, 0, False)
    tr = {}
    ref = po.smoothn([u, v], s=s, trace=tr)
    du, dv = torch.as_tensor(u).cuda(), torch.as_tensor(v).cuda()
    p = torch.empty(1, dtype=torch.float64, device="cuda")
    _lib.check(lib.piv_smoothn(shape[0], shape[1], 1, du.data_ptr(), dv.data_ptr(), None,
                               float("nan") if s is None else s, p.data_ptr(), _stream(torch)))
    tol = 1e-6 if s is not None else 1e-3
    np.testing.assert_allclose(du.cpu().numpy(), ref[0], atol=tol)
    np.testing.assert_allclose(dv.cpu().numpy(), ref[1], atol=tol)
    if s is None:
        assert abs(float(p.item()) - tr["p"]) < 1e-2


@pytest.mark.parametrize("shape,frac", [((31, 31), 0.05), ((24, 40), 0.2), ((11, 11), 0.12), ((63, 63), 0.08)])
@pytest.mark.parametrize("s", [0.8, None])
def test_weighted_smoothn_matches_oracle(env, shape, frac, s):
    """smoothn with a field mask (weighted iteration, nearest-neighbour fill of
    the masked NaNs, GCV with the w_mean <= 0.9 score for the larger masks)."""
    torch, _lib, lib = env
    u, v = _fields(17, shape, 0, False)
    y, x = np.mgrid[0:shape[0], 0:shape[1]]
    r2 = (x - 0.45 * shape[1]) ** 2 + (y - 0.55 * shape[0]) ** 2
    mask = r2 < frac * shape[0] * shape[1] / np.pi
    u[mask] = np.nan
    v[mask] = np.nan
    tr = {}
    ref = po.smoothn([u.copy(), v.copy()], mask=mask, s=s, trace=tr)
    du, dv = torch.as_tensor(u).cuda(), torch.as_tensor(v).cuda()
    dm = torch.as_tensor(mask.astype(np.uint8)).cuda()
    p = torch.empty(1, dtype=torch.float64, device="cuda")
    _lib.check(lib.piv_smoothn(shape[0], shape[1], 1, du.data_ptr(), dv.data_ptr(), dm.data_ptr(),
                               float("nan") if s is None else s, p.data_ptr(), _stream(torch)))
    tol = 1e-5 if s is not None else 1e-3
    np.testing.assert_allclose(du.cpu().numpy(), ref[0], atol=tol)
    np.testing.assert_allclose(dv.cpu().numpy(), ref[1], atol=tol)
    if s is None:
        assert abs(float(p.item()) - tr["p"]) < 2e-2


@pytest.mark.parametrize("ss,n_fft,dtype", [(8, 2, "float32"), (8, 1, "float32"), (16, 1, "float32"),
                                           (16, 2, "float32"), (32, 2, "float64"), (64, 2, "float32")])
def test_correlation_maps_match_oracle(env, ss, n_fft, dtype):
    torch, _lib, lib = env
    shape = (max(4 * ss, 96), max(5 * ss, 112))
    fa, fb = _frames(200 + ss, shape)
    g = _geom(_lib, lib, shape, ss, 0.5)
    N = po.fft_size(ss, n_fft)
    ft = np.float32 if dtype == "float32" else np.float64
    tdt = torch.float32 if dtype == "float32" else torch.float64
    da, db = torch.as_tensor(fa).cuda(), torch.as_tensor(fb).cuda()
    maps = torch.empty((1, g.m * g.n, N, N), dtype=tdt, device="cuda")
    _lib.check(lib.piv_correlate_maps(ctypes.byref(g), 1, da.data_ptr(), db.data_ptr(), 0, _lib.DTYPE[dtype], N, 1,
                                      None, maps.data_ptr(), 0, _stream(torch)))
    field = po.Field(shape, ss, ss, 0.5, True, None, ft)
    ref = po.correlate(po.get_stack(fa[0].astype(ft), field), po.get_stack(fb[0].astype(ft), field), N, True, ft)
    got = maps[0].cpu().numpy()
    scale = np.abs(ref).max(axis=(1, 2), keepdims=True)
    lag = np.arange(N) - N // 2
    no_overlap = (np.abs(lag)[:, None] >= ss) | (np.abs(lag)[None, :] >= ss)
    assert (got[:, no_overlap] == 0).all(), "lags without window overlap must be exact zeros"
    err = np.abs(got - ref) / scale
    worst = np.unravel_index(np.argmax(err), err.shape)
    assert err.max() < (1e-5 if dtype == "float32" else 1e-12), f"max rel err {err.max():.3e} at {worst}"


@pytest.mark.parametrize("method", ["spring", "median"])
def test_replacement_multi_pair_odd_field(env, method):
    """Several pairs whose field size is odd (per-pair scratch blocks must stay aligned)."""
    torch, _lib, lib = env
    shape = (31, 31)
    us, vs, vals, refs = [], [], [], []
    vkw = dict(size=1, s2n=None, s2n_tol=None, median_tol=1.0, mad_tol=None, mean_tol=None, rms_tol=None)
    for k in range(5):
        u, v = _fields(20 + k, shape, 40, False)
        val = po.validate([u, v], **vkw)
        (ru, rv), rval = po.replace_outliers([u.copy(), v.copy()], val.copy(), None, 2, method, 1, True, vkw,
                                             np.float32)
        us.append(u), vs.append(v), vals.append(val), refs.append((ru, rv, rval))
    du = torch.as_tensor(np.stack(us)).cuda()
    dv = torch.as_tensor(np.stack(vs)).cuda()
    dval = torch.as_tensor(np.stack(vals).astype(np.uint8)).cuda()
    nan = float("nan")
    _lib.check(lib.piv_replace(shape[0], shape[1], 5, du.data_ptr(), dv.data_ptr(), dval.data_ptr(), None, 2,
                               _lib.REPLACE[method], 1, 1, None, 0, 1, nan, 1.0, nan, nan, nan, 0, 0, _stream(torch)))
    for k, (ru, rv, rval) in enumerate(refs):
        np.testing.assert_allclose(du[k].cpu().numpy(), ru, atol=1e-6)
        np.testing.assert_allclose(dv[k].cpu().numpy(), rv, atol=1e-6)
        np.testing.assert_array_equal(dval[k].cpu().numpy().astype(bool), rval)


# (ss, subpixel, pixel type, frame shape). float frames with 16-byte aligned
# rows take the engine's asynchronous staging for ss 16/32, 8-bit ones for ss
# 64; the other combinations (and the 300-pixel width) load synchronously.
TC_CASES = [(16, "gaussian", "u8", (256, 288), "tensor"), (32, "gaussian", "f32", (256, 288), "tensor"),
            (16, "parabolic", "f32", (256, 288), "tensor"), (32, "centroid", "u8", (256, 300), "tensor"),
            (64, "gaussian", "u8", (256, 288), "tensor"), (64, "parabolic", "f32", (256, 288), "tensor"),
            (64, "gaussian", "u8", (256, 300), "tensor"),
            (16, "gaussian", "u8", (256, 288), "tensor_split"), (32, "gaussian", "f32", (256, 288), "tensor_split"),
            (16, "parabolic", "f32", (256, 300), "tensor_split"), (32, "centroid", "u8", (256, 300), "tensor_split"),
            (64, "gaussian", "u8", (256, 288), "tensor_split"),
            (16, "gaussian", "u8", (256, 288), "tensor_refined"), (32, "gaussian", "f32", (256, 288), "tensor_refined"),
            (64, "gaussian", "u8", (256, 288), "tensor_refined"), (64, "parabolic", "f32", (256, 300), "tensor_refined"),
            (16, "centroid", "u16", (256, 300), "tensor_refined"), (32, "parabolic", "u8", (256, 300), "tensor_refined")]

# Per engine: relative tie tolerance of the two largest map values, RMS and
# maximum displacement error (px) against the float64 oracle.
TC_TOL = {"tensor": (5e-3, 0.01, 0.1), "tensor_split": (1e-4, 1e-4, 2e-3),
          # refined: integer peaks from the fp16 maps (their tie resolution), fit values in float32
          "tensor_refined": (5e-3, 1e-4, 2e-3)}


@pytest.mark.parametrize("ss,subpix,pixel,shape,dft", TC_CASES)
def test_tensor_correlation_accuracy(env, ss, subpix, pixel, shape, dft):
    """tcgen05 engine against the float64 oracle. fp16 operands with fp32
    accumulation ("tensor"): displacement RMS within 0.01 px (the target
    accuracy of the tensor form), integer peaks equal except where the two
    largest map values are within fp16 resolution (relative 5e-3) or the
    window is fragile. hi/lo split operands ("tensor_split"): RMS within
    1e-4 px, ties within relative 1e-4. fp16 maps with the fit's five values
    recomputed in float32 ("tensor_refined", without the near-tie re-run of
    a plan): peaks as the fp16 form, RMS within 1e-4 px."""
    torch, _lib, lib = env
    tie_tol, rms_tol, max_tol = TC_TOL[dft]
    fa, fb = _frames(300 + ss, shape, n_pairs=3)
    g = _geom(_lib, lib, shape, ss, 0.5)
    N = 2 * ss
    dt = {"f32": np.float32, "u16": np.uint16}.get(pixel, np.uint8)
    da, db = torch.as_tensor(fa.astype(dt)).cuda(), torch.as_tensor(fb.astype(dt)).cuda()
    u = torch.empty((3, g.m, g.n), dtype=torch.float32, device="cuda")
    v = torch.empty_like(u)
    pi = torch.empty((3, g.m, g.n), dtype=torch.int32, device="cuda")
    pj = torch.empty_like(pi)
    _lib.check(lib.piv_correlate(ctypes.byref(g), 3, da.data_ptr(), db.data_ptr(), _lib.PIXEL[pixel], 0, N, 1,
                                 _lib.SUBPIXEL[subpix], None, u.data_ptr(), v.data_ptr(), pi.data_ptr(), pj.data_ptr(),
                                 0, 2, None, _lib.DFT[dft], _stream(torch)))
    field = po.Field(shape, ss, ss, 0.5, True, None, np.float64)
    errs, n_excl = [], 0
    for k in range(3):
        corr = po.correlate(po.get_stack(fa[k].astype(np.float64), field),
                            po.get_stack(fb[k].astype(np.float64), field), N, True, np.float64)
        i1, j1 = po.first_peak(corr)
        frag = po.fragile_windows(corr, i1, j1, subpix, ss, tie_tol=tie_tol)
        isp, jsp = po.subpixel(corr, i1, j1, subpix, np.float64)
        gi, gj = pi[k].cpu().numpy().ravel(), pj[k].cpu().numpy().ravel()
        mism = (gi != i1) | (gj != j1)
        assert not (mism & ~frag).any(), f"pair {k}: {int((mism & ~frag).sum())} integer peaks differ"
        ok = ~frag
        n_excl += int(frag.sum())
        du = u[k].cpu().numpy().ravel() - (jsp - N // 2)
        dv = v[k].cpu().numpy().ravel() - (isp - N // 2)
        errs.append(np.sqrt(du[ok] ** 2 + dv[ok] ** 2))
    e = np.concatenate(errs)
    rms = float(np.sqrt(np.mean(e ** 2)))
    print(f"{dft} ss={ss} {subpix} {pixel} {shape}: rms {rms:.2e} px, max {e.max():.2e} px, "
          f"excluded {n_excl}/{3 * g.m * g.n}")
    assert rms < rms_tol
    assert e.max() < max_tol


@pytest.mark.parametrize("ss,dft,tol", [(16, "tensor", 5e-3), (32, "tensor", 5e-3), (64, "tensor", 5e-3),
                                        (16, "tensor_split", 2e-5), (32, "tensor_split", 2e-5)])
def test_tensor_maps_match_oracle(env, ss, dft, tol):
    torch, _lib, lib = env
    shape = (192, 192) if ss == 64 else (160, 192)  # 25 windows for ss = 64: a partial last tile
    fa, fb = _frames(400 + ss, shape)
    g = _geom(_lib, lib, shape, ss, 0.5)
    N = 2 * ss
    da, db = torch.as_tensor(fa).cuda(), torch.as_tensor(fb).cuda()
    maps = torch.empty((1, g.m * g.n, N, N), dtype=torch.float32, device="cuda")
    field = po.Field(shape, ss, ss, 0.5, True, None, np.float64)
    ref = po.correlate(po.get_stack(fa[0].astype(np.float64), field), po.get_stack(fb[0].astype(np.float64), field),
                       N, True, np.float64)
    _lib.check(lib.piv_correlate_maps(ctypes.byref(g), 1, da.data_ptr(), db.data_ptr(), 0, 0, N, 1, None,
                                      maps.data_ptr(), _lib.DFT[dft], _stream(torch)))
    got = maps[0].cpu().numpy().astype(np.float64)
    lag = np.arange(N) - N // 2
    no_overlap = (np.abs(lag)[:, None] >= ss) | (np.abs(lag)[None, :] >= ss)
    ref[:, no_overlap] = 0
    scale = np.abs(ref).max(axis=(1, 2), keepdims=True)
    err = np.abs(got - ref) / scale
    print(f"{dft} maps ss={ss}: max rel err {err.max():.2e}, mean {err.mean():.2e}")
    assert (got[:, no_overlap] == 0).all()
    assert err.max() < tol


def test_tensor_pipeline_accuracy():
    """Three-pass run on the tensor engine: RMS vs the float64 oracle within
    0.01 px, and close to the float32 FFT engine."""
    import torch

    from openpiv_gpu import _build, synthetic
    from openpiv_gpu.gpu_process import PIVGPU
    from oracle.piv_oracle import OraclePIV

    _build.build()
    a, b, _, piv = synthetic.config_case(2, 3, shape=(512, 512))
    piv = dict(piv)
    mss = piv.pop("min_search_size")
    ut, vt = PIVGPU(a.shape, mss, **piv, dft="tensor")(a, b)
    us, vs = PIVGPU(a.shape, mss, **piv, dft="tensor_split")(a, b)
    ur, vr = PIVGPU(a.shape, mss, **piv, dft="tensor_refined")(a, b)
    uf, vf = PIVGPU(a.shape, mss, **piv, dft="fft")(a, b)
    piv64 = dict(piv)
    piv64["dtype_f"] = "float64"
    u64, v64 = OraclePIV(a.shape, mss, **piv64)(a, b)
    ut, vt, us, vs, uf, vf, ur, vr = (x.cpu().numpy() for x in (ut, vt, us, vs, uf, vf, ur, vr))
    rms_r = float(np.sqrt(np.mean((ur - u64) ** 2 + (vr - v64) ** 2)))
    max_rf = float(max(np.abs(ur - uf).max(), np.abs(vr - vf).max()))
    rms_t = float(np.sqrt(np.mean((ut - u64) ** 2 + (vt - v64) ** 2)))
    rms_s = float(np.sqrt(np.mean((us - u64) ** 2 + (vs - v64) ** 2)))
    rms_f = float(np.sqrt(np.mean((uf - u64) ** 2 + (vf - v64) ** 2)))
    print(f"pipeline rms vs float64 oracle: tensor {rms_t:.2e} px, tensor_split {rms_s:.2e} px, "
          f"tensor_refined {rms_r:.2e} px (max {max_rf:.1e} px from fft), fft {rms_f:.2e} px")
    assert rms_t < 0.01
    assert rms_r < 1e-4
    assert max_rf < 1e-3
    assert rms_s < 1e-4
    assert rms_f < 1e-4


def test_bounded_wait_gives_up_and_leaves_the_context_usable(env):
    """A tensor-core completion wait that nothing completes gives up after its
    poll limit and reports PIV_E_TIMEOUT through the status word (no trap, no
    hang); a correlation on the same context afterwards is still exact."""
    torch, _lib, lib = env
    st = ctypes.c_int(0)
    _lib.check(lib.piv_selftest_bounded_wait(2000, ctypes.byref(st), _stream(torch)))
    assert st.value == _lib.PIV_E_TIMEOUT
    test_tensor_maps_match_oracle(env, 16, "tensor", 5e-3)
