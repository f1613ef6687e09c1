"""Host-side checks that need no GPU: the C ABI library loads and exports every
declared function, geometry and per-iteration settings agree with the oracle,
and argument checks follow the reference's assertions."""

import ctypes

import numpy as np
import pytest

from openpiv_gpu import _build, _lib
from openpiv_gpu import gpu_process as gp
from oracle import piv_oracle as po


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load()


def test_library_exports_every_header_function(lib):
    names = _lib.header_functions()
    assert len(names) >= 16
    so = ctypes.CDLL(_build.LIB_PATH)
    missing = [n for n in names if not hasattr(so, n)]
    assert not missing, missing
    assert set(_lib._SIGNATURES) == set(names)


@pytest.mark.parametrize("shape", [(512, 512), (150, 170), (1024, 768), (97, 203), (2048, 2048)])
@pytest.mark.parametrize("ss,ov", [(16, 0.5), (32, 0.5), (16, 0.75), (64, 0.0), (8, 0.5), (24, 0.3)])
@pytest.mark.parametrize("center", [True, False])
def test_geometry_matches_oracle(lib, shape, ss, ov, center):
    if min(shape) < ss:
        pytest.skip("frame smaller than window")
    g = _lib.PivGeometry()
    _lib.check(lib.piv_field_geometry(shape[0], shape[1], ss, ss, ov, int(center), ctypes.byref(g)))
    f = po.Field(shape, ss, ss, ov, center, None, np.float32)
    assert (g.m, g.n) == f.field_shape
    assert (g.x_offset, g.y_offset) == (f.x_offset, f.y_offset)
    assert g.spacing == f.spacing


def test_geometry_rejects_bad_args(lib):
    g = _lib.PivGeometry()
    assert lib.piv_field_geometry(10, 10, 16, 16, 0.5, 1, ctypes.byref(g)) == _lib.PIV_E_ARG
    assert "smaller" in _lib.last_error()
    assert lib.piv_field_geometry(64, 64, 16, 16, 1.0, 1, ctypes.byref(g)) == _lib.PIV_E_ARG


def _correlate_args(geom, n_pairs):
    # Device pointers are never dereferenced: the geometry check returns first.
    dev = ctypes.c_void_p(256)
    return (ctypes.byref(geom), n_pairs, dev, dev, _lib.PIXEL["f32"], _lib.DTYPE["float32"], 16, 1,
            _lib.SUBPIXEL["gaussian"], None, dev, dev, None, None, 0, 2, None, _lib.DFT["fft"], None)


def test_correlation_refuses_windows_outside_the_frame(lib):
    """The correlation kernels read window rows without per-pixel frame
    checks, so the ABI refuses, before anything runs, a geometry whose search
    windows pass the frame's edge: the centred grid of an odd search size with
    no spare pixel (the reference would stack pixels it never wrote),
    hand-made fields larger than the frame, and negative pair counts."""
    g = _lib.PivGeometry()
    _lib.check(lib.piv_field_geometry(63, 63, 9, 9, 0.0, 1, ctypes.byref(g)))
    # Seven windows 9 px apart from column 1: the last one covers columns 55..63.
    assert (g.n, g.spacing, g.x_offset) == (7, 9, 1)
    assert lib.piv_correlate(*_correlate_args(g, 1)) == _lib.PIV_E_UNSUPPORTED
    assert "outside" in _lib.last_error()
    dev = ctypes.c_void_p(256)
    assert lib.piv_correlate_maps(ctypes.byref(g), 1, dev, dev, _lib.PIXEL["f32"], _lib.DTYPE["float32"], 16, 1,
                                  None, dev, _lib.DFT["fft"], None) == _lib.PIV_E_UNSUPPORTED

    ok = _lib.PivGeometry()
    _lib.check(lib.piv_field_geometry(64, 64, 16, 16, 0.5, 1, ctypes.byref(ok)))
    big = _lib.PivGeometry.from_buffer_copy(ok)
    big.m += 1
    assert lib.piv_correlate(*_correlate_args(big, 1)) == _lib.PIV_E_UNSUPPORTED
    bad = _lib.PivGeometry.from_buffer_copy(ok)
    bad.spacing = 0
    assert lib.piv_correlate(*_correlate_args(bad, 1)) == _lib.PIV_E_ARG
    assert lib.piv_correlate(*_correlate_args(ok, -1)) == _lib.PIV_E_ARG
    assert "negative" in _lib.last_error()


def test_plan_refuses_windows_outside_the_frame(lib):
    it = _lib.PivIteration(search_size=9, window_size=9, overlap_ratio=0.0, fft_size=16, deforming_order=1,
                           deforming_par=0.5, normalize=1, subpixel_method=_lib.SUBPIXEL["gaussian"],
                           validation_size=1, median_tol=2.0, num_replacing_iters=2, replacing_size=1,
                           smoothing_par=0.5)
    its = (_lib.PivIteration * 1)(it)
    cfg = _lib.PivConfig(height=63, width=63, n_iters=1, iters=its, center=1, dt=1.0, scaling_par=1.0,
                         dtype=_lib.DTYPE["float32"], pixel_type=_lib.PIXEL["f32"], max_pairs=1,
                         dft_mode=_lib.DFT["fft"])
    plan = ctypes.c_void_p()
    assert lib.piv_plan_create(ctypes.byref(cfg), ctypes.byref(plan)) == _lib.PIV_E_UNSUPPORTED
    assert "outside" in _lib.last_error() and not plan.value


@pytest.mark.parametrize("kw", [
    dict(search_size_iters=(1, 2, 2), overlap_ratio=(0.5, 0.5, 0.75), n_fft=(2, 1, 3)),
    dict(search_size_iters=(2, 1), deforming_order=(1, 3), median_tol=(2, None), smoothing_par=0.5),
    dict(search_size_iters=1, subpixel_method="centroid", s2n_tol=1.5, s2n_method="peak2mean"),
    dict(search_size_iters=(1, 1), shrink_ratio=0.5, replacing_method="median", revalidate=(True, False)),
])
def test_iteration_settings_match_oracle(lib, kw):
    proc = gp.PIVGPU((512, 512), 16, **kw)
    _, iters = po.expand_settings(16, **kw)
    assert len(proc._iterations) == len(iters)
    for k, (c, o) in enumerate(zip(proc._iterations, iters)):
        assert c.search_size == o["search_size"]
        assert c.fft_size == po.fft_size(o["search_size"], o["n_fft"])
        assert c.subpixel_method == _lib.SUBPIXEL[o["subpixel_method"]]
        assert c.deforming_order == o["deforming_order"]
        for name in ("median_tol", "s2n_tol", "mad_tol", "mean_tol", "rms_tol", "smoothing_par"):
            want = o[name]
            got = getattr(c, name)
            assert (np.isnan(got) and want is None) or got == want, (k, name)
        f = proc.piv_fields[k]
        of = po.Field((512, 512), f.window_size, f.search_size, o["overlap_ratio"], True, None, np.float32)
        assert f.field_shape == of.field_shape
        np.testing.assert_array_equal(f.x, of.x)
        np.testing.assert_array_equal(f.y, of.y)


@pytest.mark.parametrize("bad", [
    dict(min_search_size=7),
    dict(search_size_iters=(1, 0)),
    dict(overlap_ratio=1.5),
    dict(subpixel_method="quadratic"),
    dict(s2n_method="peak2x"),
    dict(replacing_method="spline"),
    dict(deforming_par=1.5),
    dict(smoothing_par=-1.0),
    dict(num_replacing_iters=-1),
    dict(mask=np.zeros((10, 10), bool)),
])
def test_argument_checks_raise_assertion(lib, bad):
    kw = dict(bad)
    mss = kw.pop("min_search_size", 16)
    with pytest.raises(AssertionError):
        gp.piv_gpu((256, 256), mss, **kw)


def test_frame_shape_check(lib):
    with pytest.raises(AssertionError, match="frame_shape"):
        gp.piv_gpu((32, 256), 16, search_size_iters=(1, 1, 1))


def test_aliases(lib):
    p = gp.piv_gpu((256, 256), min_window_size=16, window_size_iters=(1, 1))
    assert p.search_size_iters == (1, 1)
    assert p.gpu_process.piv_fields[0].search_size == 32
    assert p.field_shape == (31, 31)


def test_frame_check_on_call(lib):
    p = gp.piv_gpu((64, 64), 16)
    with pytest.raises(AssertionError, match="Both frames"):
        p(np.zeros((64, 63)), np.zeros((64, 64)))
