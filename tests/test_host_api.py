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
