"""Checked build of the library (-DPIV_BOUNDS_CHECK): every shared-memory
store, asynchronous copy, TMEM load, window read and result write of the
tensor-core correlation and peak-refinement kernels is checked against its
buffer; a failed check skips the access and is counted (piv_bounds_check).

The tensor forms run through the checked build on small cases (three-pass
pipelines of several golden shapes, including a field mask and 75% overlap,
and single correlation passes of three pairs whose window counts leave a
partial last tile): no violation may be
counted, and the results must equal the normal build's bit for bit.
"""

import ctypes

import numpy as np
import pytest

import make_golden as mg
from openpiv_gpu import synthetic as syn

pytestmark = pytest.mark.gpu

CASES = ["cfg2_256", "overlap_075", "masked64", "multi_iter", "not_centered"]
FORMS = ["tensor", "tensor_split", "tensor_refined"]


@pytest.fixture(scope="module")
def libs():
    import torch

    from openpiv_gpu import _build, _lib

    _build.build()
    _build.build(checked=True)
    torch.cuda.set_device(0)
    normal = _lib.load()
    checked = _lib.load_checked()
    flag, count = ctypes.c_int(0), ctypes.c_int(0)
    _lib.check(checked.piv_bounds_check(ctypes.byref(flag), ctypes.byref(count)))
    assert flag.value == 1, "the checked library was built without its checks"
    _lib.check(normal.piv_bounds_check(ctypes.byref(flag), ctypes.byref(count)))
    assert flag.value == 0 and count.value == 0
    return torch, _lib, normal, checked


def _chk(lib, rc):
    """Raises with the message of the library that failed (each library keeps its own)."""
    if rc != 0:
        buf = ctypes.create_string_buffer(512)
        lib.piv_last_error(buf, 512)
        raise RuntimeError(f"[{rc}] {buf.value.decode(errors='replace')}")


def _violations(_lib, checked):
    flag, count = ctypes.c_int(0), ctypes.c_int(0)
    _lib.check(checked.piv_bounds_check(ctypes.byref(flag), ctypes.byref(count)))
    return count.value


def _run_plan(torch, _lib, lib, proc, a, b):
    cfg, keep = proc._config(_lib.PIXEL["u8"], 1)
    plan = ctypes.c_void_p()
    _chk(lib, lib.piv_plan_create(ctypes.byref(cfg), ctypes.byref(plan)))
    try:
        fa = torch.as_tensor(a[None]).cuda()
        fb = torch.as_tensor(b[None]).cuda()
        m, n = proc.piv_fields[-1].field_shape
        u = torch.empty((1, m, n), dtype=torch.float64, device="cuda")
        v = torch.empty_like(u)
        _chk(lib, lib.piv_plan_run(plan, 1, fa.data_ptr(), fb.data_ptr(), 0, u.data_ptr(), v.data_ptr(), None,
                                    None, 0, torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        return u.cpu().numpy(), v.cpu().numpy()
    finally:
        lib.piv_plan_destroy(plan)


@pytest.mark.parametrize("dft", FORMS)
@pytest.mark.parametrize("name", CASES)
def test_pipeline_in_bounds(libs, name, dft):
    from openpiv_gpu.gpu_process import PIVGPU

    torch, _lib, normal, checked = libs
    case = [c for c in mg.cases() if c[0] == name][0]
    g = np.load(f"{mg.HERE}/{name}.npz")
    a, b = g["frame_a"], g["frame_b"]
    _, _, _, piv = mg.build_case(syn, case[1], a.shape, case[3], case[4])
    mss = piv.pop("min_search_size")
    proc = PIVGPU(a.shape, mss, dft=dft, **piv)
    assert _violations(_lib, checked) >= 0  # reset
    uc, vc = _run_plan(torch, _lib, checked, proc, a, b)
    assert _violations(_lib, checked) == 0, "out-of-bounds accesses counted"
    un, vn = _run_plan(torch, _lib, normal, proc, a, b)
    np.testing.assert_array_equal(uc, un)
    np.testing.assert_array_equal(vc, vn)


@pytest.mark.parametrize("dft", FORMS)
@pytest.mark.parametrize("ss,pixel,shape", [(16, "f32", (128, 144)), (32, "u8", (160, 160)), (64, "u8", (192, 192)),
                                            (64, "f32", (192, 256))])
def test_correlation_in_bounds(libs, ss, pixel, shape, dft):
    torch, _lib, normal, checked = libs
    rng = np.random.default_rng(ss)
    fa = rng.integers(0, 256, (3,) + shape).astype(np.float32 if pixel == "f32" else np.uint8)
    fb = np.roll(fa, (2, -1), axis=(1, 2))
    da, db = torch.as_tensor(fa).cuda(), torch.as_tensor(fb).cuda()
    out = []
    for lib in (checked, normal):
        g = _lib.PivGeometry()
        _chk(lib, lib.piv_field_geometry(shape[0], shape[1], ss, ss, 0.5, 1, ctypes.byref(g)))
        u = torch.empty((3, g.m, g.n), dtype=torch.float32, device="cuda")
        v = torch.empty_like(u)
        _chk(lib, lib.piv_correlate(ctypes.byref(g), 3, da.data_ptr(), db.data_ptr(), _lib.PIXEL[pixel], 0, 2 * ss,
                                     1, 0, None, u.data_ptr(), v.data_ptr(), None, None, 0, 2, None, _lib.DFT[dft],
                                     torch.cuda.current_stream().cuda_stream))
        torch.cuda.synchronize()
        out.append((u.cpu().numpy(), v.cpu().numpy()))
    assert _violations(_lib, checked) == 0, "out-of-bounds accesses counted"
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
