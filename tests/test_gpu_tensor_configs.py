"""The tensor forms across pipeline configurations the accuracy tests do not
cover: a frame mask, 75% overlap, a non-square frame, 16-bit frames, an
uncentred grid. Each run is compared with the float64 oracle (RMS over the
finite vectors within 0.01 px for the fp16 form, 1e-4 px for the hi/lo split
form, NaN / zero placement equal); float64 fields, which the tensor engines do
not serve, must give the FFT engine's result bit for bit."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _case(name):
    from openpiv_gpu import synthetic

    a, b, _, piv = synthetic.config_case(2, 5, shape=(256, 320) if name == "nonsquare" else (256, 256))
    piv = dict(piv)
    if name == "mask":
        yy, xx = np.mgrid[:a.shape[0], :a.shape[1]]
        piv["mask"] = ((yy - 128) ** 2 + (xx - 100) ** 2) < 40 ** 2
    elif name == "overlap75":
        piv["overlap_ratio"] = 0.75
    elif name == "u16":
        a, b = (x.astype(np.uint16) * 200 for x in (a, b))
    elif name == "uncentred":
        piv["center"] = False
    return a, b, piv


@pytest.mark.parametrize("dft,tol", [("tensor", 0.01), ("tensor_split", 1e-4), ("tensor_refined", 1e-4)])
@pytest.mark.parametrize("name", ["mask", "overlap75", "nonsquare", "u16", "uncentred"])
def test_tensor_forms_match_oracle(name, dft, tol):
    from openpiv_gpu import _build
    from openpiv_gpu.gpu_process import PIVGPU
    from oracle.piv_oracle import OraclePIV

    _build.build()
    a, b, piv = _case(name)
    mss = piv.pop("min_search_size")
    ug, vg = PIVGPU(a.shape, mss, **piv, dft=dft)(a, b)
    ug, vg = ug.cpu().numpy(), vg.cpu().numpy()
    piv64 = dict(piv)
    piv64["dtype_f"] = "float64"
    u64, v64 = OraclePIV(a.shape, mss, **piv64)(a, b)
    assert ug.shape == u64.shape
    np.testing.assert_array_equal(np.isnan(ug), np.isnan(u64))
    fin = np.isfinite(u64) & np.isfinite(v64)
    rms = float(np.sqrt(np.mean((ug[fin] - u64[fin]) ** 2 + (vg[fin] - v64[fin]) ** 2)))
    print(f"{name} {dft}: rms {rms:.2e} px over {int(fin.sum())} vectors")
    assert rms < tol


def test_float64_fields_fall_back_to_the_fft_engine():
    from openpiv_gpu import _build
    from openpiv_gpu.gpu_process import PIVGPU

    _build.build()
    a, b, piv = _case("overlap75")
    piv["dtype_f"] = "float64"
    mss = piv.pop("min_search_size")
    ut, vt = PIVGPU(a.shape, mss, **piv, dft="tensor")(a, b)
    uf, vf = PIVGPU(a.shape, mss, **piv, dft="fft")(a, b)
    np.testing.assert_array_equal(ut.cpu().numpy(), uf.cpu().numpy())
    np.testing.assert_array_equal(vt.cpu().numpy(), vf.cpu().numpy())
