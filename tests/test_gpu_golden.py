"""GPU parity against the reference's own outputs (tests/golden/*.npz).

Every case runs through the public API (piv_gpu -> PIVGPU -> C ABI plan) on
the GPU and is compared stage by stage with the reference run captured in the
fixture:

* integer correlation peaks: identical;
* subpixel displacements of every pass and the final field: within 1e-3 px;
* validation masks (initial outliers of every pass, final val_locations and
  outliers): identical.

Windows the oracle flags as fragile (a near tie of the two largest map values,
or a Gaussian-fit stencil that touches a lag without window overlap, whose
exact value is zero and whose computed value is FFT rounding noise) are
excluded and counted; their 3x3 neighbourhoods are excluded from the mask
comparison of the same pass. A fragile window that changes the result of a
non-final pass makes the later passes incomparable, and the case is skipped
from there with a message.
"""

import numpy as np
import pytest

import make_golden as mg
from openpiv_gpu import synthetic as syn

pytestmark = pytest.mark.gpu

TOL_PX = 1e-3       # displacement tolerance vs the reference path
NEAR_TIE = 1e-5     # relative gap of the two largest correlation values
CASES = mg.cases()


@pytest.fixture(scope="module")
def api():
    import torch

    from openpiv_gpu import _build

    _build.build()
    torch.cuda.set_device(0)
    from openpiv_gpu import gpu_process

    return gpu_process


def _load(name, cfg, shape, pair_index, overrides, store):
    g = np.load(f"{mg.HERE}/{name}.npz")
    if store:
        a, b = g["frame_a"], g["frame_b"]
        _, _, _, piv = mg.build_case(syn, cfg, a.shape, pair_index, overrides)
    else:
        a, b, _, piv = mg.build_case(syn, cfg, shape, pair_index, overrides)
        if mg._digest(a) != str(g["sha_a"]) or mg._digest(b) != str(g["sha_b"]):
            pytest.skip("synthetic generator output differs from the fixture's frames on this NumPy")
    return g, a, b, piv


def _close(a, b, tol):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    nan_a, nan_b = np.isnan(a), np.isnan(b)
    assert (nan_a == nan_b).all(), "NaN pattern differs"
    d = np.abs(a - b)[~nan_a]
    return float(d.max()) if d.size else 0.0


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_pipeline_matches_reference(api, case):
    from oracle.piv_oracle import OraclePIV

    name = case[0]
    g, a, b, piv = _load(*case)
    mss = piv.pop("min_search_size")
    proc = api.piv_gpu(a.shape, mss, **piv)
    u, v = proc(a, b)
    stages = proc.gpu_process.iteration_outputs()
    oracle = OraclePIV(a.shape, mss, **piv)
    oracle(a, b)
    assert len(stages) == int(g["n_iters"])
    report = []
    last = len(stages) - 1
    affected = None
    for k, st in enumerate(stages):
        m, n = st["u_corr"].shape
        gi, gj = g[f"it{k}_i_peak"].ravel(), g[f"it{k}_j_peak"].ravel()
        pi, pj = st["i_peak"], st["j_peak"]
        sel = np.ones(m * n, bool)
        if oracle.fields[k].field_mask is not None:  # the reference keeps unmasked windows only
            sel = ~oracle.fields[k].field_mask.ravel()
            pi, pj = pi[sel], pj[sel]
        frag = oracle.trace[k]["fragile"]
        mism = (pi != gi) | (pj != gj)
        assert not (mism & ~frag).any(), f"it{k}: {int((mism & ~frag).sum())} integer peaks differ"
        frag_full = np.zeros(m * n, bool)
        frag_full[sel] = frag
        frag_full = frag_full.reshape(m, n)
        du = np.abs(st["u_corr"].astype(np.float64) - g[f"it{k}_u_corr"])
        dv = np.abs(st["v_corr"].astype(np.float64) - g[f"it{k}_v_corr"])
        bad = np.nan_to_num(np.maximum(du, dv), nan=0.0) > TOL_PX
        assert not (bad & ~frag_full).any(), \
            f"it{k} correlation displacement differs by {np.nanmax(np.where(frag_full, 0, np.maximum(du, dv))):.3e} px"
        ok = ~frag_full & ~np.isnan(du)
        report.append(f"it{k} corr {float(np.max(np.maximum(du, dv)[ok], initial=0)):.1e} fragile {int(frag.sum())}")
        affected = bad
        if bad.any():
            grow = np.zeros_like(bad)
            s_ = int(piv.get("validation_size", 1))
            for a_ in range(-s_, s_ + 1):
                for b_ in range(-s_, s_ + 1):
                    grow |= np.roll(np.roll(bad, a_, 0), b_, 1)
            affected = grow
        keep = ~affected
        np.testing.assert_array_equal(st["val0"][keep], g[f"it{k}_val0"][keep], err_msg=f"it{k} validation mask")
        if bad.any() and k < last:
            print(name, "; ".join(report))
            pytest.skip(f"{int(bad.sum())} fragile window(s) changed iteration {k}; later passes not comparable")
        if f"it{k}_u_smooth" in g:
            ds = max(_close(st["u_out"], g[f"it{k}_u_smooth"], TOL_PX), _close(st["v_out"], g[f"it{k}_v_smooth"], TOL_PX))
            report.append(f"smooth {ds:.1e} p {st['p']:.6f}/{np.log10(float(g[f'it{k}_smooth_s'])):.6f}")
            assert ds <= TOL_PX, f"it{k} smoothed field differs by {ds:.3e} px"
        if f"it{k}_s2n" in g:
            s_gpu, s_ref = st["s2n"], g[f"it{k}_s2n"]
            fin = np.isfinite(s_ref)
            np.testing.assert_array_equal(np.isfinite(s_gpu), fin)
            # peak2mean/peak2energy count the positive map values; the lag -ss row
            # and column are zero in exact arithmetic and carry rounding noise of
            # either sign in an FFT (see test_gpu_stages.test_s2n_matches_oracle).
            rtol = 1e-4 if piv.get("s2n_method", "peak2peak") == "peak2peak" or piv.get("n_fft", 2) == 1 else 5e-2
            np.testing.assert_allclose(s_gpu[fin], s_ref[fin], rtol=rtol)
    assert u.dtype == g["u"].dtype
    keep = ~affected
    dfin = max(_close(u[keep], g["u"][keep], TOL_PX), _close(v[keep], g["v"][keep], TOL_PX))
    report.append(f"final {dfin:.1e}")
    print(name, "; ".join(report))
    assert dfin <= TOL_PX, f"final field differs by {dfin:.3e} px"
    np.testing.assert_array_equal(proc.val_locations[keep], g["val_locations"][keep])
    np.testing.assert_array_equal(proc.outliers[keep], g["outliers"][keep])
    x, y = proc.coords
    np.testing.assert_array_equal(x, g["x"])
    np.testing.assert_array_equal(y, g["y"])
