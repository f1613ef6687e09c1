"""GPU parity against the reference's own outputs (tests/golden/*.npz).

Every case runs through the public API (piv_gpu -> PIVGPU -> C ABI plan) on
the GPU, once per correlation engine ("fft": float32/float64 FFT; "tensor_split":
tcgen05 DFTs on fp16 hi/lo operand pairs; "tensor_refined": tcgen05 DFTs on fp16
operands for the integer peaks, the fit's five values in float32, near ties
correlated again by the float32 FFT; "tensor": tcgen05 DFTs on fp16 operands),
and is compared stage by stage with the reference run captured in the fixture.

The FFT, split and refined forms are held to the reference-parity bar:

* integer correlation peaks: identical, except near ties;
* subpixel displacements of every pass and of the final field: within 1e-3 px;
* validation masks (initial outliers of every pass, final val_locations and
  outliers): identical.

Near ties are counted and printed. A window is excused when the product flags
it (its two largest map values are within the engine's own map accuracy,
piv_plan_near_ties), when the reference's own map has its two largest values
within NEAR_TIE of each other, or when a Gaussian-fit stencil touches a lag
without window overlap (exact value zero, computed value rounding noise of
either sign). An excused window that changes a non-final pass makes the later
passes incomparable, and the case is skipped from there with a message.

The fp16 tensor form trades accuracy for speed (about 1e-4 px per window): its
pass-0 peaks must equal the reference's except near ties, and the deviating
windows (beyond 1e-3 px) and validation-mask flips are counted, printed and
bounded.
"""

import numpy as np
import pytest

import make_golden as mg
from openpiv_gpu import synthetic as syn

pytestmark = pytest.mark.gpu

TOL_PX = 1e-3           # displacement tolerance vs the reference path
NEAR_TIE = 2.0 ** -20   # reference-side near tie: relative gap of its two largest map values (8 float32 ulps)
CASES = mg.cases()
DFTS = ("fft", "tensor_split", "tensor_refined", "tensor")
# fp16 tensor form: bounds of what deviates from the reference.
F16_PASS0_MAX_PX = 0.02     # pass-0 displacement, outside near ties
F16_FINAL_RMS_PX = 0.01     # final field RMS over the windows that kept the reference's peak
F16_PEAK_JUMP_PX = 0.1      # a final vector further off took another correlation peak
F16_MAX_FLIP_FRAC = 0.01    # validation-mask flips per pass and final peak jumps, fraction of the windows


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


def _grow(bad, size):
    grow = np.zeros_like(bad)
    for a_ in range(-size, size + 1):
        for b_ in range(-size, size + 1):
            grow |= np.roll(np.roll(bad, a_, 0), b_, 1)
    return grow


def _run(api, case, dft):
    from oracle.piv_oracle import OraclePIV

    g, a, b, piv = _load(*case)
    mss = piv.pop("min_search_size")
    proc = api.piv_gpu(a.shape, mss, dft=dft, **piv)
    u, v = proc(a, b)
    stages = proc.gpu_process.iteration_outputs()
    ties = proc.gpu_process.near_ties()
    oracle = OraclePIV(a.shape, mss, **piv)
    oracle(a, b)
    assert len(stages) == int(g["n_iters"])
    return g, piv, proc, u, v, stages, ties, oracle


def _pass_peaks(g, k, st, oracle):
    """Peak mismatches, product near ties and the excused set of pass k (over
    the windows the reference correlates)."""
    m, n = st["u_corr"].shape
    gi, gj = g[f"it{k}_i_peak"].ravel(), g[f"it{k}_j_peak"].ravel()
    pi, pj, tie = st["i_peak"], st["j_peak"], st["near_tie"].ravel()
    sel = np.ones(m * n, bool)
    if oracle.fields[k].field_mask is not None:  # the reference keeps unmasked windows only
        sel = ~oracle.fields[k].field_mask.ravel()
        pi, pj, tie = pi[sel], pj[sel], tie[sel]
    tr = oracle.trace[k]
    ref_tie = tr["peak_gap"] < NEAR_TIE
    excused = tie | ref_tie | tr["stencil"]
    mism = (pi != gi) | (pj != gj)
    full = np.zeros(m * n, bool)
    full[sel] = excused
    return mism, tie, ref_tie, excused, full.reshape(m, n)


@pytest.mark.parametrize("dft", DFTS)
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_pipeline_matches_reference(api, case, dft):
    name = case[0]
    g, piv, proc, u, v, stages, ties, oracle = _run(api, case, dft)
    if dft == "tensor":
        return _tensor_report(name, g, piv, proc, u, v, stages, ties, oracle)
    report = [f"[{dft}]"]
    last = len(stages) - 1
    affected = None
    for k, st in enumerate(stages):
        mism, tie, ref_tie, excused, exc_full = _pass_peaks(g, k, st, oracle)
        assert int(st["near_tie"].sum()) == ties[k], "near-tie flags and count disagree"
        assert not (mism & ~excused).any(), f"it{k}: {int((mism & ~excused).sum())} integer peaks differ"
        du = np.abs(st["u_corr"].astype(np.float64) - g[f"it{k}_u_corr"])
        dv = np.abs(st["v_corr"].astype(np.float64) - g[f"it{k}_v_corr"])
        bad = np.nan_to_num(np.maximum(du, dv), nan=0.0) > TOL_PX
        assert not (bad & ~exc_full).any(), \
            f"it{k} correlation displacement differs by {np.nanmax(np.where(exc_full, 0, np.maximum(du, dv))):.3e} px"
        ok = ~exc_full & ~np.isnan(du)
        report.append(f"it{k} corr {float(np.max(np.maximum(du, dv)[ok], initial=0)):.1e} near-ties {ties[k]} "
                      f"(ref {int(ref_tie.sum())}, stencil {int(oracle.trace[k]['stencil'].sum())}, "
                      f"peaks differing {int(mism.sum())})")
        affected = _grow(bad, int(piv.get("validation_size", 1))) if bad.any() else bad
        keep = ~affected
        np.testing.assert_array_equal(st["val0"][keep], g[f"it{k}_val0"][keep], err_msg=f"it{k} validation mask")
        if bad.any() and k < last:
            print(name, "; ".join(report))
            pytest.skip(f"{int(bad.sum())} near-tie window(s) changed iteration {k}; later passes not comparable")
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


def _tensor_report(name, g, piv, proc, u, v, stages, ties, oracle):
    """fp16 tensor form against the reference: pass-0 peaks identical except
    near ties, deviations counted and bounded."""
    report = ["[tensor]"]
    for k, st in enumerate(stages):
        mism, tie, ref_tie, excused, exc_full = _pass_peaks(g, k, st, oracle)
        assert int(st["near_tie"].sum()) == ties[k], "near-tie flags and count disagree"
        du = np.abs(st["u_corr"].astype(np.float64) - g[f"it{k}_u_corr"])
        dv = np.abs(st["v_corr"].astype(np.float64) - g[f"it{k}_v_corr"])
        d = np.nan_to_num(np.maximum(du, dv), nan=0.0)
        flips = int((st["val0"] != g[f"it{k}_val0"]).sum())
        n_win = d.size
        report.append(f"it{k} peaks differing {int(mism.sum())} (near ties {ties[k]}), windows > {TOL_PX:g} px "
                      f"{int((d > TOL_PX).sum())}/{n_win}, max {float(d.max()):.1e} px, mask flips {flips}")
        if k == 0:
            assert not (mism & ~excused).any(), f"it0: {int((mism & ~excused).sum())} integer peaks differ"
            assert float(np.where(exc_full, 0, d).max()) <= F16_PASS0_MAX_PX, "it0 displacement deviation"
        assert flips <= max(1, int(F16_MAX_FLIP_FRAC * n_win)), f"it{k}: {flips} validation-mask flips"
    du, dv = u - g["u"], v - g["v"]
    fin = np.isfinite(du) & np.isfinite(dv)
    d = np.maximum(np.abs(np.where(fin, du, 0)), np.abs(np.where(fin, dv, 0)))
    jumps = fin & (d > F16_PEAK_JUMP_PX)
    keep = fin & ~jumps
    rms = float(np.sqrt(np.mean(du[keep] ** 2 + dv[keep] ** 2))) if keep.any() else 0.0
    report.append(f"final rms {rms:.1e} px over {int(keep.sum())} vectors, peak jumps {int(jumps.sum())} "
                  f"(max {float(d.max(initial=0)):.1e} px)")
    print(name, "; ".join(report))
    assert rms <= F16_FINAL_RMS_PX, f"final field rms {rms:.3e} px"
    assert int(jumps.sum()) <= max(2, int(F16_MAX_FLIP_FRAC * d.size)), f"{int(jumps.sum())} final peak jumps"
