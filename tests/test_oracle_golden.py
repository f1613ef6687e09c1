"""Pins the CPU oracle to the reference: every golden case under tests/golden/
was produced by the unmodified reference (see make_golden.py); the oracle must
reproduce its outputs and stage intermediates exactly."""

import numpy as np
import pytest

import make_golden as mg
from openpiv_gpu import synthetic as syn
from oracle.piv_oracle import OraclePIV

CASES = mg.cases()


def _load_case(name, cfg, shape, pair_index, overrides, store):
    g = np.load(f"{mg.HERE}/{name}.npz")
    if store:
        a, b = g["frame_a"], g["frame_b"]
        _, _, _, piv = mg.build_case(syn, cfg, a.shape, pair_index, overrides)
    else:
        a, b, _, piv = mg.build_case(syn, cfg, shape, pair_index, overrides)
        if mg._digest(a) != str(g["sha_a"]) or mg._digest(b) != str(g["sha_b"]):
            pytest.skip("synthetic generator output differs from the fixture's frames on this NumPy")
    return g, a, b, piv


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_oracle_matches_reference(case):
    g, a, b, piv = _load_case(*case)
    mss = piv.pop("min_search_size")
    o = OraclePIV(a.shape, mss, **piv)
    u, v = o(a, b)
    assert u.dtype == g["u"].dtype
    np.testing.assert_array_equal(u, g["u"])
    np.testing.assert_array_equal(v, g["v"])
    x, y = o.coords
    np.testing.assert_array_equal(x, g["x"])
    np.testing.assert_array_equal(y, g["y"])
    vl = o.val_locations if o.val_locations is not None else np.zeros(u.shape, bool)
    ol = o.outliers if o.outliers is not None else np.zeros(u.shape, bool)
    np.testing.assert_array_equal(vl, g["val_locations"])
    np.testing.assert_array_equal(ol, g["outliers"])
    assert len(o.trace) == int(g["n_iters"])
    for k, tr in enumerate(o.trace):
        np.testing.assert_array_equal(tr["u_corr"], g[f"it{k}_u_corr"])
        np.testing.assert_array_equal(tr["v_corr"], g[f"it{k}_v_corr"])
        np.testing.assert_array_equal(tr["i_peak"], g[f"it{k}_i_peak"])
        np.testing.assert_array_equal(tr["j_peak"], g[f"it{k}_j_peak"])
        np.testing.assert_array_equal(tr["val0"], g[f"it{k}_val0"])
        if f"it{k}_smooth_s" in g:
            assert np.power(10, tr["p"]) == pytest.approx(float(g[f"it{k}_smooth_s"]), rel=1e-14)
            np.testing.assert_array_equal(tr["u_smooth"], g[f"it{k}_u_smooth"])
        if f"it{k}_s2n" in g:
            np.testing.assert_array_equal(tr["s2n"], g[f"it{k}_s2n"])
