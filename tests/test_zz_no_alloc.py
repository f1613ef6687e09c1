"""piv_smoothn_noalloc: the smoothn entry point for callers that cannot
allocate device memory (its scratch is a fixed array inside the library).

Checked through the C ABI against piv_smoothn, the allocating entry point, on
two calls in a row with different inputs and shapes (the second call reuses
the array the first one left behind), with the smoothn tests' tolerance.
The file sorts last so that a run stopping at the first failure has already
run every other test.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FIXED_S = 1e-6  # the smoothn tests' tolerance at a given smoothing parameter


def _fields(seed, shape, n_pairs):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:shape[0], 0:shape[1]]
    u = np.stack([3 * np.sin(x / (5.0 + k)) + rng.normal(0, 0.2, shape) for k in range(n_pairs)])
    v = np.stack([2 * np.cos(y / (7.0 + k)) + rng.normal(0, 0.2, shape) for k in range(n_pairs)])
    return u, v


def _smooth(torch, lib, fn, u, v, s):
    n_pairs, m, n = u.shape
    du, dv = torch.as_tensor(u).cuda(), torch.as_tensor(v).cuda()
    p = torch.empty(n_pairs, dtype=torch.float64, device="cuda")
    rc = getattr(lib, fn)(m, n, n_pairs, du.data_ptr(), dv.data_ptr(), None, s, p.data_ptr(),
                          torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, du.cpu().numpy(), dv.cpu().numpy(), p.cpu().numpy()


def test_noalloc_smoothn_matches_allocating_entry_point():
    import torch

    from openpiv_gpu import _build, _lib

    _build.build()
    torch.cuda.set_device(0)
    lib = _lib.load()
    calls = [((63, 63), 2, 0.8, 5), ((31, 47), 3, float("nan"), 6)]
    for shape, n_pairs, s, seed in calls:
        u, v = _fields(seed, shape, n_pairs)
        rc_a, ua, va, pa = _smooth(torch, lib, "piv_smoothn", u, v, s)
        rc_b, ub, vb, pb = _smooth(torch, lib, "piv_smoothn_noalloc", u, v, s)
        assert rc_a == 0, _lib.last_error()
        assert rc_b == 0, _lib.last_error()
        np.testing.assert_allclose(ub, ua, atol=TOL_FIXED_S, rtol=0)
        np.testing.assert_allclose(vb, va, atol=TOL_FIXED_S, rtol=0)
        np.testing.assert_allclose(pb, pa, atol=1e-12, rtol=0)


def test_noalloc_smoothn_rejects_sizes_beyond_its_array():
    import torch

    from openpiv_gpu import _build, _lib

    _build.build()
    torch.cuda.set_device(0)
    lib = _lib.load()
    u, v = _fields(7, (256, 256), 4)
    rc, _, _, _ = _smooth(torch, lib, "piv_smoothn_noalloc", u, v, 0.8)
    assert rc == _lib.PIV_E_ARG
    assert "fixed" in _lib.last_error()
