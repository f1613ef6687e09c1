"""piv_smoothn_noalloc: the smoothn entry point for callers that cannot
allocate device memory (its scratch is a fixed array inside the library).

Checked through the C ABI against piv_smoothn, the allocating entry point, on
three calls in a row with different inputs and shapes, unmasked and masked
(each call reuses the array the previous one left behind), with the smoothn
tests' tolerance; and its refusals: a request beyond the array, and a masked
request that fits the unmasked path but not the weighted one.
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


def _smooth(torch, lib, fn, u, v, s, mask=None):
    n_pairs, m, n = u.shape
    du, dv = torch.as_tensor(u).cuda(), torch.as_tensor(v).cuda()
    p = torch.empty(n_pairs, dtype=torch.float64, device="cuda")
    dm = None if mask is None else torch.as_tensor(mask.astype(np.uint8)).cuda()
    rc = getattr(lib, fn)(m, n, n_pairs, du.data_ptr(), dv.data_ptr(), None if dm is None else dm.data_ptr(), s,
                          p.data_ptr(), torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return rc, du.cpu().numpy(), dv.cpu().numpy(), p.cpu().numpy()


def _mask(shape, seed):
    """A field mask with a disc and a few scattered cells masked."""
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:shape[0], 0:shape[1]]
    m = (y - shape[0] / 3) ** 2 + (x - shape[1] / 2) ** 2 < (min(shape) / 6) ** 2
    m.flat[rng.choice(m.size, 12, replace=False)] = True
    return m


def test_noalloc_smoothn_matches_allocating_entry_point():
    import torch

    from openpiv_gpu import _build, _lib

    _build.build()
    torch.cuda.set_device(0)
    lib = _lib.load()
    # Unmasked at a given s, unmasked with GCV, then the masked (weighted)
    # path, which lays the array out differently, with GCV: three calls in a
    # row, each finding the array as the previous one left it.
    calls = [((63, 63), 2, 0.8, 5, None), ((31, 47), 3, float("nan"), 6, None),
             ((63, 63), 2, float("nan"), 8, _mask((63, 63), 8))]
    for shape, n_pairs, s, seed, mask in calls:
        u, v = _fields(seed, shape, n_pairs)
        rc_a, ua, va, pa = _smooth(torch, lib, "piv_smoothn", u, v, s, mask)
        rc_b, ub, vb, pb = _smooth(torch, lib, "piv_smoothn_noalloc", u, v, s, mask)
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
    # 4 pairs of 128 x 128 fit the unmasked path but not the weighted one.
    u, v = _fields(9, (128, 128), 4)
    rc, _, _, _ = _smooth(torch, lib, "piv_smoothn_noalloc", u, v, 0.8)
    assert rc == _lib.PIV_OK, _lib.last_error()
    rc, _, _, _ = _smooth(torch, lib, "piv_smoothn_noalloc", u, v, 0.8, _mask((128, 128), 9))
    assert rc == _lib.PIV_E_ARG
    assert "masked" in _lib.last_error()
