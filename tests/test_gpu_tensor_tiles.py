"""The tensor-core engines give every window the same result however many
tiles each CTA of the launch processes.

The 64-px engine pipelines consecutive tiles of a CTA (window corners set up
four tiles ahead, rows copied one tile ahead, statistics of the next tile
during stage 2, peak keys double-buffered, fits of a tile in the fit warp
during the next one); the 16/32-px engines keep three tile slots and overlap
a tile's fits with the next tile's staging. A pair correlated alone (about
one tile per CTA on 512 x 512 frames) must match the same pair inside
batches of 5 and 12 pairs (up to about ten tiles per CTA, partial last
tiles, tiles that straddle two pairs) bit for bit: fields and integer
peaks, for the fp16, hi/lo split and refined forms."""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (512, 512)
CASES = [(64, "tensor", "u8"), (64, "tensor_refined", "u8"), (32, "tensor", "f32"), (32, "tensor_split", "f32"),
         (32, "tensor_refined", "f32"), (16, "tensor", "f32"), (16, "tensor_split", "f32"),
         (16, "tensor_refined", "f32")]


@pytest.fixture(scope="module")
def env():
    import torch

    from openpiv_gpu import _build, _lib, synthetic

    _build.build()
    torch.cuda.set_device(0)
    a, b = [], []
    for k in range(12):
        fa, fb = synthetic.render_pair(SHAPE, synthetic.uniform_field(1.7 + 0.1 * k, -0.8), 700 + k, density=0.03)
        a.append(fa)
        b.append(fb)
    return torch, _lib, _lib.load(), np.stack(a), np.stack(b)


def _correlate(env, ss, dft, pixel, first, count):
    torch, _lib, lib, fa, fb = env
    g = _lib.PivGeometry()
    _lib.check(lib.piv_field_geometry(SHAPE[0], SHAPE[1], ss, ss, 0.5, 1, ctypes.byref(g)))
    dt = np.uint8 if pixel == "u8" else np.float32
    da = torch.as_tensor(fa[first:first + count].astype(dt)).cuda()
    db = torch.as_tensor(fb[first:first + count].astype(dt)).cuda()
    u = torch.full((count, g.m, g.n), float("nan"), dtype=torch.float32, device="cuda")
    v = torch.full_like(u, float("nan"))
    pi = torch.full((count, g.m, g.n), -1, dtype=torch.int32, device="cuda")
    pj = torch.full_like(pi, -1)
    s = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.piv_correlate(ctypes.byref(g), count, da.data_ptr(), db.data_ptr(), _lib.PIXEL[pixel], 0, 2 * ss,
                                 1, _lib.SUBPIXEL["gaussian"], None, u.data_ptr(), v.data_ptr(), pi.data_ptr(),
                                 pj.data_ptr(), 0, 2, None, _lib.DFT[dft], s))
    torch.cuda.synchronize()
    return [t.cpu().numpy() for t in (u, v, pi, pj)], g.m * g.n


@pytest.mark.parametrize("ss,dft,pixel", CASES)
def test_results_do_not_depend_on_tiles_per_cta(env, ss, dft, pixel):
    big, n_win = _correlate(env, ss, dft, pixel, 0, 12)
    mid, _ = _correlate(env, ss, dft, pixel, 3, 5)
    assert np.isfinite(big[0]).all() and (big[2] >= 0).all()
    for k in (0, 5, 11):
        alone, _ = _correlate(env, ss, dft, pixel, k, 1)
        for name, x, y in zip("u v peak_i peak_j".split(), alone, big):
            np.testing.assert_array_equal(x[0], y[k], err_msg=f"pair {k} alone vs in 12: {name}")
    for k in range(5):
        for name, x, y in zip("u v peak_i peak_j".split(), mid, big):
            np.testing.assert_array_equal(x[k], y[3 + k], err_msg=f"pair {3 + k} in 5 vs in 12: {name}")
    tiles = 12 * n_win // (128 // ss)
    print(f"{dft} ss={ss}: {n_win} windows per pair, {tiles} tiles in the 12-pair launch")
