"""Autotuner of the correlation launch variants (piv_plan_autotune).

Variants of the tensor engines (CTAs per SM, staging) give bit-identical
fields; variants of the FFT engine (radix split, windows and threads per CTA)
give the same correlation up to rounding; the autotuner times every variant of
every pass, keeps the fastest, and a second plan of the same geometry reuses
the choice without timing."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (512, 512)


def _case(B=2):
    from openpiv_gpu import _build, synthetic

    _build.build()
    pairs = [synthetic.config_case(2, k, shape=SHAPE)[:2] for k in range(B)]
    kw = dict(synthetic.CONFIGS[2]["piv"])
    mss = kw.pop("min_search_size")
    fa = np.stack([p[0] for p in pairs])
    fb = np.stack([p[1] for p in pairs])
    return fa, fb, mss, kw


def _run(proc, fa, fb, variants=None):
    from openpiv_gpu import _lib

    plan = proc.plan_handle(fa, len(fa))
    if variants is not None:
        for k, v in enumerate(variants):
            _lib.check(_lib.lib().piv_plan_set_variant(plan, k, v))
    u, v = proc.run_batch(fa, fb)
    per_pass = [proc.iteration_outputs(p) for p in range(len(fa))]
    return u.cpu().numpy(), v.cpu().numpy(), per_pass


def _counts(proc):
    return [len(t["variants"]) for t in proc.tuning()]


@pytest.mark.parametrize("dft", ["tensor", "tensor_split"])
def test_tensor_variants_are_identical(dft):
    from openpiv_gpu.gpu_process import PIVGPU

    fa, fb, mss, kw = _case()
    proc = PIVGPU(SHAPE, mss, **kw, dft=dft)
    u0, v0, _ = _run(proc, fa, fb)
    counts = _counts(proc)
    names = [t["variants"] for t in proc.tuning()]
    n_passes = len(counts)
    checked = 0
    for k in range(n_passes):
        if not names[k][0].startswith("tensor"):
            continue
        for var in range(1, counts[k]):
            sel = [0] * n_passes
            sel[k] = var
            u, v, _ = _run(proc, fa, fb, sel)
            np.testing.assert_array_equal(u, u0, err_msg=f"pass {k} variant {names[k][var]}")
            np.testing.assert_array_equal(v, v0, err_msg=f"pass {k} variant {names[k][var]}")
            checked += 1
    print(f"{dft}: {checked} variants identical; {names}")
    assert checked > 0


def test_fft_variants_agree_up_to_rounding():
    from openpiv_gpu.gpu_process import PIVGPU

    fa, fb, mss, kw = _case()
    proc = PIVGPU(SHAPE, mss, **kw, dft="fft")
    _, _, ref = _run(proc, fa, fb)
    counts = _counts(proc)
    names = [t["variants"] for t in proc.tuning()]
    for k, nv in enumerate(counts):
        assert nv > 1, f"pass {k} has one FFT variant"
        for var in range(1, nv):
            sel = [0] * len(counts)
            sel[k] = var
            _, _, got = _run(proc, fa, fb, sel)
            d = np.concatenate([np.abs(np.concatenate([(got[p][k]["u_corr"] - ref[p][k]["u_corr"]).ravel(),
                                                       (got[p][k]["v_corr"] - ref[p][k]["v_corr"]).ravel()]))
                                for p in range(len(fa))])
            d = d[np.isfinite(d)]
            far = float(np.mean(d > 1e-3))
            print(f"pass {k} {names[k][var]}: median {np.median(d):.1e}, p99 {np.percentile(d, 99):.1e}, "
                  f"far {far:.4f}")
            assert np.median(d) < 1e-5
            assert far < 2e-3  # integer-peak near-ties may flip under a different summation order


def test_autotune_picks_fastest_and_caches():
    from openpiv_gpu import _lib
    from openpiv_gpu.gpu_process import PIVGPU

    fa, fb, mss, kw = _case()
    _lib.lib().piv_autotune_cache_clear()
    base = PIVGPU(SHAPE, mss, **kw, dft="tensor")
    u0, v0, _ = _run(base, fa, fb)
    for dft in ("tensor", "fft"):
        proc = PIVGPU(SHAPE, mss, **kw, dft=dft, autotune=True)
        u, v = proc.run_batch(fa, fb)
        tuning = proc.tuning()
        for k, t in enumerate(tuning):
            assert all(ms is not None and ms > 0 for ms in t["ms"]), (k, t)
            assert t["variant"] == int(np.argmin(t["ms"])), (k, t)
            print(f"{dft} pass {k}: {t['name']} ({min(t['ms']):.3f} ms; default {t['ms'][0]:.3f} ms)")
        if dft == "tensor":
            np.testing.assert_array_equal(u.cpu().numpy(), u0)
            np.testing.assert_array_equal(v.cpu().numpy(), v0)
        again = PIVGPU(SHAPE, mss, **kw, dft=dft, autotune=True)
        again.run_batch(fa, fb)
        for t1, t2 in zip(tuning, again.tuning()):
            assert t2["variant"] == t1["variant"]
            assert all(ms is None for ms in t2["ms"])  # taken from the process-wide results


def test_set_variant_rejects_out_of_range():
    from openpiv_gpu import _lib
    from openpiv_gpu.gpu_process import PIVGPU

    fa, fb, mss, kw = _case(B=1)
    proc = PIVGPU(SHAPE, mss, **kw, dft="fft")
    _run(proc, fa, fb)
    plan = proc.plan_handle(fa, 1)
    n = _counts(proc)[0]
    assert _lib.lib().piv_plan_set_variant(plan, 0, n) == _lib.PIV_E_ARG
    assert _lib.lib().piv_plan_set_variant(plan, 0, -1) == _lib.PIV_E_ARG
    assert _lib.lib().piv_plan_set_variant(plan, 99, 0) == _lib.PIV_E_ARG
