"""The smoothing parameter search (L-BFGS-B on one bounded variable, as the
reference's smoothn calls scipy.optimize.fmin_l_bfgs_b, gpu_smoothn.py:191-193):

* the restatement in oracle/lbfgsb_1d.py against SciPy on seeded GCV problems
  of smoothn's own form (the GCV curve of noisy fields of many shapes, the
  start point from the 10-point scan): final p within 2e-6, and within a few
  ulps in most cases (a one-ulp difference in one iterate moves the later
  iterates by up to ~1e-6, because each step divides score differences by
  1e-8);
* the device search (csrc/piv_lbfgsb1.cuh, compiled for the host with FMA
  contraction off) against the restatement: identical steps and result.
"""

import ctypes
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from oracle import piv_oracle as po
from oracle.lbfgsb_1d import lbfgsb_1d

HERE = os.path.dirname(os.path.abspath(__file__))


def _problems(count, seed=0):
    """(fun, p0, p_min, p_max): GCV scores of smoothn for seeded noisy fields."""
    rng = np.random.default_rng(seed)
    out = []
    for t in range(count):
        m, n = int(rng.integers(5, 70)), int(rng.integers(5, 70))
        y, x = np.mgrid[0:m, 0:n]
        noise = rng.uniform(0.001, 2)
        u = rng.uniform(0.5, 5) * np.sin(x / rng.uniform(2, 20)) + noise * rng.normal(size=(m, n))
        v = rng.uniform(0.5, 5) * np.cos(y / rng.uniform(2, 20)) + noise * rng.normal(size=(m, n))
        if t % 7 == 0:  # pure noise: the flat GCV curves
            u, v = noise * rng.normal(size=(m, n)), noise * rng.normal(size=(m, n))
        args = ([po.dct2(u), po.dct2(v)], po.smoothn_lambda((m, n)) ** 2, m * n, m * n, 2)
        fun = (lambda a: (lambda q: float(po.gcv_score(np.asarray(q, dtype=np.float64), *a))))(args)
        p_min, p_max = po.p_bounds((m, n))
        span = np.arange(10) * (1 / 9) * (p_max - p_min) + p_min
        p0 = float(span[np.argmin([fun(q) for q in span])])
        out.append((fun, p0, p_min, p_max))
    return out


def test_restatement_matches_scipy():
    scipy_opt = pytest.importorskip("scipy.optimize")
    diffs = []
    for fun, p0, lo, hi in _problems(80):
        ref = scipy_opt.fmin_l_bfgs_b(lambda q: fun(q[0]), np.array([p0]), fprime=None, factr=10,
                                      approx_grad=True, bounds=[(lo, hi)])[0][0]
        diffs.append(abs(lbfgsb_1d(fun, p0, lo, hi) - ref))
    diffs = np.array(diffs)
    same = diffs <= 1e-12
    print(f"|p - p_scipy|: max {diffs.max():.2e}, within 1e-12: {int(same.sum())}/{diffs.size}")
    assert diffs.max() <= 2e-6
    assert same.mean() >= 0.8


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc) and not shutil.which("nvcc"):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("lb") / "liblb1.so")
    cmd = [nvcc, "-std=c++17", "-O2", "-shared", "-Xcompiler", "-fPIC,-ffp-contract=off",
           os.path.join(HERE, "lbfgsb_harness.cu"), "-o", out]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(out)
    lib.lb1_minimize.restype = ctypes.c_double
    return lib


def test_device_search_matches_restatement(harness):
    CB = ctypes.CFUNCTYPE(ctypes.c_double, ctypes.c_double)
    harness.lb1_minimize.argtypes = [CB, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                     ctypes.POINTER(ctypes.c_int)]
    for fun, p0, lo, hi in _problems(40, seed=1):
        trace = []
        want = lbfgsb_1d(fun, p0, lo, hi, trace=trace)
        n = ctypes.c_int(0)
        got = harness.lb1_minimize(CB(fun), p0, lo, hi, ctypes.byref(n))
        assert got == want
        assert n.value == 2 * len(trace)
