"""The FLOP counts behind the bench line's roofline (CPU).

Algorithmic work of one window-pair correlation: two real-to-complex and one
complex-to-real 2-D FFT of N x N at 2.5 N^2 log2(N^2) each, the conjugate
product over the N (N/2 + 1) half spectrum (6 FLOP per complex product) and
the two mean removals (2 ss^2 each). Executed tensor-core work, counted here
stage by stage from the products' shapes per window pair:
  stage 1 (per frame): rows y (ss) x K = x (ss) x packed f_c (N);
  stage 2 (per frame): rows c (N, both row tiles) x K = y (ss) x packed f_r (N);
  stage 3: rows c (N/2) x two products of K = N (folded frequency pairs) x r (N);
  stage 4: rows r (N) x K = (Re|Im, c) (N) x s (N);
two FLOP per MAC, three products per stage with hi/lo split operands."""

import math
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import bench  # noqa: E402


@pytest.mark.parametrize("ss,expected", [(16, 81088), (32, 385408), (64, 1786624)])
def test_algorithmic_flops_per_window(ss, expected):
    n = 2 * ss
    fft = 2.5 * n * n * math.log2(n * n)
    assert bench.corr_flops(ss, n) == pytest.approx(3 * fft + 6 * n * (n // 2 + 1) + 4 * ss * ss)
    assert bench.corr_flops(ss, n) == expected


@pytest.mark.parametrize("ss", [16, 32, 64])
def test_executed_tensor_flops_per_window(ss):
    n = 2 * ss
    macs = 2 * (ss * ss * n)        # stage 1, both frames
    macs += 2 * (n * ss * n)        # stage 2, both frames
    macs += (n // 2) * 2 * n * n    # stage 3, folded pairs
    macs += n * n * n               # stage 4
    assert bench.tc_executed_flops(ss, n) == 2 * macs
    assert bench.tc_executed_flops(ss, n, split=True) == 6 * macs
    # Executed MMA work exceeds the FFT count (dense DFTs against butterflies).
    assert bench.tc_executed_flops(ss, n) > bench.corr_flops(ss, n)


def test_executed_flops_of_the_bench_passes():
    assert [bench.tc_executed_flops(ss, 2 * ss) for ss in (16, 32, 64)] == [229376, 1835008, 14680064]
