"""The bench's measurement helpers on the CPU: the relMSE definition and the
time-to-plain-relMSE interpolation (bench.interpolate_to_target), checked on
synthetic points of a known error model err(n) = V / n + B and time
t(n) = a + b n, where the answer has a closed form."""
import os
import sys

import numpy as np
import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_relmse_definition():
    ref = np.array([[0.0, 1.0], [2.0, 0.5]])
    x = np.array([[0.1, 1.5], [2.0, 0.0]])
    want = np.mean((x - ref) ** 2 / (ref ** 2 + 1e-2))
    assert bench._relmse(x, ref) == pytest.approx(want, rel=1e-12)
    assert bench._relmse(ref, ref) == 0.0


def _points(spps, V, B, a, b):
    return [(n, a + b * n, V / n + B) for n in spps]


def test_interpolation_hits_a_point_exactly():
    pts = _points([128, 256, 512], 1.0, 0.0, 10.0, 2.0)
    n, t, reached = bench.interpolate_to_target(pts, 1.0 / 256)
    assert reached and n == pytest.approx(256.0) and t == pytest.approx(10.0 + 2.0 * 256)


def test_interpolation_is_exact_for_a_power_law():
    # err = V / n is a straight line in log-log: the interpolated spp is exact
    V, a, b = 3.0, 40.0, 0.9
    pts = _points([100, 400], V, 0.0, a, b)
    target = V / 250.0
    n, t, reached = bench.interpolate_to_target(pts, target)
    assert reached
    assert n == pytest.approx(250.0, rel=1e-9)
    assert t == pytest.approx(a + b * 250.0, rel=1e-9)


def test_interpolation_with_a_bias_floor_stays_between_the_brackets():
    V, B, a, b = 1.0, 2e-4, 20.0, 0.5
    pts = _points([200, 500, 900, 1400], V, B, a, b)
    target = V / 700.0 + B  # exact answer: 700 spp
    n, t, reached = bench.interpolate_to_target(pts, target)
    assert reached and 500 < n < 900
    # log-log interpolation of a curve that flattens toward B is close, not exact
    assert n == pytest.approx(700.0, rel=0.05)
    assert t == pytest.approx(a + b * n, rel=1e-9)


def test_interpolation_points_unsorted_and_out_of_range():
    pts = _points([800, 200, 400], 1.0, 0.0, 0.0, 1.0)
    n, _, reached = bench.interpolate_to_target(pts, 1.0 / 300)
    assert reached and n == pytest.approx(300.0, rel=1e-9)
    # every point above the target: the largest spp, not reached
    n, t, reached = bench.interpolate_to_target(pts, 1e-6)
    assert not reached and n == 800.0 and t == 800.0
    # every point below the target: the smallest spp, reached
    n, t, reached = bench.interpolate_to_target(pts, 1.0)
    assert reached and n == 200.0
