"""The bench's measurement helpers on the CPU: the relMSE definition and the
time-to-plain-relMSE fit (bench.fit_to_target), checked on
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


def test_fit_is_exact_for_a_power_law():
    # err = V / n is a line of slope -1 in log-log: the crossing is exact
    V, a, b = 3.0, 40.0, 0.9
    pts = _points([100, 400, 1600], V, 0.0, a, b)
    n, t, reached = bench.fit_to_target(pts, V / 250.0)
    assert reached
    assert n == pytest.approx(250.0, rel=1e-9)
    assert t == pytest.approx(a + b * 250.0, rel=1e-9)


def test_fit_with_a_bias_floor_uses_the_points_near_the_crossing():
    V, B, a, b = 1.0, 2e-4, 20.0, 0.5
    pts = _points([100, 200, 500, 800, 1400, 4000], V, B, a, b)
    n, t, reached = bench.fit_to_target(pts, V / 700.0 + B)  # exact answer: 700 spp
    assert reached and n == pytest.approx(700.0, rel=0.05)
    assert t == pytest.approx(a + b * n, rel=1e-6)


def test_fit_tolerates_one_noisy_point():
    # three points on err = 1/n and one 25 % high: the answer moves little
    pts = _points([300, 500, 700], 1.0, 0.0, 0.0, 1.0) + [(600, 600.0, 1.25 / 600)]
    n, _, _ = bench.fit_to_target(pts, 1.0 / 550)
    assert n == pytest.approx(550.0, rel=0.12)


def test_fit_clamps_a_rising_slope():
    # noise can make the error rise with spp between two points; the slope is
    # then held at -0.2, so the crossing lies below both points
    pts = [(1024, 367.0, 2.57e-4), (1344, 474.0, 3.09e-4)]
    n, t, reached = bench.fit_to_target(pts, 3.23e-4)
    assert reached and 200 < n < 1024 and 0 < t < 367.0


def test_fit_all_points_above_the_target():
    pts = _points([100, 200], 1.0, 0.0, 0.0, 1.0)
    n, t, reached = bench.fit_to_target(pts, 1.0 / 800)
    assert not reached and n == pytest.approx(800.0, rel=1e-9) and t == pytest.approx(800.0)
