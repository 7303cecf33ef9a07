"""The guided leg's time-to-error arithmetic in bench.py, on synthetic progressive error curves
(no GPU): a tracer whose samples cost c times a plain one and carry v times its error reaches
plain's error in c * v of plain's time."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def _curve(wave_s, spp_per_wave, err_per_spp, waves):
    return [(wave_s * i, spp_per_wave * i, err_per_spp / (spp_per_wave * i)) for i in range(1, waves + 1)]


def test_time_to_error_interpolates_between_waves():
    curve = [(1.0, 16, 0.4), (2.0, 32, 0.2), (3.0, 48, 0.1)]
    assert bench.time_to_error(curve, 0.3) == pytest.approx(1.5)
    assert bench.time_to_error(curve, 0.1) == pytest.approx(3.0)
    assert bench.time_to_error(curve, 0.5) == pytest.approx(1.0)  # reached by the first wave
    assert bench.time_to_error(curve, 0.05) is None                # never reached
    assert bench.time_to_error([], 0.1) is None


def test_time_ratio_curve_is_cost_times_error_ratio():
    plain = _curve(0.08, 16, 1.0, 130)    # 10.4 s
    guided = _curve(0.125, 16, 0.4, 90)   # costs 1.5625x, 0.4x the error per sample
    pts = bench.time_ratio_curve(plain, guided)
    assert [p["plain_s"] for p in pts] == [2.0, 4.0, 6.0, 8.0, 10.0]
    for p in pts:
        assert p["time_ratio"] == pytest.approx(1.5625 * 0.4, abs=2e-3)


def test_time_ratio_curve_stops_at_plain_budget_and_marks_unreached():
    plain = _curve(0.5, 16, 1.0, 9)     # 4.5 s
    guided = _curve(0.5, 16, 3.0, 9)    # worse per sample: never reaches plain's later errors
    pts = bench.time_ratio_curve(plain, guided)
    assert [p["plain_s"] for p in pts] == [2.0, 4.0]
    assert all(p["time_ratio"] is None for p in pts)
