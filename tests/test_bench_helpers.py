"""The error arithmetic of the time-to-relMSE measurement (bench.py), on
synthetic images with known noise: the reference's own noise estimate is
unbiased, so subtracting it recovers the error against the truth, and the
time-to-target helpers interpolate and extrapolate as documented."""
import os
import sys

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


def test_reference_noise_is_taken_out_without_bias():
    rng = np.random.default_rng(7)
    shape = (400, 500, 3)
    truth = rng.uniform(0.05, 2.0, size=shape)
    sigma, tau = 0.05, 0.12  # noise of the reference, of the render
    half_a = truth + rng.normal(0, sigma * np.sqrt(2), size=shape)
    half_b = truth + rng.normal(0, sigma * np.sqrt(2), size=shape)
    ref = 0.5 * (half_a + half_b)
    x = truth + rng.normal(0, tau, size=shape)
    floor = bench.reference_noise(half_a, half_b)
    expected_floor = float(np.mean(sigma ** 2 / (ref ** 2 + 0.01)))
    assert abs(floor - expected_floor) < 0.02 * expected_floor
    against_truth = float(np.mean(tau ** 2 / (ref ** 2 + 0.01)))
    corrected = bench.rel_mse(x, ref) - floor
    assert abs(corrected - against_truth) < 0.02 * against_truth
    # uncorrected, the reference's noise is added on top
    assert bench.rel_mse(x, ref) > 1.1 * against_truth


def test_time_to_target_interpolates_and_extrapolates():
    pts = [(16, 1.0, 0.08), (32, 2.0, 0.04), (64, 4.0, 0.005)]
    t, how = bench.time_to_target(pts, 0.01)
    assert how == "interpolated" and 2.0 < t < 4.0
    # log-log between (2 s, 0.04) and (4 s, 0.005): 0.01 lies 2/3 of the way
    assert abs(t - 2.0 * 2.0 ** (2.0 / 3.0)) < 1e-9
    t, how = bench.time_to_target([(16, 1.0, 0.16), (32, 2.0, 0.08), (64, 4.0, 0.04)], 0.01)
    assert how.startswith("extrapolated") and abs(t - 16.0) < 1e-9
    t, how = bench.time_to_target([(16, 1.0, 0.009)], 0.01)
    assert how == "measured" and t == 1.0
