"""The closed-form pieces the kernels use, checked in numpy: the series for
sinh(t)/t below t = 1 and the one-division form of the sinh cell's chord
conductance (csrc/common.cuh)."""
import math

import numpy as np

COEF = [1 / math.factorial(2 * k + 1) for k in range(7)]   # 1/1!, 1/3!, ..., 1/13!


def sinhc_series(t, dtype):
    u = (t * t).astype(dtype)
    p = dtype(COEF[6])
    for c in reversed(COEF[:6]):
        p = (p * u + dtype(c)).astype(dtype)
    return p


def test_series_truncation_and_fp32_rounding():
    t = np.linspace(0.0, 1.0, 20001)
    exact = np.where(t > 0, np.sinh(t) / np.where(t > 0, t, 1), 1.0)
    assert np.abs(sinhc_series(t, np.float64) / exact - 1).max() < 1e-12     # truncation
    t32 = t.astype(np.float32)
    got = sinhc_series(t32, np.float32).astype(np.float64)
    ref = np.where(t32 > 0, np.sinh(t32.astype(np.float64)) / np.where(t32 > 0, t32, 1), 1.0)
    assert np.abs(got / ref - 1).max() < 4 * 2.0 ** -24                      # a few FP32 ulps


def test_chord_conductance_one_division_form():
    rng = np.random.default_rng(0)
    z = rng.random(1000)
    x = rng.random(1000) * 0.5
    a_on, b_on, a_off, b_off = 2.0, 1e-4, 2.0, 1e-6
    r0_on, r0_off = 1 / (a_on * b_on), 1 / (a_off * b_off)
    s_on = np.sinh(a_on * x) / (a_on * x)
    s_off = np.sinh(a_off * x) / (a_off * x)
    three = 1 / ((1 - z) * r0_on / s_on + z * r0_off / s_off)
    one = s_on * s_off / ((1 - z) * r0_on * s_off + z * r0_off * s_on)
    np.testing.assert_allclose(one, three, rtol=1e-14)
    # and the cell law itself: I = (1-z)-weighted series of the on and off sinh branches
    V = x
    R = (1 - z) * V / (b_on * np.sinh(a_on * V)) + z * V / (b_off * np.sinh(a_off * V))
    np.testing.assert_allclose(one, 1 / R, rtol=1e-13)
