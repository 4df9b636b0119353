"""Known-answer test of the device Boys function (csrc/boys.cuh) that every ERI kernel evaluates.

Golden values (tests/golden/boys_values.npz, make_boys_golden.py): F_0 .. F_9 at 481 values of T in
[0, 60] from the reference's Boys::calculateBoys (src/Boys.cpp:14-71) and from mpmath at 40 digits.

Tolerances:
* FP64, T <= 30 (Taylor expansion about the nearest grid point, downward recursion): 1e-14 relative to
  the exact value.
* FP64, T > 30: the reference and this engine both switch to the asymptotic form F_0 = sqrt(pi/T)/2,
  F_{m+1} = (m + 1/2) F_m / T, which drops terms of order e^{-T}; the device must agree with the
  reference's values to 1e-13 relative, and with the exact values to 1e-14 of F_0(T) absolute.
* FP32: 1e-6 relative for T <= 30 (float rounding, 6e-8 per operation, dominates the 2.6e-9 truncation
  of the 5-term expansion), and above 30, against the reference's asymptotic values, 2.5e-7 (m + 1) + 3e-7
  relative for order m (float rounding of each upward step).
"""
import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def _golden():
    import os

    return dict(np.load(os.path.join(GOLDEN, "boys_values.npz")))


@pytest.mark.parametrize("m_max", [0, 1, 4, 8, 9])
def test_gpu_boys_fp64_known_answers(m_max):
    from hfgpu.engine import boys_eval

    g = _golden()
    T, ex, rf = g["T"], g["F_exact"][:, :m_max + 1], g["F_ref"][:, :m_max + 1]
    F = boys_eval(m_max, T)
    lo = T <= 30.0
    assert np.max(np.abs(F[lo] - ex[lo]) / ex[lo]) <= 1e-14
    hi = ~lo
    assert np.max(np.abs(F[hi] - rf[hi]) / rf[hi]) <= 1e-13
    # The asymptotic form drops e^{-T} / (2T) in each of the m upward steps (each step scales earlier
    # errors by (k + 1/2) / T < 1 for T > 30): |F_m - exact| <= m e^{-T} / (2T) plus rounding.
    m = np.arange(m_max + 1)[None, :]
    bound = m * (np.exp(-T[hi]) / (2 * T[hi]))[:, None] + 1e-14 * ex[hi]
    assert np.all(np.abs(F[hi] - ex[hi]) <= bound)


@pytest.mark.parametrize("m_max", [0, 2, 5, 8])
def test_gpu_boys_fp32_known_answers(m_max):
    from hfgpu.engine import boys_eval

    g = _golden()
    T, ex, rf = g["T"], g["F_exact"][:, :m_max + 1], g["F_ref"][:, :m_max + 1]
    F = boys_eval(m_max, T, fp32=True)
    lo = T <= 30.0
    assert np.max(np.abs(F[lo] - ex[lo]) / ex[lo]) <= 1e-6
    # Above 30 each upward step (m + 1/2) / T * F_m rounds about three times in float (6e-8 each), on top
    # of rsqrtf's F_0: 2.5e-7 per order plus 3e-7.
    m = np.arange(m_max + 1)[None, :]
    assert np.all(np.abs(F[~lo] - rf[~lo]) / rf[~lo] <= 2.5e-7 * (m + 1) + 3e-7)


def test_gpu_boys_rejects_bad_arguments():
    from hfgpu.engine import HfgError, boys_eval

    with pytest.raises(HfgError):
        boys_eval(10, [1.0])
    with pytest.raises(HfgError):
        boys_eval(2, [-1.0])
    with pytest.raises(HfgError):
        boys_eval(2, [float("nan")])
