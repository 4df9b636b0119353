"""Golden Boys-function values for the device known-answer test (tests/test_gpu_boys.py).

    python tests/golden/make_boys_golden.py          (needs oracle/_ref)

For 481 values of T in [0, 60] -- a uniform grid, T = 0, random points, and points on both sides of the
asymptotic switch at T = 30 -- stores F_0 .. F_9 from the reference's Boys::calculateBoys
(src/Boys.cpp:14-71, via oracle/_ref) and the exact values F_m(T) = gamma(m + 1/2, T) / (2 T^(m + 1/2))
from mpmath at 40 significant digits.
"""
import os
import sys

import mpmath
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import ref  # noqa: E402

M_MAX = 9


def exact(m, T):
    if T == 0.0:
        return 1.0 / (2 * m + 1)
    t = mpmath.mpf(T)
    return float(mpmath.gammainc(m + mpmath.mpf(1) / 2, 0, t) / (2 * t ** (m + mpmath.mpf(1) / 2)))


def main():
    mpmath.mp.dps = 40
    rng = np.random.default_rng(2024)
    T = np.concatenate([np.linspace(0.0, 60.0, 241), rng.uniform(0.0, 30.0, 160), rng.uniform(30.0, 60.0, 60),
                        [0.0, 1e-12, 1e-6, 1e-3, 29.95, 29.999999, 30.0, 30.000001, 30.05, 30.5],
                        rng.uniform(0.0, 0.1, 10)])
    F_ref = np.array([ref.boys(M_MAX, float(t)) for t in T])
    F_exact = np.array([[exact(m, float(t)) for m in range(M_MAX + 1)] for t in T])
    np.savez_compressed(os.path.join(HERE, "boys_values.npz"), T=T, F_ref=F_ref, F_exact=F_exact, m_max=M_MAX)
    print("boys_values.npz:", T.size, "points; max rel |ref - exact| for T <= 30:",
          float(np.max(np.abs(F_ref - F_exact)[T <= 30] / F_exact[T <= 30])))


if __name__ == "__main__":
    main()
