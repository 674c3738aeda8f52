"""How far the LSM regression coefficients are determined by the data (CPU).

The reference fits each exercise date by a sequential Householder QR
(src/core/linalg.cpp:7-71) over the in-the-money paths in path order.  Where
those paths fill a narrow band of S/K -- early dates of out-of-the-money puts --
the Laguerre design matrix is ill-conditioned (cond up to ~1e7), and the
coefficients are fixed by the data only to ~1e-9 relative: the reference's own
algorithm, run on the same rows in another order, moves them that much.  The
fitted continuation values, which the exercise decisions compare against, stay
within ~1e-13 of the coefficient scale.  This is the yardstick for the GPU's
Cholesky-QR2 fit: its coefficients are compared through the fitted values
(tests/test_gpu_lsm_grid.py), and its prices agree with the reference to 1e-12.
"""
from __future__ import annotations

import ctypes as C

import numpy as np


def _laguerre(x):
    e = np.exp(-x / 2)
    return np.stack([e, e * (1 - x), e * (1 - 2 * x + .5 * x * x), e * (1 - 3 * x + 1.5 * x * x - x ** 3 / 6)], -1)


def _householder(orc, X, y):
    a = np.ascontiguousarray(X, dtype=np.float64).copy()
    yy = np.ascontiguousarray(y, dtype=np.float64).copy()
    beta = np.zeros(X.shape[1])
    P = C.POINTER(C.c_double)
    orc.orc_householder_least_squares(a.ctypes.data_as(P), len(yy), X.shape[1], yy.ctypes.data_as(P),
                                      beta.ctypes.data_as(P))
    return beta


def test_householder_coefficients_are_conditioning_limited(orc):
    rng = np.random.default_rng(11)
    worst_coef, worst_fit = 0.0, 0.0
    for (s0, vol, t) in [(44, .2, .06), (42, .2, .02), (36, .2, .5)]:
        n = 1 << 18
        s = s0 * np.exp((0.06 - vol * vol / 2) * t + vol * np.sqrt(t) * rng.standard_normal(n))
        s_next = s * np.exp((0.06 - vol * vol / 2) * .5 + vol * np.sqrt(.5) * rng.standard_normal(n))
        itm = s < 40
        X = _laguerre(s[itm] / 40)
        y = np.maximum(40 - s_next[itm], 0) * np.exp(-0.06 * .5)
        b_fwd = _householder(orc, X, y)
        b_rev = _householder(orc, X[::-1], y[::-1])
        scale = np.abs(b_fwd).sum()
        band = _laguerre(np.linspace(s[itm].min() / 40, 1.0, 26))
        coef = np.abs(b_rev - b_fwd).max() / scale
        fit = np.abs(band @ (b_rev - b_fwd)).max() / scale
        worst_coef, worst_fit = max(worst_coef, coef), max(worst_fit, fit)
        assert fit < 1e-11, (s0, vol, t, fit)
    print(f"row order moves the reference's coefficients by up to {worst_coef:.1e} of their scale, "
          f"the fitted values by {worst_fit:.1e}")
    assert worst_coef > 1e-10  # the narrow-band dates leave the coefficients loosely determined
