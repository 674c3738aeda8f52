"""Fits the polynomials of the FP32 inverse normal (device_common.cuh,
normal_from_bits_f32) and prints them as C++ initialisers.

For q in (0, 1/2] let x = 1 - 2q and w = -ln(4 q (1 - q)) = -ln(1 - x^2).  Then
Phi^-1(1 - q) = x P(w) with P smooth in w (the change of variable of M. Giles,
"Approximating the erfinv function", GPU Computing Gems Jade, 2011).  Two
polynomials cover the 32-bit inputs (q >= 2^-33, so w <= 21.5):
  central  w < 5:  P ~ degree 8 in t = w - 2.5      (q > 0.0017: 99.66 % of draws)
  tail     w >= 5: P ~ degree 9 in t = sqrt(w) - 3
The coefficients here are fitted to scipy's double-precision ndtri by weighted least
squares on the relative error with Lawson's iterative reweighting toward the minimax
solution; the script is deterministic.

    python derivative-pricing_gb300/csrc/fit_inverse_normal.py
"""
from __future__ import annotations

import numpy as np
from scipy.special import ndtri

W_SPLIT = 5.0
W_MAX = 22.5  # > -ln(4 q (1 - q)) at q = 2^-33


def q_of_w(w):
    return (1.0 - np.sqrt(-np.expm1(-w))) / 2.0


def fit(region: str, degree: int, samples: int = 200_001, iterations: int = 60):
    if region == "central":
        w = np.linspace(1e-9, W_SPLIT, samples)
        t = w - 2.5
    else:
        s = np.linspace(np.sqrt(W_SPLIT), np.sqrt(W_MAX), samples)
        w = s * s
        t = s - 3.0
    q = q_of_w(w)
    p = -ndtri(q) / (1.0 - 2.0 * q)
    v = np.vander(t, degree + 1)
    weights = np.ones_like(t)
    for _ in range(iterations):
        scale = weights / np.abs(p)
        coef, *_ = np.linalg.lstsq(v * scale[:, None], p * scale, rcond=None)
        err = (v @ coef - p) / p
        weights = weights * np.sqrt(np.abs(err)) + 1e-30
        weights /= weights.max()
    return coef, float(np.abs(err).max())


def main():
    for region, degree in (("central", 8), ("tail", 9)):
        coef, err = fit(region, degree)
        body = ", ".join(f"{c:.9e}f" for c in coef)
        print(f"// {region}: degree {degree}, max relative fit error {err:.2e} (highest power first)")
        print(f"{{{body}}}")


if __name__ == "__main__":
    main()
