"""Natural cubic splines on the host (FP64), the table format the GPU receives.

Follows ``spline_interpolation`` in ``src/discoeb/spline_interpolation.py``:
construction by a Thomas solve for the second derivatives with natural end
conditions (``spline_interpolation.py:47-88``), evaluation by the standard
``A y_i + B y_{i+1} + ((A^3-A) S_i + (B^3-B) S_{i+1}) h^2/6`` form with the
interval found by a left ``searchsorted`` (``spline_interpolation.py:130-153``).

The three arrays ``_x_``, ``_y_``, ``_S_full_`` carry the same names as the
reference pytree fields, so a reference ``param`` dict and one built here are
read the same way by :mod:`tables`.
"""
from __future__ import annotations

import numpy as np


def natural_second_derivatives(x: np.ndarray, y: np.ndarray) -> np.ndarray:
    """Second derivatives S at the knots, S[0] = S[-1] = 0 (Thomas algorithm).

    Same elimination order as ``spline_interpolation.py:50-85`` so the table
    values agree to rounding.
    """
    n = x.shape[0]
    if n < 2:
        raise ValueError("There must be at least two data points.")
    S = np.zeros(n)
    m = n - 2
    if m <= 0:
        return S
    h = x[1:] - x[:-1]
    lo = h[:-1]
    di = 2.0 * (h[:-1] + h[1:])
    up = h[1:]
    rhs = 6.0 * ((y[2:] - y[1:-1]) / h[1:] - (y[1:-1] - y[:-2]) / h[:-1])
    cp = np.zeros(m)
    dp = np.zeros(m)
    cp[0] = up[0] / di[0]
    dp[0] = rhs[0] / di[0]
    for i in range(1, m):
        den = di[i] - lo[i] * cp[i - 1]
        cp[i] = up[i] / den if i < m - 1 else 0.0
        dp[i] = (rhs[i] - lo[i] * dp[i - 1]) / den
    Si = np.zeros(m)
    Si[m - 1] = dp[m - 1]
    for i in range(m - 2, -1, -1):
        Si[i] = dp[i] - cp[i] * Si[i + 1]
    S[1:-1] = Si
    return S


class SplineInterpolation:
    """Natural cubic spline y(x) with the reference's field names."""

    def __init__(self, x, y):
        x = np.asarray(x, dtype=np.float64).copy()
        y = np.asarray(y, dtype=np.float64).copy()
        if x.shape != y.shape or x.ndim != 1:
            raise ValueError("x and y must be 1D arrays of the same length")
        self._x_ = x
        self._y_ = y
        self._S_full_ = natural_second_derivatives(x, y)
        self._n_ = x.shape[0]

    def _locate(self, xn):
        n = self._x_.shape[0]
        idx = np.clip(np.searchsorted(self._x_, xn, side="left") - 1, 0, n - 2)
        return idx

    def evaluate(self, x_new):
        xn = np.asarray(x_new, dtype=np.float64)
        idx = self._locate(xn)
        x, y, S = self._x_, self._y_, self._S_full_
        h = x[idx + 1] - x[idx]
        t = (xn - x[idx]) / h
        A = 1.0 - t
        B = t
        return A * y[idx] + B * y[idx + 1] + ((A**3 - A) * S[idx] + (B**3 - B) * S[idx + 1]) * (h**2) / 6.0

    def derivative(self, x_new):
        xn = np.asarray(x_new, dtype=np.float64)
        idx = self._locate(xn)
        x, y, S = self._x_, self._y_, self._S_full_
        h = x[idx + 1] - x[idx]
        d = xn - x[idx]
        b = (y[idx + 1] - y[idx]) / h - h * (S[idx + 1] + 2.0 * S[idx]) / 6.0
        c = S[idx] / 2.0
        dd = (S[idx + 1] - S[idx]) / (6.0 * h)
        return b + 2.0 * c * d + 3.0 * dd * d**2
