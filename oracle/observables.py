"""CPU restatement of the reference's observables -- TEST INFRASTRUCTURE ONLY.

numpy/scipy versions of ``src/discoeb/perturbations.py`` get_xi_from_P
(:1065-1098), get_power (:1101-1123), get_power_smoothed (:1126-1159),
power_Kaiser (:1162-1199) and power_multipoles (:1202-1224), with the
Savitzky-Golay filter of ``util.py:407-444``.  The FFTLog phase uses
scipy.special.loggamma, independent of the Lanczos series the GPU code
evaluates; the smoothing window is pinned to scipy.signal.savgol_coeffs by
the CPU tests.
"""
from __future__ import annotations

import numpy as np


def get_power(k, y, idx, param):
    return 2 * np.pi**2 * param["A_s"] * (k / param.get("k_p", 0.05)) ** (param["n_s"] - 1) * k ** (-3.0) * y[..., idx] ** 2


def savgol_window(window_length, polyorder):
    halflen, rem = divmod(window_length, 2)
    pos = halflen - 0.5 if rem == 0 else halflen
    x = np.arange(-pos, window_length - pos, dtype=float)[::-1]
    A = x ** np.arange(polyorder + 1).reshape(-1, 1)
    Y = np.zeros(polyorder + 1)
    Y[0] = 1.0
    return np.linalg.lstsq(A, Y, rcond=None)[0]


def get_power_smoothed(k, y, dlogk, idx, param):
    w = int(round(dlogk / (np.log(k[1]) - np.log(k[0]))))
    w += (w + 1) % 2
    Pm = get_power(k, y, idx, param)
    Pms = np.exp(np.convolve(np.log(Pm), savgol_window(w, 3), mode="same"))
    Pms[: w // 2] = Pm[: w // 2]
    Pms[-w // 2:] = Pm[-w // 2:]
    return Pms


def power_Kaiser(y, kmodes, bias, nmu, param, mu_sampling=True, smooth_dlogk=None):
    mu = np.linspace(-1, 1, nmu) if mu_sampling else np.cos(np.linspace(0, np.pi, nmu))
    if smooth_dlogk is None:
        amp = np.sqrt(2 * np.pi**2 * param["A_s"] * (kmodes / param.get("k_p", 0.05)) ** (param["n_s"] - 1) * kmodes ** (-3.0))
        d, th = amp * y[:, 4], amp * y[:, 5]
    else:
        d = np.sqrt(get_power_smoothed(kmodes, y, smooth_dlogk, 4, param))
        th = -np.sqrt(get_power_smoothed(kmodes, y, smooth_dlogk, 5, param))
    return (bias * d[:, None] - mu[None, :] ** 2 * th[:, None]) ** 2, mu


def power_multipoles(y, kmodes, b, param):
    amp = np.sqrt(2 * np.pi**2 * param["A_s"] * (kmodes / param.get("k_p", 0.05)) ** (param["n_s"] - 1) * kmodes ** (-3.0))
    d, th = amp * y[:, 4], amp * y[:, 5]
    return (b**2 * d**2 - 2 * b / 3 * d * th + th**2 / 5, -4 * b / 3 * d * th + 4 / 7 * th**2, 8 / 35 * th**2)


def get_xi_from_P(k, Pk, ell=0):
    from scipy.special import loggamma

    N = len(k)
    L = np.log(k[-1] / k[0])
    fPk = np.fft.rfft(Pk * k**1.5)
    ki = np.pi * np.arange(N // 2 + 1) / L
    theta = np.imag(loggamma((1.5 + ell) / 2 + 1j * ki))
    fPk = fPk * np.exp(2j * (theta - np.log(np.pi) * ki))
    r = 2 * np.pi / k
    xi = np.real(1j**ell * np.fft.irfft(fPk, n=N) / (2 * np.pi * r) ** 1.5)
    return xi[::-1], r[::-1]
