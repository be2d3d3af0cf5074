"""Observables: the CPU restatement pinned to scipy, and the host helpers."""
import numpy as np
import pytest

import oracle.observables as ob


@pytest.mark.parametrize("w", [5, 7, 11, 31])
def test_savgol_window_equals_scipy(w):
    signal = pytest.importorskip("scipy.signal")
    np.testing.assert_allclose(ob.savgol_window(w, 3), signal.savgol_coeffs(w, 3), rtol=1e-10, atol=1e-13)


def test_product_window_equals_restatement():
    from discoeb_gb300.observables import savgol_coeffs, smoothing_window

    np.testing.assert_allclose(savgol_coeffs(11, 3), ob.savgol_window(11, 3), rtol=1e-12, atol=1e-15)
    k = np.geomspace(1e-4, 10.0, 512)
    w = smoothing_window(k, 1.0)
    assert w % 2 == 1 and abs(w - 1.0 / np.log(k[1] / k[0])) <= 1.0


def test_fftlog_of_a_gaussian_in_log_k_is_finite_and_ordered():
    k = np.geomspace(1e-4, 1e2, 256)
    P = np.exp(-np.log(k / 0.1) ** 2)
    xi, r = ob.get_xi_from_P(k, P)
    assert np.all(np.diff(r) > 0) and np.isfinite(xi).all()
