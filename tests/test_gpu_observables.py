"""Observables on the GPU against the CPU restatement (oracle/observables.py):
multipoles, Kaiser P(k, mu) with and without smoothing, smoothed P(k) and the
FFTLog correlation function, on a GPU solve of flat LCDM (128 k)."""
import numpy as np
import pytest

import oracle.observables as ob
import discoeb_gb300 as deb
import discoeb_gb300.background as bg
from discoeb_gb300 import observables as gobs
from discoeb_gb300.workloads import lcdm_massless_param

pytestmark = pytest.mark.gpu

DIMS = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=8, nqmax=3)


@pytest.fixture(scope="module")
def sol():
    p = bg.evolve_background(param=lcdm_massless_param())
    y, k, p = deb.evolve_perturbations(param=p, aexp_out=[0.5, 1.0], kmin=1e-4, kmax=1.0, num_k=128, rtol=1e-4,
                                       atol=1e-7, max_steps=20000, **DIMS)
    return p, y, k


def test_multipoles(sol):
    p, y, k = sol
    got = gobs.power_multipoles(y=y[:, -1, :], kmodes=k, b=1.7, param=p)
    want = ob.power_multipoles(y[:, -1, :], k, 1.7, p)
    for g, w in zip(got, want):
        np.testing.assert_allclose(g, w, rtol=1e-12, atol=1e-14 * np.abs(w).max())
    # all outputs at once
    got2 = gobs.power_multipoles(y=y, kmodes=k, b=1.7, param=p)
    np.testing.assert_allclose(got2[0][:, -1], got[0], rtol=1e-14)


@pytest.mark.parametrize("mu_sampling", [True, False])
@pytest.mark.parametrize("smooth", [None, 0.4])
def test_kaiser(sol, mu_sampling, smooth):
    p, y, k = sol
    got, mu = gobs.power_Kaiser(y=y[:, -1, :], kmodes=k, bias=2.0, mu_sampling=mu_sampling, smooth_dlogk=smooth,
                                nmu=9, param=p)
    want, mu_w = ob.power_Kaiser(y[:, -1, :], k, 2.0, 9, p, mu_sampling=mu_sampling, smooth_dlogk=smooth)
    np.testing.assert_allclose(mu, mu_w, rtol=0, atol=1e-15)
    np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-14 * np.abs(want).max())


def test_power_smoothed(sol):
    p, y, k = sol
    for dlogk in (0.3, 1.0):
        got = gobs.get_power_smoothed(k=k, y=y[:, -1, :], dlogk=dlogk, idx=4, param=p)
        want = ob.get_power_smoothed(k, y[:, -1, :], dlogk, 4, p)
        np.testing.assert_allclose(got, want, rtol=1e-11)


@pytest.mark.parametrize("ell", [0, 2, 4])
def test_fftlog(sol, ell):
    p, y, k = sol
    P = deb.get_power(k=k, y=y[:, -1, :], idx=4, param=p)
    xi, r = gobs.get_xi_from_P(k=k, Pk=P, N=len(k), ell=ell)
    xi_w, r_w = ob.get_xi_from_P(k, P, ell=ell)
    np.testing.assert_allclose(r, r_w, rtol=1e-14)
    np.testing.assert_allclose(xi, xi_w, rtol=0, atol=1e-9 * np.abs(xi_w).max())


def test_tensor_in_tensor_out(sol):
    import torch

    p, y, k = sol
    yt = torch.as_tensor(y[:, -1, :]).cuda()
    kt = torch.as_tensor(k).cuda()
    P0, P2, P4 = gobs.power_multipoles(y=yt, kmodes=kt, b=1.0, param=p)
    assert torch.is_tensor(P0) and P0.is_cuda
    np.testing.assert_allclose(P4.cpu().numpy(), ob.power_multipoles(y[:, -1, :], k, 1.0, p)[2], rtol=1e-12)
