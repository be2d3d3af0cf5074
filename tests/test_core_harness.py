"""The kernel's per-mode logic (deb_core.cuh, host build) against the oracle (CPU).

deb_core.cuh is the code the CUDA kernel runs; compiling it for the host lets
its structured factorization, analytic Jacobian pieces and step control be
checked here.  The GPU tests repeat the comparisons on the device.
"""
import numpy as np
import pytest

import oracle
import discoeb_gb300.background as bg
import discoeb_gb300.tables as tb
from discoeb_gb300.workloads import fiducial_mnu_param, lcdm_massless_param
from native import harness as H

FID = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=17, nqmax=15)
LCDM = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=8, nqmax=3)


@pytest.fixture(scope="module")
def fid():
    return bg.evolve_background(param=fiducial_mnu_param())


@pytest.fixture(scope="module")
def lcdm():
    return bg.evolve_background(param=lcdm_massless_param())


def _dims(d):
    return (d["lmaxg"], d["lmaxgp"], d["lmaxr"], d["lmaxnu"], d["nqmax"])


def _state(blob, dims, k, grow=30.0, seed=1):
    t0, y0 = oracle.initial(blob, dims, k, 1e4)
    rng = np.random.default_rng(seed)
    y = y0 * (1 + 0.1 * rng.standard_normal(y0.shape)) + 1e-3 * rng.standard_normal(y0.shape)
    y[0] = y0[0] * grow
    return t0 * grow, y


@pytest.mark.parametrize("k", [1e-4, 0.05, 3.0])
def test_rhs_and_a_column(fid, k):
    dims = _dims(FID)
    blob = tb.pack_cosmology(fid, 15)
    tau, y = _state(blob, dims, k)
    f_o = oracle.rhs(blob, dims, k, tau, y)
    J, _ = oracle.jacobian(blob, dims, k, tau, y)
    f_h, jc = H.rhs(blob, dims, k, tau, y)
    np.testing.assert_allclose(f_h, f_o, rtol=1e-13, atol=1e-13 * np.abs(f_o).max())
    np.testing.assert_allclose(jc, J[:, 0], rtol=1e-12, atol=1e-13 * np.abs(J[:, 0]).max())


@pytest.mark.parametrize("k,dt_over_tau", [(1e-3, 1e-3), (0.05, 0.1), (0.3, 3.0), (3.0, 100.0)])
@pytest.mark.parametrize("dense", [False, True])
def test_structured_solve_equals_dense_solve(fid, k, dt_over_tau, dense):
    """W^{-1} b from the structured elimination (and the dense LU path)
    against numpy's dense solve of I/(gamma h) - J with the oracle's J."""
    dims = _dims(FID)
    blob = tb.pack_cosmology(fid, 15)
    tau, y = _state(blob, dims, k)
    J, _ = oracle.jacobian(blob, dims, k, tau, y)
    n = y.shape[0]
    dt = dt_over_tau * tau
    b = np.random.default_rng(7).standard_normal(n)
    W = np.eye(n) / (dt * 0.19) - J
    x_ref = np.linalg.solve(W, b)
    x = H.solve_W(blob, dims, k, tau, y, dt, b, dense=dense)
    assert np.abs(x - x_ref).max() <= 1e-10 * np.abs(x_ref).max()


def test_full_solve_matches_oracle_lcdm(lcdm):
    """64 modes, n=80, rtol 1e-3: P(k) and matter fields agree with the oracle."""
    k = np.geomspace(1e-4, 1.0, 64)
    blob = tb.pack_cosmology(lcdm, 3)
    tau = tb.tau_of_a(lcdm, [1.0])
    yo, so = oracle.solve(blob, k, tau, rtol=1e-3, atol=1e-6, **LCDM)
    yh, sh = H.solve(blob, k, tau, rtol=1e-3, atol=1e-6, **LCDM)
    assert (so[:, 0] == 0).all() and (sh[:, 0] == 0).all()
    P_o, P_h = yo[:, 0, 4] ** 2, yh[:, 0, 4] ** 2
    np.testing.assert_allclose(P_h, P_o, rtol=1e-6)
    for f in (6, 8, 10):  # delta_bc, delta_c, delta_b
        np.testing.assert_allclose(yh[:, 0, f], yo[:, 0, f], rtol=1e-6, atol=1e-9 * np.abs(yo[:, 0, f]).max())
    # step counts: same controller, rounding-level differences only
    assert abs(int(sh[:, 1].sum()) - int(so[:, 1].sum())) <= 0.02 * so[:, 1].sum()


@pytest.mark.parametrize("rtol", [1e-5, 1e-8])
def test_both_converge_to_tight_solution(lcdm, rtol):
    k = np.array([1e-3, 0.05, 0.2, 0.5])
    blob = tb.pack_cosmology(lcdm, 3)
    tau = tb.tau_of_a(lcdm, [1.0])
    ref, _ = oracle.solve(blob, k, tau, rtol=1e-10, atol=1e-13, max_steps=400000, **LCDM)
    yh, _ = H.solve(blob, k, tau, rtol=rtol, atol=rtol * 1e-3, max_steps=400000, **LCDM)
    err = np.abs(yh[:, 0, 4] ** 2 / ref[:, 0, 4] ** 2 - 1).max()
    assert err < 100 * rtol


def test_kernel_spline_matches_reference_form(fid):
    """FP32 search + FP64 fix-up gives the left-searchsorted interval exactly,
    and the polynomial form agrees with the A/B form of
    spline_interpolation.py:150-152 at knots, interior points and outside."""
    blob = tb.pack_cosmology(fid, 15)
    for which, key in enumerate(tb.SPLINE_KEYS):
        sp = fid[key]
        x0 = sp._x_
        x = np.concatenate([x0, x0[:-1] + 0.5 * np.diff(x0), np.nextafter(x0, np.inf), np.nextafter(x0, -np.inf),
                            [x0[0] - 1.0, x0[-1] + 1.0]])
        val, idx = H.spline(blob, which, x)
        ref_idx = np.clip(np.searchsorted(x0, x, side="left") - 1, 0, x0.shape[0] - 2)
        assert (idx == ref_idx).all(), key
        ref = sp.evaluate(x)
        scale = np.maximum(np.abs(sp._y_).max(), np.abs(ref))   # far extrapolation grows cubically
        assert (np.abs(val - ref) <= 1e-13 * scale).all(), key


def test_replay_on_nominal_tables_reproduces_the_solve(fid):
    """Recording the accepted steps and replaying them with the same tables
    gives the nominal outputs bit for bit (the replay takes no decisions)."""
    dims = dict(lmaxg=8, lmaxgp=8, lmaxr=10, lmaxnu=8, nqmax=3)
    a_out = np.linspace(0.2, 1.0, 8)
    k = np.geomspace(1e-3, 1.0, 5)
    b0 = tb.pack_cosmology(bg.evolve_background(param=fiducial_mnu_param()), 3)
    p0 = bg.evolve_background(param=fiducial_mnu_param())
    tau0 = tb.tau_of_a(p0, a_out)
    y0, s0, rec, nrec = H.solve_rr(b0, 1, k, tau0, record=True, rtol=1e-6, atol=1e-9, max_steps=20000, **dims)
    assert (s0[:, 0] == 0).all() and (nrec == s0[:, 1]).all()
    yr, sr, _, _ = H.solve_rr(b0, 1, k, tau0, rec=rec, nrec=nrec, replay=True, rtol=1e-6, atol=1e-9, max_steps=20000,
                              **dims)
    assert (sr[:, 0] == 0).all() and (sr[:, 1] == nrec).all()
    assert np.array_equal(yr, y0)


def test_frozen_step_gradient_at_end_time_matches_tight_differences():
    """d log P(k, a=1) / d Omega_m from the replay (rtol 1e-6; start time
    recomputed per table set, recorded step times scaled with it, final step
    at the set's own output time) against central differences of two
    independent rtol 1e-9 solves."""
    from discoeb_gb300.workloads import fiducial_mnu_param as fp
    dims = dict(lmaxg=8, lmaxgp=8, lmaxr=10, lmaxnu=8, nqmax=3)
    base = fp()
    k = np.geomspace(1e-3, 1.0, 5)
    eps = 1e-4 * base["Omegam"]
    p0 = bg.evolve_background(param=base)
    pp = bg.evolve_background(param=dict(base, Omegam=base["Omegam"] + eps))
    pm = bg.evolve_background(param=dict(base, Omegam=base["Omegam"] - eps))
    b0 = tb.pack_cosmology(p0, 3)
    _, s0, rec, nrec = H.solve_rr(b0, 1, k, tb.tau_of_a(p0, [1.0]), record=True, rtol=1e-6, atol=1e-9,
                                  max_steps=20000, **dims)
    tabs = np.stack([tb.pack_cosmology(pp, 3), tb.pack_cosmology(pm, 3)])
    taus = np.stack([tb.tau_of_a(pp, [1.0]), tb.tau_of_a(pm, [1.0])])
    ys, ss, _, _ = H.solve_rr(tabs, 2, k, taus, rec=rec, nrec=nrec, replay=True, rtol=1e-6, atol=1e-9, max_steps=20000,
                              **dims)
    g = (np.log(ys[:5, 0, 4] ** 2) - np.log(ys[5:, 0, 4] ** 2)) / (2 * eps)
    ya, _ = H.solve(tabs[0], k, taus[0], rtol=1e-9, atol=1e-12, max_steps=2000000, **dims)
    yb, _ = H.solve(tabs[1], k, taus[1], rtol=1e-9, atol=1e-12, max_steps=2000000, **dims)
    gt = (np.log(ya[:, 0, 4] ** 2) - np.log(yb[:, 0, 4] ** 2)) / (2 * eps)
    assert np.abs(g - gt).max() <= 1e-5 * np.abs(gt).max()
