"""The discrete adjoint (deb_adjoint.cuh) on the CPU: the host build of the
kernel's code checked piece by piece and end to end.

* the bilinear form B(r, Y) with the coefficient function phi reproduces
  r^T f(tau, Y) of the kernel's RHS and its a-column exactly (to rounding);
* J^T x equals the transpose of the oracle's dense forward-mode Jacobian,
  (dJ/da)^T x its finite difference in a;
* W^-T b from the structured factors equals numpy's dense solve of W^T;
* the adjoint's output conversion equals the kernel's;
* one Rosenbrock step's adjoint equals central differences of the step in
  y0, t0, dt and theta (the map is linear in y0 except through a, so exact
  steps are used there);
* the whole solve backwards (checkpoints, recomputed segments, outputs by
  in-step interpolation or landing steps, tau_start, ICs and output times)
  equals central differences of the recorded-step replay -- the
  frozen-step-sequence derivative jax.jacfwd takes through diffrax
  (perturbations.py:765) -- within 1e-6 of each parameter's largest
  |d ln P / d theta| (observed ~1e-8).
"""
import numpy as np
import pytest

import oracle
import discoeb_gb300.tables as tb
from discoeb_gb300 import tables_gpu
from discoeb_gb300.gradient import perturbed_params
from discoeb_gb300.workloads import fiducial_mnu_param
from native import harness as H

DIMS = (8, 8, 10, 8, 3)
WIDE = (12, 12, 17, 17, 15)


@pytest.fixture(scope="module")
def sets():
    base = fiducial_mnu_param()
    pert = perturbed_params(base)
    flat = [base] + [q for (_, _, a, b) in pert for q in (a, b)]
    lead = tables_gpu.follow_nominal(1, len(flat) - 1)
    tabs3, _ = tables_gpu.evolve_background_tables_host(flat, 3, leader=lead)
    tabs15, _ = tables_gpu.evolve_background_tables_host(flat, 15, leader=lead)
    eps = np.array([e for (_, e, _, _) in pert])
    return tabs3, tabs15, eps


def _states(blob, dims, k):
    """An early state (perturbed ICs) and a late state (a ~ 0.3, from stepping)."""
    tau0, y0 = oracle.initial(blob, dims, k, 1e4)
    rng = np.random.default_rng(0)
    ye = y0 * (1 + 0.1 * rng.standard_normal(y0.shape)) + 1e-3 * rng.standard_normal(y0.shape)
    ye[0] = y0[0] * 300.0
    y, t = y0.copy(), tau0
    while t < 8000.0:
        y = H.step_adj(blob[None], np.zeros(0), dims, k, t, 0.05 * t, y)
        t *= 1.05
    return [(tau0 * 300.0, ye), (t, y)]


def test_lead_row_inverse_tables():
    assert H.lib().h_adj_ok() == 1


@pytest.mark.parametrize("dims,k", [(DIMS, 0.3), (WIDE, 0.02)])
def test_bilinear_form_reproduces_the_rhs(sets, dims, k):
    blob = (sets[0] if dims[4] == 3 else sets[1])[0]
    rng = np.random.default_rng(1)
    for tau, y in _states(blob, dims, k):
        x = rng.standard_normal(y.shape)
        phi, xf, dphi, xdf, dphit = H.adj_phi(blob, dims, k, tau, x, y)
        assert abs(phi - xf) <= 1e-12 * max(abs(xf), 1e-300)
        assert abs(dphi - xdf) <= 1e-11 * max(abs(xdf), 1e-300)
        ht = 1e-5 * tau
        fd = x @ (H.rhs(blob, dims, k, tau + ht, y)[0] - H.rhs(blob, dims, k, tau - ht, y)[0]) / (2 * ht)
        assert abs(dphit - fd) <= 1e-6 * max(abs(fd), 1e-300)


@pytest.mark.parametrize("dims,k", [(DIMS, 0.3), (WIDE, 0.02)])
def test_transposed_jacobian_matches_dense_oracle(sets, dims, k):
    blob = (sets[0] if dims[4] == 3 else sets[1])[0]
    rng = np.random.default_rng(2)
    for tau, y in _states(blob, dims, k):
        x = rng.standard_normal(y.shape)
        J, _ = oracle.jacobian(blob, dims, k, tau, y)
        ref = J.T @ x
        z = H.adj_jt(blob, dims, k, tau, x, y)
        assert np.abs(z - ref).max() <= 1e-12 * np.abs(ref).max()
        h = 1e-6 * y[0]
        yp, ym = y.copy(), y.copy()
        yp[0] += h
        ym[0] -= h
        dref = ((oracle.jacobian(blob, dims, k, tau, yp)[0] - oracle.jacobian(blob, dims, k, tau, ym)[0]) / (2 * h)).T @ x
        zd = H.adj_jt(blob, dims, k, tau, x, y, der=True)
        assert np.abs(zd[1:] - dref[1:]).max() <= 1e-7 * np.abs(dref).max()


@pytest.mark.parametrize("dims,k", [(DIMS, 0.3), (WIDE, 0.02)])
def test_transposed_w_solve_matches_dense(sets, dims, k):
    blob = (sets[0] if dims[4] == 3 else sets[1])[0]
    rng = np.random.default_rng(3)
    for tau, y in _states(blob, dims, k):
        J, _ = oracle.jacobian(blob, dims, k, tau, y)
        for dt in (1e-3 * tau, 0.1 * tau):
            W = np.eye(y.shape[0]) / (0.19 * dt) - J
            b = rng.standard_normal(y.shape)
            ref = np.linalg.solve(W.T, b)
            z = H.adj_solve_wt(blob, dims, k, tau, y, dt, b)
            assert np.abs(z - ref).max() <= 1e-10 * np.abs(ref).max()


def test_output_fields_as_the_kernel_converts_them(sets):
    blob = sets[1][0]
    for _, y in _states(blob, WIDE, 0.02):
        rk, rs = H.adj_outputs_pair(blob, WIDE, 0.02, y)
        np.testing.assert_allclose(rs, rk, rtol=1e-12, atol=1e-14 * np.abs(rk).max())


def test_step_adjoint_matches_finite_differences(sets):
    tabs, _, eps = sets
    k = 0.1
    (_, _), (t, y) = _states(tabs[0], DIMS, k)
    dt = 0.05 * t
    n = y.shape[0]
    lam = np.random.default_rng(4).standard_normal(n)
    _, yb, tbv, th = H.step_adj(tabs, eps, DIMS, k, t, dt, y, lam)
    L = lambda yy, tt, dd, tb_=tabs: lam @ H.step_adj(tb_, eps, DIMS, k, tt, dd, yy)
    scale = np.sqrt(np.mean(y[1:] ** 2))
    for j in range(n):
        h = 1e-6 * abs(y[j]) if j == 0 else 1e-3 * scale
        yp, ym = y.copy(), y.copy()
        yp[j] += h
        ym[j] -= h
        fd = (L(yp, t, dt) - L(ym, t, dt)) / (2 * h)
        assert abs(fd - yb[j]) <= 1e-7 * np.abs(yb).max(), j
    ht, hd = 1e-5 * t, 1e-6 * dt
    np.testing.assert_allclose(tbv[0], (L(y, t + ht, dt) - L(y, t - ht, dt)) / (2 * ht), rtol=1e-6)
    np.testing.assert_allclose(tbv[1], (L(y, t, dt + hd) - L(y, t, dt - hd)) / (2 * hd), rtol=1e-6)
    for p in range(eps.shape[0]):
        fd = (L(y, t, dt, tabs[[1 + 2 * p]]) - L(y, t, dt, tabs[[2 + 2 * p]])) / (2 * eps[p])
        assert abs(th[p] - fd) <= 1e-6 * abs(fd) + 1e-12 * np.abs(th).max(), p


def _replay_fd(tabs, eps, k, taus, idx, kw):
    y0, _, rec, nrec = H.solve_rr(tabs[:1], 1, np.array([k]), taus[:1], record=True, lmaxg=8, lmaxgp=8, lmaxr=10,
                                  lmaxnu=8, nqmax=3, **kw)
    ys, ss, _, _ = H.solve_rr(tabs[1:], tabs.shape[0] - 1, np.array([k]), taus[1:], rec=rec, nrec=nrec, replay=True,
                              lmaxg=8, lmaxgp=8, lmaxr=10, lmaxnu=8, nqmax=3, **kw)
    assert (ss[:, 0] == 0).all()
    lp = np.log(ys[:, :, idx] ** 2)
    return y0[0], (lp[0::2] - lp[1::2]) / (2 * eps[:, None])


@pytest.mark.parametrize("step_to_outputs", [False, True])
def test_solve_adjoint_matches_replay_differences(sets, step_to_outputs):
    tabs, _, eps = sets
    a_out = np.array([0.3, 1.0])
    taus = tb.tau_of_a_blob(tabs, a_out)
    kw = dict(rtol=1e-6, atol=1e-9, max_steps=20000, step_to_outputs=step_to_outputs)
    for k in (1e-3, 0.03, 0.2):
        y0, fd = _replay_fd(tabs, eps, k, taus, 4, kw)
        for o in range(a_out.size):
            gy = np.zeros((a_out.size, 20))
            gy[o, 4] = 2.0 / y0[o, 4]
            g, y, info, st = H.adjoint(tabs, eps, k, taus, DIMS, gy, ck_cap=8, **kw)
            assert st == 0 and info[0] == 0
            np.testing.assert_array_equal(y, y0)
            assert np.abs(g - fd[:, o]).max() <= 1e-6 * np.abs(fd[:, o]).max(), (k, o, g, fd[:, o])


def test_checkpoint_thinning_does_not_change_the_gradient(sets):
    """8 or 4096 checkpoint slots: the recomputed segments give the same
    states, so the same gradient bit for bit."""
    tabs, _, eps = sets
    taus = tb.tau_of_a_blob(tabs, np.array([1.0]))
    gy = np.zeros((1, 20))
    gy[0, 4] = 1.0
    kw = dict(rtol=1e-5, atol=1e-8, max_steps=20000)
    g8, _, info8, _ = H.adjoint(tabs, eps, 0.1, taus, DIMS, gy, ck_cap=8, **kw)
    gb, _, infob, _ = H.adjoint(tabs, eps, 0.1, taus, DIMS, gy, ck_cap=4096, **kw)
    assert info8[2] > 1 and infob[2] == 1
    np.testing.assert_array_equal(g8, gb)


def test_checkpoint_caps_fit_step_counts():
    """Per-mode slots: room for a state after every recorded step with a
    margin, even, and never below 2 max_steps / SEG_CAP, so that a mode whose
    step count outgrows its slots thins them to a stride within the adjoint
    plan's segment buffer; offsets lay the modes end to end."""
    from discoeb_gb300.gradient import SEG_CAP, checkpoint_caps

    nrec = np.array([0, 10, 255, 1000, 5001])
    caps, offs, total, floor = checkpoint_caps(nrec, 8192)
    assert floor == -(-2 * 8192 // SEG_CAP)
    assert (caps % 2 == 0).all() and (caps >= floor).all() and (caps >= 1.25 * nrec).all()
    assert offs[0] == 0 and (np.diff(offs) == caps[:-1]).all() and total == int(caps.sum())
    assert (2 * 8192 / caps <= SEG_CAP).all()
