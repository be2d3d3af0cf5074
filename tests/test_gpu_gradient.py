"""GPU gradient d log P / d theta (jacfwd-style tangents of the step sequence) against the host.

* the GPU's own recorded nominal step sequence replayed by the host build of
  the kernel core for every theta +- eps table set: both sides evaluate the
  same branch-free map, so the difference quotients agree to 1e-6 of each
  parameter's largest |d log P / d theta| (rounding / eps); all outputs with
  steps landing on the output times, and the end time with the reference's
  default outputs (linear interpolation inside a step, where an interior
  output's derivative is the slope of that interpolant);
* central differences of two independent tight-tolerance oracle solves
  (rtol 1e-9): the end time with default outputs, and every output with
  steps landing on the output times, 1e-4 of the parameter's largest
  derivative (the required bar is 1e-3).
"""
import numpy as np
import pytest

import oracle
import discoeb_gb300 as deb
import discoeb_gb300.tables as tb
from discoeb_gb300.gradient import THETA, GradientProblem, evolve_backgrounds, perturbed_params
from discoeb_gb300.workloads import fiducial_mnu_param
from native import harness as H

pytestmark = pytest.mark.gpu

DIMS = dict(lmaxg=8, lmaxgp=8, lmaxr=10, lmaxnu=8, nqmax=3)


@pytest.fixture(scope="module")
def setup():
    base = fiducial_mnu_param()
    pert = perturbed_params(base)
    flat = [base] + [q for (_, _, a, b) in pert for q in (a, b)]
    bgs = evolve_backgrounds(flat, processes=1)
    return base, pert, bgs


def _gpu_and_host_replay(base, pert, bgs, a_out, step_to_outputs):
    """GPU gradient and the host replay of the GPU's recorded step sequence."""
    k = np.geomspace(1e-3, 1.0, 6)
    kw = dict(rtol=1e-6, atol=1e-9, max_steps=20000, step_to_outputs=step_to_outputs)
    gp = GradientProblem([base], [bgs], [pert], k, a_out, **kw, **DIMS)
    _, Dd = gp.run()
    gp.check()
    D = Dd.reshape(6, len(a_out), len(THETA)).cpu().numpy()
    rec, nrec = gp.d_rec.cpu().numpy(), gp.d_nrec.cpu().numpy()
    assert (nrec > 0).all()
    tabs = np.stack([tb.pack_cosmology(q, 3) for q in bgs[1:]])
    taus = np.stack([tb.tau_of_a(q, a_out) for q in bgs[1:]])
    ys, ss, _, _ = H.solve_rr(tabs, len(bgs) - 1, k, taus, rec=np.ascontiguousarray(rec), nrec=np.ascontiguousarray(nrec),
                              replay=True, **kw, **DIMS)
    assert (ss[:, 0] == 0).all()
    lp = np.log(ys[..., 4] ** 2).reshape(len(bgs) - 1, 6, len(a_out))
    return D, lp, k


def test_gradient_matches_host_replay_of_the_gpu_record(setup):
    base, pert, bgs = setup
    a_out = np.linspace(0.2, 1.0, 8)
    D, lp, k = _gpu_and_host_replay(base, pert, bgs, a_out, True)
    for j, (name, eps, _, _) in enumerate(pert):
        g = (lp[2 * j] - lp[2 * j + 1]) / (2 * eps)
        col = THETA.index(name)
        assert np.abs(D[:, :, col] - g).max() <= 1e-6 * np.abs(g).max(), name
    # analytic parameters (perturbations.py:1123)
    np.testing.assert_allclose(D[:, :, THETA.index("A_s")], 1.0 / base["A_s"])
    np.testing.assert_allclose(D[:, :, THETA.index("n_s")], np.log(k / 0.05)[:, None] * np.ones((1, 8)))


def test_default_output_semantics_match_host_replay_of_the_gpu_record(setup):
    """Reference output semantics (interpolation inside the step): every
    output, including the interpolant slopes, equals the host replay."""
    base, pert, bgs = setup
    a_out = np.linspace(0.2, 1.0, 8)
    D, lp, k = _gpu_and_host_replay(base, pert, bgs, a_out, False)
    for j, (name, eps, _, _) in enumerate(pert):
        g = (lp[2 * j] - lp[2 * j + 1]) / (2 * eps)
        col = THETA.index(name)
        assert np.abs(D[:, :, col] - g).max() <= 1e-6 * np.abs(g).max(), name


def test_end_time_gradient_matches_tight_oracle_differences(setup):
    base, pert, bgs = setup
    P, D, k = deb.evolve_perturbations_grad(params=base, aexp_out=[1.0], kmin=1e-3, kmax=1.0, num_k=5, rtol=1e-6,
                                            atol=1e-9, max_steps=20000, backgrounds=[bgs], **DIMS)
    for j, (name, eps, _, _) in enumerate(pert):
        bp, bm = bgs[1 + 2 * j], bgs[2 + 2 * j]
        yp, sp = oracle.solve(tb.pack_cosmology(bp, 3), k, tb.tau_of_a(bp, [1.0]), rtol=1e-9, atol=1e-12,
                              max_steps=2000000, **DIMS)
        ym, sm = oracle.solve(tb.pack_cosmology(bm, 3), k, tb.tau_of_a(bm, [1.0]), rtol=1e-9, atol=1e-12,
                              max_steps=2000000, **DIMS)
        assert (sp[:, 0] == 0).all() and (sm[:, 0] == 0).all()
        gt = (np.log(yp[:, 0, 4] ** 2) - np.log(ym[:, 0, 4] ** 2)) / (2 * eps)
        col = THETA.index(name)
        assert np.abs(D[:, 0, col] - gt).max() <= 1e-4 * np.abs(gt).max(), name


def test_interior_output_gradient_matches_tight_oracle_differences(setup):
    """All 8 outputs in a = [0.2, 1] with steps landing on the output times:
    GPU gradient (rtol 1e-6) against central differences of two rtol 1e-9
    oracle solves run the same way."""
    base, pert, bgs = setup
    a_out = np.linspace(0.2, 1.0, 8)
    P, D, k = deb.evolve_perturbations_grad(params=base, aexp_out=a_out, kmin=1e-3, kmax=1.0, num_k=4, rtol=1e-6,
                                            atol=1e-9, max_steps=20000, backgrounds=[bgs], step_to_outputs=True, **DIMS)
    for j, (name, eps, _, _) in enumerate(pert[:3]):
        bp, bm = bgs[1 + 2 * j], bgs[2 + 2 * j]
        yp, sp = oracle.solve(tb.pack_cosmology(bp, 3), k, tb.tau_of_a(bp, a_out), rtol=1e-9, atol=1e-12,
                              max_steps=2000000, step_to_outputs=True, **DIMS)
        ym, sm = oracle.solve(tb.pack_cosmology(bm, 3), k, tb.tau_of_a(bm, a_out), rtol=1e-9, atol=1e-12,
                              max_steps=2000000, step_to_outputs=True, **DIMS)
        assert (sp[:, 0] == 0).all() and (sm[:, 0] == 0).all()
        gt = (np.log(yp[..., 4] ** 2) - np.log(ym[..., 4] ** 2)) / (2 * eps)
        col = THETA.index(name)
        assert np.abs(D[:, :, col] - gt).max() <= 1e-4 * np.abs(gt).max(), name


def test_fisher_matrix_is_symmetric_and_positive(setup):
    base, pert, bgs = setup
    P, D, k = deb.evolve_perturbations_grad(params=base, aexp_out=np.linspace(0.2, 1.0, 8), kmin=1e-3, kmax=1.0,
                                            num_k=16, rtol=1e-5, atol=1e-8, max_steps=20000, backgrounds=[bgs], **DIMS)
    F = deb.fisher_matrix(k, D, volume_mpc3=(1000.0 / 0.6774) ** 3)
    assert F.shape == (8, 8) and np.isfinite(F).all()
    np.testing.assert_allclose(F, F.T, rtol=1e-12)
    assert np.linalg.eigvalsh(F).min() >= -1e-8 * np.abs(F).max()


def test_autograd_function_backward_is_P_times_dlogP(setup):
    """PowerSpectrum.apply: forward equals evolve_perturbations_grad's P; the
    gradient of a weighted sum of P is sum w P d ln P / d theta."""
    import torch

    base, pert, bgs = setup
    from discoeb_gb300.gradient import THETA, _get

    opts = dict(aexp_out=[0.5, 1.0], kmin=1e-3, kmax=0.5, num_k=5, rtol=1e-5, atol=1e-8, max_steps=20000,
                backgrounds=[bgs], **DIMS)
    theta = torch.tensor([float(_get(base, n)) for n in THETA], dtype=torch.float64, device="cuda", requires_grad=True)
    P = deb.PowerSpectrum.apply(theta, base, opts)
    P0, D0, _ = deb.evolve_perturbations_grad(params=base, **opts)
    np.testing.assert_allclose(P.detach().cpu().numpy(), P0, rtol=1e-12)
    w = torch.linspace(1.0, 2.0, P.numel(), dtype=torch.float64, device="cuda").reshape(P.shape)
    (w * P).sum().backward()
    expect = np.einsum("ka,ka,kat->t", w.cpu().numpy(), P0, D0)
    np.testing.assert_allclose(theta.grad.cpu().numpy(), expect, rtol=1e-10)
