"""The discrete adjoint on the GPU (deb_forward_record_ckpt + deb_adjoint).

* against the GPU's own replay of the recorded steps on the theta +- eps
  tables (central differences of the same frozen-step map, the derivative
  jax.jacfwd takes through diffrax at perturbations.py:765), each side on
  the same tables, at eps = 1e-4 and 3e-5 theta: 1e-6 of each parameter's
  largest derivative -- on the small hierarchy at one output, at eight
  outputs with steps landing on them, at four interpolated outputs, and at
  nvar 323 with 128 k and 8 outputs (steps landing on the outputs), the
  gradient workload of the fiducial cosmology.  Where a recorded step end
  lies within a few eps of an output time the two perturbed solves order
  them differently and the replay's quotient straddles a kink of the
  replayed map; such (mode, output) pairs are left out of that eps's
  comparison (a small fraction, asserted), while the adjoint -- the
  derivative inside the nominal step, as jacfwd takes it -- has no kink.
  The tables of the theta +- eps sets follow the nominal set's RECFAST steps
  and branches, so the adjoints of the two eps agree with each other to
  1e-6 everywhere;
* the checkpoint count does not change the result (8 slots, strides up to
  a few hundred, vs a slot per step, vs slots laid out per mode from the
  step counts);
* PowerSpectrum.backward (one adjoint sweep with grad_P) against the
  contraction of the replay's Jacobian.
The host build of the same code (tests/test_adjoint_cpu.py) is not a GPU
oracle at 1e-8: CUDA's and the host compiler's rounding differ in the last
bit, and from the first steps on the two take different adaptive step
sequences -- two discrete maps whose derivatives differ by their
discretisation error.
"""
import numpy as np
import pytest

import discoeb_gb300 as deb
from discoeb_gb300.gradient import THETA, GradientProblem, perturbed_params, _get
from discoeb_gb300.workloads import fiducial_mnu_param

pytestmark = pytest.mark.gpu

DIMS = dict(lmaxg=8, lmaxgp=8, lmaxr=10, lmaxnu=8, nqmax=3)
FID = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=17, nqmax=15)


@pytest.fixture(scope="module")
def base():
    return fiducial_mnu_param()


def _kinks(gp, rs, width=3.0):
    """[nmode, nout] True where an output time lies within width * rs
    (relative) of a recorded step end other than one clipped to it: the
    replayed map may order the two differently at theta + eps and - eps."""
    rec, nrec = gp.d_rec.cpu().numpy(), gp.d_nrec.cpu().numpy()
    tau = gp.d_tau0.cpu().numpy()[gp.d_com.cpu().numpy()]
    out = np.zeros(tau.shape, dtype=bool)
    for m in range(rec.shape[0]):
        ends = rec[m, 1:nrec[m]]
        ends = ends[ends > 0]
        if ends.size:
            d = np.abs(tau[m][:, None] - ends[None, :]).min(axis=1) / tau[m]
            out[m] = d < width * rs
    return out


def _both(base, k, a_out, dims, ck_cap=32, **kw):
    """[(adjoint, replay quotients, kink mask, eps per theta)] on the tables of
    eps = 1e-4 and 3e-5 theta."""
    pairs = []
    for rs in (1e-4, 3e-5):
        pert = [perturbed_params(base, rel_step=rs)]
        ga = GradientProblem([base], "native", pert, k, a_out, method="adjoint", ck_cap=ck_cap, **kw, **dims)
        _, Da = ga.run()
        ga.check()
        gr = GradientProblem([base], "native", pert, k, a_out, method="replay", **kw, **dims)
        _, Dr = gr.run()
        gr.check()
        n_a, n_r = ga.d_nrec.cpu().numpy(), gr.d_nrec.cpu().numpy()
        np.testing.assert_array_equal(n_a, n_r)
        ra, rr = ga.d_rec.cpu().numpy(), gr.d_rec.cpu().numpy()
        for m, n in enumerate(n_a):
            np.testing.assert_array_equal(ra[m, :n], rr[m, :n])
        eps = np.full(len(THETA), np.inf)
        for (name, e, _, _) in pert[0]:
            eps[THETA.index(name)] = e
        pairs.append((Da.cpu().numpy(), Dr.cpu().numpy(), _kinks(gr, rs), eps))
    return pairs


def _close(pairs, bar, lnp_round=4e-12):
    """Within bar of each parameter's largest derivative, plus the rounding of
    the replayed ln P divided by 2 eps (a few 1e-12 after thousands of steps:
    7e-7 absolute for w_a's eps = 3e-6, 2e-7 for Omega_m's), at every (mode, output)
    that is kink-free at one eps at least (most of them, asserted); and the
    adjoints of the two eps agree everywhere."""
    mask = np.stack([p[2] for p in pairs])
    both = mask.all(axis=0)
    assert both.sum() <= max(1, 0.15 * both.size), mask.mean(axis=(1, 2))
    for j, name in enumerate(THETA):
        scale = np.abs(pairs[0][1][..., j]).max()
        err = np.stack([np.where(mk, np.nan, np.abs(Da[..., j] - Dr[..., j]) - lnp_round / (2 * eps[j]))
                        for Da, Dr, mk, eps in pairs])
        err = np.nanmin(np.where(np.isnan(err).all(axis=0), 0.0, err), axis=0)
        assert err.max() <= bar * scale, (name, err.max() / scale)
    if len(pairs) > 1:
        for j, name in enumerate(THETA):
            scale = np.abs(pairs[0][0][..., j]).max()
            assert np.abs(pairs[0][0][..., j] - pairs[1][0][..., j]).max() <= bar * scale, name


@pytest.mark.parametrize("a_out,step_ts,kmax", [([1.0], False, 1.0), (list(np.linspace(0.2, 1.0, 8)), True, 1.0),
                                                ([0.35, 0.5, 0.75, 1.0], False, 0.03)])
def test_adjoint_matches_replay_differences(base, a_out, step_ts, kmax):
    """Outputs at the end time, at step ends (steps land on them) and
    interpolated inside steps (the reference's SaveAt semantics; there the
    replay's quotient straddles a kink wherever an output time lies near a
    step end, which above k ~ 0.1 -- steps of 3e-4 tau -- is nearly every
    output, so that case stops at k = 0.03)."""
    k = np.geomspace(1e-3, kmax, 6)
    pairs = _both(base, k, a_out, DIMS, rtol=1e-6, atol=1e-9, max_steps=20000, step_to_outputs=step_ts)
    _close(pairs, 1e-6)


def test_checkpoint_count_does_not_change_the_gradient(base):
    k = np.geomspace(1e-3, 1.0, 5)
    kw = dict(rtol=1e-6, atol=1e-9, max_steps=20000)
    pert = [perturbed_params(base)]
    out = []
    for cap in (8, 20002):
        gp = GradientProblem([base], "native", pert, k, [1.0], method="adjoint", ck_cap=cap, **kw, **DIMS)
        _, D = gp.run()
        gp.check()
        out.append((D.cpu().numpy(), gp.d_ckstride.cpu().numpy()))
    assert out[0][1].max() > 1 and out[1][1].max() == 1
    scale = np.abs(out[1][0]).max(axis=(0, 1))
    assert (np.abs(out[0][0] - out[1][0]) <= 1e-9 * scale).all()
    # slots laid out per mode from the step counts: stride 1 everywhere
    gp = GradientProblem([base], "native", pert, k, [1.0], method="adjoint", ck_cap=8, **kw, **DIMS)
    gp.run()
    gp.fit_checkpoints()
    _, D = gp.run()
    gp.check()
    assert gp.d_ckstride.cpu().numpy().max() == 1 and gp.d_ckoff is not None
    assert (np.abs(D.cpu().numpy() - out[1][0]) <= 1e-9 * scale).all()


def test_adjoint_at_the_fiducial_gradient_workload(base):
    """nvar 323, 128 k in [1e-3, 1], 8 outputs a in [0.2, 1] with steps landing
    on the outputs, rtol 1e-5: the cosmology and sizes of the gradient
    workload, adjoint (8 seeds per mode) against the replay."""
    k = np.geomspace(1e-3, 1.0, 128)
    pairs = _both(base, k, list(np.linspace(0.2, 1.0, 8)), FID, rtol=1e-5, atol=1e-5, max_steps=20000,
                  step_to_outputs=True)
    _close(pairs, 1e-6)


def test_power_spectrum_backward_is_one_adjoint_sweep(base):
    import torch

    opts = dict(aexp_out=[0.5, 1.0], kmin=1e-3, kmax=0.5, num_k=5, rtol=1e-6, atol=1e-9, max_steps=20000, **DIMS)
    theta = torch.tensor([float(_get(base, n)) for n in THETA], dtype=torch.float64, device="cuda", requires_grad=True)
    P = deb.PowerSpectrum.apply(theta, base, opts)
    P0, D0, _ = deb.evolve_perturbations_grad(params=base, method="replay", **opts)
    np.testing.assert_allclose(P.detach().cpu().numpy(), P0, rtol=1e-12)
    w = torch.linspace(1.0, 2.0, P.numel(), dtype=torch.float64, device="cuda").reshape(P.shape)
    (w * P).sum().backward()
    expect = np.einsum("ka,ka,kat->t", w.cpu().numpy(), P0, D0)
    got = theta.grad.cpu().numpy()
    scale = np.abs(np.einsum("ka,ka,kat->kat", w.cpu().numpy(), P0, D0)).sum(axis=(0, 1))
    assert (np.abs(got - expect) <= 1e-6 * scale).all(), (got, expect)


def test_adjoint_reports_bad_items_and_leaves_others():
    """An invalid k gets a failed status and NaN gradients; the other modes
    are unaffected."""
    base = fiducial_mnu_param()
    k = np.array([1e-3, -1.0, 0.1])
    pert = [perturbed_params(base)]
    gp = GradientProblem([base], "native", pert, k, [1.0], method="adjoint", rtol=1e-5, atol=1e-8,
                         max_steps=20000, **DIMS)
    _, D = gp.run()
    ast = gp.d_ast.cpu().numpy()
    D = D.cpu().numpy()
    assert ast[1] != 0 and ast[0] == 0 and ast[2] == 0
    ode = [THETA.index(n) for n in gp.ode_names]
    assert np.isnan(D[1, 0, ode]).all() and np.isfinite(D[[0, 2]][:, 0, ode]).all()


def test_loglike_gradient_is_the_contracted_jacobian():
    """loglike_grad (one adjoint sweep per mode with the likelihood's
    cotangent) against sum_{k,a} -w (ln P - lnP_data) d ln P / d theta from
    the Jacobian of evolve_perturbations_grad; two cosmologies, two calls (the
    second replays the captured graph with new data)."""
    from discoeb_gb300.workloads import sample_cosmologies

    params = sample_cosmologies(2, seed=3)[0]
    a_out = [0.5, 1.0]
    kw = dict(aexp_out=a_out, kmin=1e-3, kmax=0.5, num_k=6, rtol=1e-6, atol=1e-9, max_steps=20000, **DIMS)
    P, D, k = deb.evolve_perturbations_grad(params=params, method="adjoint", **kw)
    rng = np.random.default_rng(11)
    w = rng.uniform(0.5, 2.0, size=(6, 2))
    for call in range(3):
        data = np.log(P) + 0.05 * rng.standard_normal(P.shape)
        Pl, lnL, g, _ = deb.loglike_grad(params=params, lnP_data=data, weights=w, **kw)
        np.testing.assert_allclose(Pl, P, rtol=1e-12)
        r = np.log(P) - data
        np.testing.assert_allclose(lnL, -0.5 * (w * r * r).sum(axis=(1, 2)), rtol=1e-10)
        expect = np.einsum("cka,ckat->ct", -w * r, D)
        scale = np.einsum("cka,ckat->ct", np.abs(w * r), np.abs(D))
        assert (np.abs(g - expect) <= 1e-7 * scale).all(), (call, g, expect)
