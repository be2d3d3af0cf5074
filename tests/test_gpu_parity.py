"""GPU parity: the CUDA path through the C ABI against the oracle.

Tolerances (FP64 on both sides, same method and controller):
  * P(k) and matter fields at the end time: 1e-6 relative at rtol 1e-3
    (n=80) and 1e-5 at rtol 1e-5 (n=323).  Observed differences are ~1e-8
    except where a rounding-level difference flips one accept/reject
    decision near err = 1 (cond(W) reaches 1e15 in tight coupling), after
    which that mode's step sequence and its discretisation error differ;
  * interior outputs use the reference's linear in-step interpolation, so
    they agree to the interpolation error of the step: 1e-3 relative;
  * W^{-1} b structured vs dense on the device: 1e-10 relative.
"""
import numpy as np
import pytest

import oracle
import discoeb_gb300 as deb
import discoeb_gb300.background as bg
import discoeb_gb300.tables as tb
from discoeb_gb300.workloads import fiducial_mnu_param, lcdm_massless_param, sample_cosmologies

pytestmark = pytest.mark.gpu

LCDM = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=8, nqmax=3)
FID = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=17, nqmax=15)


@pytest.fixture(scope="module")
def lcdm():
    return bg.evolve_background(param=lcdm_massless_param())


@pytest.fixture(scope="module")
def fid():
    return bg.evolve_background(param=fiducial_mnu_param())


def _power(p, k, y):
    return 2 * np.pi**2 * p["A_s"] * (k / p.get("k_p", 0.05)) ** (p["n_s"] - 1) * k**-3 * y**2


def test_lcdm_64_modes_vs_oracle(lcdm):
    """Flat LCDM, 64 k in [1e-4, 1], n=80, rtol 1e-3 / atol 1e-6, a=1."""
    y, k, par = deb.evolve_perturbations(param=dict(lcdm), aexp_out=[1.0], kmin=1e-4, kmax=1.0, num_k=64,
                                         rtol=1e-3, atol=1e-6, **LCDM)
    assert y.shape == (64, 1, 20) and par["nout"] == 1
    yo, so = oracle.solve(tb.pack_cosmology(lcdm, 3), k, tb.tau_of_a(lcdm, [1.0]), rtol=1e-3, atol=1e-6, **LCDM)
    assert (so[:, 0] == 0).all()
    P = deb.get_power(k=k, y=y[:, 0, :], idx=4, param=lcdm)
    np.testing.assert_allclose(P, _power(lcdm, k, yo[:, 0, 4]), rtol=1e-6)
    for f in (6, 8, 10):
        np.testing.assert_allclose(y[:, 0, f], yo[:, 0, f], rtol=1e-6, atol=1e-9 * np.abs(yo[:, 0, f]).max())


def test_massive_nu_de_fluid_vs_oracle(fid):
    """m_nu=0.06 eV, nq=15, lmaxnu=17 (n=323), w0=-0.9, wa=0.1, rtol 1e-5; 24 modes over [1e-4, 10]."""
    k = np.geomspace(1e-4, 10.0, 24)
    blob = tb.pack_cosmology(fid, 15)
    tau = tb.tau_of_a(fid, [1.0])
    y, st = deb.solve(blob[None], k, tau[None], rtol=1e-5, atol=1e-5, return_stats=True, **FID)
    yo, so = oracle.solve(blob, k, tau, rtol=1e-5, atol=1e-5, **FID)
    assert (st["status"] == 0).all() and (so[:, 0] == 0).all()
    np.testing.assert_allclose(y[:, 0, 4] ** 2, yo[:, 0, 4] ** 2, rtol=1e-5)
    np.testing.assert_allclose(y[:, 0, 6], yo[:, 0, 6], rtol=1e-5)
    np.testing.assert_allclose(y[:, 0, 16], yo[:, 0, 16], rtol=1e-3)


def test_batched_cosmologies_vs_oracle():
    """4 sampled cosmologies x 8 modes in one launch (per-mode cosmology index)."""
    params, _ = sample_cosmologies(4, seed=7)
    ps = [bg.evolve_background(param=p) for p in params]
    y, k = deb.evolve_perturbations_multi(params=ps, aexp_out=[1.0], kmin=1e-3, kmax=1.0, num_k=8, rtol=1e-5,
                                          atol=1e-5, **FID)
    assert y.shape == (4, 8, 1, 20)
    for c, p in enumerate(ps):
        yo, so = oracle.solve(tb.pack_cosmology(p, 15), k, tb.tau_of_a(p, [1.0]), rtol=1e-5, atol=1e-5, **FID)
        assert (so[:, 0] == 0).all()
        np.testing.assert_allclose(y[c, :, 0, 4] ** 2, yo[:, 0, 4] ** 2, rtol=1e-5)


def test_dense_path_equals_structured(lcdm):
    k = np.geomspace(1e-3, 0.5, 16)
    blob = tb.pack_cosmology(lcdm, 3)
    tau = tb.tau_of_a(lcdm, [1.0])
    ys = deb.solve(blob[None], k, tau[None], rtol=1e-6, atol=1e-9, max_steps=20000, linear_solver="structured", **LCDM)
    yd = deb.solve(blob[None], k, tau[None], rtol=1e-6, atol=1e-9, max_steps=20000, linear_solver="dense", **LCDM)
    np.testing.assert_allclose(ys[:, 0, 4], yd[:, 0, 4], rtol=1e-6)


def test_interior_outputs_and_return_full(fid):
    """8 outputs in a=[0.2, 1]; full state returned; interior outputs carry the
    reference's linear in-step interpolation (perturbations.py:770).  Late
    steps span tens of percent in tau, so that interpolation is only good to
    ~1 % (a grows like tau^2); where a rounding-level difference moves the
    steps of a mode the interpolation error moves with them, hence 1e-2.
    Step-landing outputs are compared tightly in the step_to_outputs test."""
    a_out = np.linspace(0.2, 1.0, 8)
    k = np.geomspace(1e-3, 1.0, 8)
    blob = tb.pack_cosmology(fid, 15)
    tau = tb.tau_of_a(fid, a_out)
    y = deb.solve(blob[None], k, tau[None], rtol=1e-5, atol=1e-5, return_full=True, **FID)
    yo, so = oracle.solve(blob, k, tau, rtol=1e-5, atol=1e-5, return_full=True, **FID)
    assert y.shape == yo.shape == (8, 8, 323)
    np.testing.assert_allclose(y[:, :, 0], yo[:, :, 0], rtol=1e-2)        # a(tau_out)
    np.testing.assert_allclose(y[:, :, 3], yo[:, :, 3], rtol=1e-2)        # delta_c
    np.testing.assert_allclose(y[:, -1, 3], yo[:, -1, 3], rtol=1e-5)      # delta_c at the end time


def test_failure_statuses_are_reported_not_trapped(lcdm):
    """Host-made failures: w0 = -1 exactly (1/(1+w) in the DE equation),
    max_steps reached, k <= 0.  Each returns a status; the context stays usable."""
    p1 = bg.evolve_background(param=lcdm_massless_param(w0=-1.0))
    k = np.array([0.01, 0.1])
    _, st = deb.solve(tb.pack_cosmology(p1, 3)[None], k, tb.tau_of_a(p1, [1.0])[None], rtol=1e-3, atol=1e-6,
                      throw=False, return_stats=True, **LCDM)
    assert (st["status"] == 3).all()
    blob = tb.pack_cosmology(lcdm, 3)
    tau = tb.tau_of_a(lcdm, [1.0])
    _, st = deb.solve(blob[None], np.array([0.1]), tau[None], rtol=1e-3, atol=1e-6, max_steps=4, throw=False,
                      return_stats=True, **LCDM)
    assert st["status"][0] == 1 and st["steps"][0].sum() == 4
    y, st = deb.solve(blob[None], np.array([-1.0, 0.1]), tau[None], rtol=1e-3, atol=1e-6, throw=False,
                      return_stats=True, **LCDM)
    assert st["status"][0] == 4 and st["status"][1] == 0 and np.isnan(y[0]).all()
    with pytest.raises(RuntimeError):
        deb.solve(blob[None], np.array([0.1]), tau[None], rtol=1e-3, atol=1e-6, max_steps=4, **LCDM)
    # the device is still healthy
    y2 = deb.solve(blob[None], np.array([0.1]), tau[None], rtol=1e-3, atol=1e-6, **LCDM)
    assert np.isfinite(y2).all()


def test_empty_and_single_mode(lcdm):
    blob = tb.pack_cosmology(lcdm, 3)
    tau = tb.tau_of_a(lcdm, [1.0])
    y = deb.solve(blob[None], np.zeros(0), tau[None], **LCDM)
    assert y.shape == (0, 1, 20)
    y = deb.solve(blob[None], np.array([0.02]), tau[None], rtol=1e-3, atol=1e-6, **LCDM)
    assert y.shape == (1, 1, 20) and np.isfinite(y).all()


def test_get_power_matches_formula(lcdm):
    k = np.geomspace(1e-4, 1, 5)
    y = np.random.default_rng(3).standard_normal((5, 3, 20))
    P = deb.get_power(k=k, y=y, idx=6, param=lcdm)
    assert P.shape == (5, 3)
    np.testing.assert_allclose(P, _power(lcdm, k[:, None], y[:, :, 6]), rtol=1e-14)


def test_reference_test_cosmology_vs_class(test_cosmology):
    """The reference's own CLASS check on the GPU path: P_bc(k) at a=0.01 within
    5e-3, lmax 31, nqmax 5, 512 modes, as tests/test_perturbations.py:95-109
    (the small_kmax variant, k in [1e-5, 10]) with the per-mode tolerance
    rtol=atol=1e-5 of tests/test_perturbations.py:128-134.

    The k <= 100 variant is not reproduced: for k > 0.07 aH(tau_min) ~ 52/Mpc
    the start-time bisection (perturbations.py:678) has no sign change because
    the tau table's first knot sits at the second sampling point
    (thermodynamics_recfast.py:452,494-499); such modes start at tau ~ 32 Mpc
    and need > 1e4 steps, beyond that test's max_steps=2048, in the reference
    algorithm as in this one."""
    import json, os
    g = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "class_pkbc_a0p01.json")))
    kc, Pc = np.array(g["k"]), np.array(g["Pkbc"])
    y, k, _ = deb.evolve_perturbations(param=dict(test_cosmology), aexp_out=[0.01], kmin=1e-5, kmax=1e1, num_k=512,
                                       lmaxg=31, lmaxgp=31, lmaxr=31, lmaxnu=31, nqmax=5, max_steps=2048,
                                       rtol=1e-5, atol=1e-5)
    P = deb.get_power(k=k, y=y[:, -1, :], idx=6, param=test_cosmology)
    m = (kc >= 1e-5) & (kc <= 1e1)
    np.testing.assert_allclose(np.interp(kc[m], k, P), Pc[m], rtol=5e-3)


@pytest.mark.parametrize("exec_mode", ["lane", "warp"])
def test_execution_modes_agree_with_oracle(fid, exec_mode):
    """One thread per mode (state interleaved in global memory) and one warp
    per mode (state in shared memory) run the same algorithm."""
    k = np.geomspace(1e-4, 10.0, 40)
    blob = tb.pack_cosmology(fid, 15)
    tau = tb.tau_of_a(fid, [1.0])
    y, st = deb.solve(blob[None], k, tau[None], rtol=1e-5, atol=1e-5, max_steps=20000, return_stats=True,
                      exec_mode=exec_mode, **FID)
    yo, so = oracle.solve(blob, k, tau, rtol=1e-5, atol=1e-5, max_steps=20000, **FID)
    assert (st["status"] == 0).all()
    # 1e-4: at rtol = atol = 1e-5 a single flipped accept/reject moves a
    # high-k mode by up to ~1e-4 (its own discretisation error)
    np.testing.assert_allclose(y[:, 0, 4] ** 2, yo[:, 0, 4] ** 2, rtol=1e-4)
    np.testing.assert_allclose(y[:, 0, 6], yo[:, 0, 6], rtol=1e-4)
    assert abs(int(st["steps"][:, 0].sum()) - int(so[:, 1].sum())) <= 0.02 * so[:, 1].sum()


@pytest.mark.parametrize("exec_mode", ["lane", "warp"])
def test_dense_path_both_modes(lcdm, exec_mode):
    k = np.geomspace(1e-3, 0.5, 8)
    blob = tb.pack_cosmology(lcdm, 3)
    tau = tb.tau_of_a(lcdm, [1.0])
    ys = deb.solve(blob[None], k, tau[None], rtol=1e-4, atol=1e-7, max_steps=20000, exec_mode=exec_mode, **LCDM)
    yd = deb.solve(blob[None], k, tau[None], rtol=1e-4, atol=1e-7, max_steps=20000, exec_mode=exec_mode,
                   linear_solver="dense", **LCDM)
    np.testing.assert_allclose(ys[:, 0, 4], yd[:, 0, 4], rtol=1e-5)


def test_step_to_outputs_interior_outputs_vs_oracle(fid):
    """With steps landing on the output times, interior outputs are step ends
    (no interpolation): P(k) at 8 scale factors agrees with the oracle run
    the same way."""
    a_out = np.linspace(0.2, 1.0, 8)
    k = np.geomspace(1e-3, 1.0, 8)
    blob = tb.pack_cosmology(fid, 15)
    tau = tb.tau_of_a(fid, a_out)
    y = deb.solve(blob[None], k, tau[None], rtol=1e-5, atol=1e-5, max_steps=20000, step_to_outputs=True, **FID)
    yo, so = oracle.solve(blob, k, tau, rtol=1e-5, atol=1e-5, max_steps=20000, step_to_outputs=True, **FID)
    assert (so[:, 0] == 0).all()
    np.testing.assert_allclose(y[:, :, 4] ** 2, yo[:, :, 4] ** 2, rtol=1e-4)


def test_queue_order_does_not_change_results(fid):
    """Any permutation handed to deb_plan_set_order gives bit-identical outputs,
    status and step counts (only which warp takes which mode changes)."""
    import torch
    from discoeb_gb300 import perturbations as pt

    k = np.geomspace(1e-4, 10.0, 40)
    blob = tb.pack_cosmology(fid, 15)
    tau = tb.tau_of_a(fid, [0.5, 1.0])
    prob = deb.DeviceProblem(blob[None], k, tau[None], **FID)
    cfg = pt._cfg(1e-5, 1e-5, 0.25, 0.80, 0.0, 20.0, 0.3, 20000)
    runs = []
    for order in (None, np.random.default_rng(3).permutation(40).astype(np.int32), np.arange(40)[::-1].copy()):
        prob.order = None if order is None else torch.as_tensor(order).cuda()
        prob.launch(cfg)
        torch.cuda.synchronize()
        runs.append((prob.y.cpu().numpy().copy(), prob.status.cpu().numpy().copy(), prob.steps.cpu().numpy().copy()))
    for y, st, sp in runs[1:]:
        assert np.array_equal(y, runs[0][0]) and np.array_equal(st, runs[0][1]) and np.array_equal(sp, runs[0][2])
    prob.reorder_by_steps()
    prob.launch(cfg)
    torch.cuda.synchronize()
    assert np.array_equal(prob.y.cpu().numpy(), runs[0][0])


def test_more_chains_and_gather_entries_than_lanes():
    """nqmax 30: 33 chains and 36-entry gather lists exceed the 32 lanes of a
    warp, so every lane-strided loop over them takes two passes; small lmax
    keeps the oracle's dense LU quick (nvar 246).  Six modes at rtol 1e-6."""
    p = bg.evolve_background(param=fiducial_mnu_param())
    dims = dict(lmaxg=8, lmaxgp=8, lmaxr=8, lmaxnu=6, nqmax=30)
    k = np.geomspace(1e-3, 1.0, 6)
    blob = tb.pack_cosmology(p, 30)
    tau = tb.tau_of_a(p, [1.0])
    y, st = deb.solve(blob[None], k, tau[None], rtol=1e-6, atol=1e-6, return_stats=True, max_steps=20000, **dims)
    yo, so = oracle.solve(blob, k, tau, rtol=1e-6, atol=1e-6, max_steps=20000, **dims)
    assert (st["status"] == 0).all() and (so[:, 0] == 0).all()
    np.testing.assert_allclose(y[:, 0, 4], yo[:, 0, 4], rtol=1e-5)
    np.testing.assert_allclose(y[:, 0, 8], yo[:, 0, 8], rtol=1e-5, atol=1e-9 * np.abs(yo[:, 0, 8]).max())


def test_config4_hierarchy_against_the_oracle():
    """lmax 32 everywhere and 30 momentum bins (nvar 1098, the large batched
    workload's hierarchy) at rtol 1e-6, three low-k modes and two outputs,
    against the oracle's dense-LU solve.  At this size a mode's 16 vectors
    do not fit shared memory with two modes per SM, so the kernel runs its
    global stage-vector shape."""
    from discoeb_gb300.workloads import sample_cosmologies

    p = bg.evolve_background(param=sample_cosmologies(1, seed=7)[0][0])
    d4 = dict(lmaxg=32, lmaxgp=32, lmaxr=32, lmaxnu=32, nqmax=30)
    assert deb.nvar(**d4) == 1098
    k = np.array([1e-5, 3e-5, 1e-4])
    blob = tb.pack_cosmology(p, 30)
    tau = tb.tau_of_a(p, [0.5, 1.0])
    y, st = deb.solve(blob[None], k, tau[None], rtol=1e-6, atol=1e-6, return_stats=True, max_steps=4000, **d4)
    yo, so = oracle.solve(blob, k, tau, rtol=1e-6, atol=1e-6, max_steps=4000, **d4)
    assert (st["status"] == 0).all() and (so[:, 0] == 0).all()
    np.testing.assert_allclose(y[:, 1, 4], yo[:, 1, 4], rtol=1e-6)
    np.testing.assert_allclose(y[:, :, 4], yo[:, :, 4], rtol=1e-4)
    for f in (8, 10, 12):
        np.testing.assert_allclose(y[:, 1, f], yo[:, 1, f], rtol=1e-6, atol=1e-9 * np.abs(yo[:, 1, f]).max())
