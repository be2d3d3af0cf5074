"""The oracle pinned against the reference's own golden vectors (CPU only)."""
import json
import os

import numpy as np
import pytest

import oracle
import discoeb_gb300.tables as tb
from discoeb_gb300.spline import SplineInterpolation

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_class_pkbc_at_a0p01(test_cosmology):
    """P_bc(k) at a=0.01 vs CLASS within 5e-3, the reference's own bar
    (tests/test_perturbations.py:128-142: lmax 31, nqmax 5, rtol=atol=1e-5)."""
    g = json.load(open(os.path.join(GOLD, "class_pkbc_a0p01.json")))
    kc, Pc = np.array(g["k"]), np.array(g["Pkbc"])
    sel = np.arange(0, kc.shape[0], 20)
    p = test_cosmology
    blob = tb.pack_cosmology(p, 5)
    tau_out = tb.tau_of_a(p, [0.01])
    y, st = oracle.solve(blob, kc[sel], tau_out, lmaxg=31, lmaxgp=31, lmaxr=31, lmaxnu=31, nqmax=5,
                         rtol=1e-5, atol=1e-5, max_steps=2048)
    assert (st[:, 0] == 0).all()
    k = kc[sel]
    P = 2 * np.pi**2 * p["A_s"] * (k / 0.05) ** (p["n_s"] - 1) * k**-3 * y[:, 0, 6] ** 2
    np.testing.assert_allclose(P, Pc[sel], rtol=5e-3)


# Redshift bands of the RECFAST checks and the largest |x_e / fixture - 1|
# allowed in each.  Measured with this producer (reference test cosmology):
#   * z >= 3000: no integration (HeIII -> HeII by Saha, x_H = x_He = 1); the
#     tables sample a in [1e-9, 1/3001] at 12 geometric points
#     (thermodynamics_recfast.py:324-360), and the natural spline through the
#     HeII transition misses both fixtures by up to 4.9% at z ~ 5400, for any
#     integrator: the reference's own sampling cannot meet 5e-3 there;
#   * 600 <= z < 1600: the reference's GRK4A keeps every stage at t0
#     (ode_integrators_stiff.py:192-200) while the ionisation equations depend
#     on a explicitly, so x_e lags its equilibrium by up to 8%; with the
#     stages at their own times (or a tight Radau solve of the same
#     equations) the producer follows CLASS's RECFAST to 2.6e-3 through the
#     recombination peak;
#   * z < 1000: the accurate solution of the reference's equations sits
#     1.4-1.9% above CLASS's RECFAST (the equations, not the integrator).
# The two fixtures agree with each other to 1.5% at every z.
BANDS = ((8000, 1e9), (3000, 8000), (1600, 3000), (1000, 1600), (600, 1000), (200, 600), (0, 200))


def _xe_rel(p, fixture):
    g = json.load(open(os.path.join(GOLD, fixture)))
    a, xr = np.array(g["a"]), np.array(g["xe"])
    m = a <= 1.0
    xe = p["xe_of_tau_spline"].evaluate(p["tau_of_a_spline"].evaluate(a[m]))
    rel = np.abs(xe / xr[m] - 1)
    z = 1.0 / a[m] - 1.0
    return [float(rel[(z >= lo) & (z < hi)].max()) for lo, hi in BANDS]


def _assert_bands(worst, bars):
    bad = {BANDS[i]: (w, b) for i, (w, b) in enumerate(zip(worst, bars)) if not w <= b}
    assert not bad, bad


def test_recfast_equations_vs_class_recfast():
    """The ionisation equations integrated accurately (GRK4A with its stages
    at their own times) against CLASS's RECFAST (reference fixture
    RECFAST_CLASS_data.json): within the reference's 5e-3 from z = 1000 to
    3000, the recombination peak included."""
    import discoeb_gb300.background as bg
    from discoeb_gb300.workloads import reference_test_param

    p = bg.evolve_background(param=reference_test_param(), recfast_stage_times=True)
    _assert_bands(_xe_rel(p, "recfast_xe_class.json"), (3e-3, 5.5e-2, 5e-3, 5e-3, 2e-2, 2.5e-2, 2.5e-2))


def test_recfast_xe_vs_v010_baseline(test_cosmology):
    """The tables as the reference computes them (all GRK4A stages at t0)
    against the DISCO-EB v0.1.0 fixture (tests/test_background.py:71-75),
    band by band at what this algorithm reaches (see BANDS)."""
    _assert_bands(_xe_rel(test_cosmology, "recfast_xe_v010.json"), (3e-3, 5.5e-2, 1.5e-2, 8e-2, 8e-2, 1.2e-2, 4e-2))
    _assert_bands(_xe_rel(test_cosmology, "recfast_xe_class.json"), (3e-3, 5.5e-2, 5e-3, 8.5e-2, 9e-2, 1.2e-2, 4e-2))


def test_recfast_recombination_gap_is_the_frozen_stage_time():
    """With the stages at their own times the gap to the v0.1.0 fixture
    through recombination shrinks from ~7% to under 2%."""
    import discoeb_gb300.background as bg
    from discoeb_gb300.workloads import reference_test_param

    p = bg.evolve_background(param=reference_test_param(), recfast_stage_times=True)
    worst = _xe_rel(p, "recfast_xe_v010.json")
    assert worst[3] < 2e-2 and worst[4] < 2e-2, worst


def test_oracle_jacobian_matches_finite_differences(test_cosmology):
    dims = (12, 12, 17, 17, 15)
    blob = tb.pack_cosmology(test_cosmology, 15)
    k = 0.3
    tau0, y0 = oracle.initial(blob, dims, k, 1e4)
    rng = np.random.default_rng(0)
    y = y0 * (1 + 0.1 * rng.standard_normal(y0.shape)) + 1e-3 * rng.standard_normal(y0.shape)
    y[0] = y0[0] * 3.0
    tau = tau0 * 3.0
    J, dT = oracle.jacobian(blob, dims, k, tau, y)
    n = y.shape[0]
    for j in list(range(0, 12)) + [n - 2, n - 1]:
        h = 1e-6 * max(abs(y[j]), 1e-8)
        yp, ym = y.copy(), y.copy()
        yp[j] += h
        ym[j] -= h
        fd = (oracle.rhs(blob, dims, k, tau, yp) - oracle.rhs(blob, dims, k, tau, ym)) / (2 * h)
        scale = np.abs(J[:, j]).max() + 1e-300
        assert np.abs(fd - J[:, j]).max() <= 1e-4 * scale, j
    ht = 1e-6 * tau
    fdt = (oracle.rhs(blob, dims, k, tau + ht, y) - oracle.rhs(blob, dims, k, tau - ht, y)) / (2 * ht)
    np.testing.assert_allclose(dT, fdt, rtol=1e-5, atol=1e-12 * np.abs(fdt).max())


def test_oracle_spline_matches_host_spline(test_cosmology):
    p = test_cosmology
    blob = tb.pack_cosmology(p, 3)
    for which, key in enumerate(tb.SPLINE_KEYS):
        sp = p[key]
        x = np.sort(np.concatenate([sp._x_[:-1] + 0.37 * np.diff(sp._x_), sp._x_]))
        np.testing.assert_allclose(oracle.spline_eval(blob, which, x), sp.evaluate(x), rtol=1e-13, atol=1e-300)


def test_natural_spline_reproduces_cubic_interior():
    x = np.linspace(0.0, 2.0, 41)
    s = SplineInterpolation(x, np.sin(x))
    xx = np.linspace(0.3, 1.7, 57)
    np.testing.assert_allclose(s.evaluate(xx), np.sin(xx), atol=2e-6)
