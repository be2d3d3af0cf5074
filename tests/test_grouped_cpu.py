"""The reference's batched variant (groups sharing one step sequence) on the CPU:
the oracle's grouped solve and the kernel's group driver built for the host.

* batch_size 1 reduces to the per-mode solve exactly (same start time, same
  error norm), for both;
* the kernel's driver agrees with the oracle's grouped solve to 1e-6 in P(k)
  (observed ~1e-9: the dense LU and the structured solve round differently,
  which can move one accept/reject decision);
* every mode of a group reports the group's step counts.
"""
import numpy as np
import pytest

import oracle
import discoeb_gb300.background as bg
import discoeb_gb300.tables as tb
from discoeb_gb300.workloads import fiducial_mnu_param
from native import harness as H

DIMS = dict(lmaxg=8, lmaxgp=8, lmaxr=10, lmaxnu=8, nqmax=3)


@pytest.fixture(scope="module")
def case():
    p = bg.evolve_background(param=fiducial_mnu_param())
    return tb.pack_cosmology(p, 3), tb.tau_of_a(p, [1.0]), np.geomspace(1e-3, 1.0, 8)


def test_batch_of_one_is_the_per_mode_solve(case):
    blob, tau, k = case
    y1, s1 = oracle.solve(blob, k, tau, rtol=1e-4, atol=1e-4, **DIMS)
    yg, sg = oracle.solve_grouped(blob, k, tau, 1, rtol=1e-4, atol=1e-4, **DIMS)
    np.testing.assert_array_equal(yg, y1)
    np.testing.assert_array_equal(sg, s1)
    yh, sh = H.solve_grouped(blob, k, tau, 1, rtol=1e-4, atol=1e-4, **DIMS)
    yp, sp = H.solve(blob, k, tau, rtol=1e-4, atol=1e-4, **DIMS)
    np.testing.assert_array_equal(yh, yp)


def test_kernel_group_driver_matches_the_oracle(case):
    blob, tau, k = case
    yo, so = oracle.solve_grouped(blob, k, tau, 4, rtol=1e-4, atol=1e-4, **DIMS)
    yh, sh = H.solve_grouped(blob, k, tau, 4, rtol=1e-4, atol=1e-4, **DIMS)
    assert (so[:, 0] == 0).all() and (sh[:, 0] == 0).all()
    np.testing.assert_allclose(yh[:, 0, 4] ** 2, yo[:, 0, 4] ** 2, rtol=1e-6)
    for g in range(2):
        assert len(set(map(tuple, sh[4 * g:4 * g + 4, 1:]))) == 1
        assert len(set(map(tuple, so[4 * g:4 * g + 4, 1:]))) == 1
    # sharing a step sequence is a different discretisation from per-mode steps
    y1, _ = oracle.solve(blob, k, tau, rtol=1e-4, atol=1e-4, **DIMS)
    assert np.abs(yo[:, 0, 4] / y1[:, 0, 4] - 1).max() < 1e-2


def test_groups_must_divide_the_modes(case):
    blob, tau, k = case
    with pytest.raises(RuntimeError):
        oracle.solve_grouped(blob, k[:7], tau, 4, **DIMS)


def test_groups_over_several_cosmologies_and_outputs():
    """Groups never straddle cosmologies; each group runs on its own
    cosmology's tables and output times (two cosmologies, two outputs)."""
    from discoeb_gb300.workloads import sample_cosmologies

    ps = [bg.evolve_background(param=p) for p in sample_cosmologies(2, seed=3)[0]]
    tabs = tb.pack_batch(ps, 3)
    taus = np.stack([tb.tau_of_a(p, [0.5, 1.0]) for p in ps])
    k = np.tile(np.geomspace(1e-3, 1.0, 4), 2)
    com = np.repeat(np.arange(2, dtype=np.int32), 4)
    yo, so = oracle.solve_grouped(tabs, k, taus, 2, cosmo_of_mode=com, rtol=1e-4, atol=1e-4, **DIMS)
    yh, sh = H.solve_grouped(tabs, k, taus, 2, cosmo_of_mode=com, rtol=1e-4, atol=1e-4, **DIMS)
    assert (so[:, 0] == 0).all() and (sh[:, 0] == 0).all()
    np.testing.assert_allclose(yh[:, 1, 4] ** 2, yo[:, 1, 4] ** 2, rtol=1e-6)
    np.testing.assert_allclose(yh[:, 0, 4] ** 2, yo[:, 0, 4] ** 2, rtol=1e-3)   # a = 0.5: in-step interpolation
    # each group equals that group solved alone
    for g in range(4):
        sl = slice(2 * g, 2 * g + 2)
        c = int(com[2 * g])
        y1, _ = oracle.solve_grouped(tabs[c], k[sl], taus[c], 2, rtol=1e-4, atol=1e-4, **DIMS)
        np.testing.assert_array_equal(y1, yo[sl])


def test_group_failure_statuses(case):
    """A step budget that runs out stops the whole group with MAX_STEPS (1);
    the kernel's group driver and the oracle agree on it."""
    blob, tau, k = case
    yo, so = oracle.solve_grouped(blob, k, tau, 4, rtol=1e-4, atol=1e-4, max_steps=5, **DIMS)
    yh, sh = H.solve_grouped(blob, k, tau, 4, rtol=1e-4, atol=1e-4, max_steps=5, **DIMS)
    assert (so[:, 0] == 1).all() and (sh[:, 0] == 1).all()
    assert (sh[:, 1] + sh[:, 2] == 5).all()
