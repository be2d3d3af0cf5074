"""The reference's batched variant on the GPU (deb_forward_grouped) against the
oracle's grouped solve, at rtol 1e-4: P(k) 1e-5 relative (same method and
controller, FP64 both; the structured solve and the dense LU round
differently, and one rounding-level difference near err = 1 moves every mode
of a group onto another step sequence); batch_size 1 against the per-mode
kernel: the same per-mode arithmetic compiled into another kernel, whose
roundings can steer a mode onto another valid step sequence, so compared at
rtol 1e-8 to 1e-6 in P(k)."""
import numpy as np
import pytest

import oracle
import discoeb_gb300 as deb
import discoeb_gb300.background as bg
import discoeb_gb300.tables as tb
from discoeb_gb300.workloads import fiducial_mnu_param

pytestmark = pytest.mark.gpu

DIMS = dict(lmaxg=8, lmaxgp=8, lmaxr=10, lmaxnu=8, nqmax=3)


@pytest.fixture(scope="module")
def fid():
    return bg.evolve_background(param=fiducial_mnu_param())


def test_grouped_batches_vs_oracle(fid):
    y, k = deb.evolve_perturbations_batched(param=dict(fid), aexp_out=[1.0], kmin=1e-3, kmax=1.0, num_k=16,
                                            rtol=1e-4, atol=1e-4, batch_size=4, **DIMS)
    yo, so = oracle.solve_grouped(tb.pack_cosmology(fid, 3), k, tb.tau_of_a(fid, [1.0]), 4, rtol=1e-4, atol=1e-4,
                                  **DIMS)
    assert (so[:, 0] == 0).all()
    np.testing.assert_allclose(y[:, 0, 4] ** 2, yo[:, 0, 4] ** 2, rtol=1e-5)
    np.testing.assert_allclose(y[:, 0, 10], yo[:, 0, 10], rtol=1e-5)


def test_batch_of_one_equals_the_per_mode_kernel(fid):
    """At rtol 1e-8 two valid step sequences of a mode agree to ~1e-7 in P(k):
    the group kernel with batch_size 1 gives the per-mode answer."""
    blob = tb.pack_cosmology(fid, 3)
    tau = tb.tau_of_a(fid, [1.0])
    k = np.geomspace(1e-3, 1.0, 8)
    kw = dict(rtol=1e-8, atol=1e-8, max_steps=20000, return_stats=True, **DIMS)
    yg, sg = deb.perturbations.solve_grouped(blob[None], k, tau[None], 1, **kw)
    yp, sp = deb.solve(blob[None], k, tau[None], **kw)
    assert (sg["status"] == 0).all() and (sp["status"] == 0).all()
    np.testing.assert_allclose(yg[:, 0, 4] ** 2, yp[:, 0, 4] ** 2, rtol=1e-6)


def test_group_status_and_bad_groups(fid):
    blob = tb.pack_cosmology(fid, 3)
    tau = tb.tau_of_a(fid, [1.0])
    k = np.geomspace(1e-3, 1.0, 8)
    k[5] = -1.0     # invalid wavenumber: its whole group is refused, the other group runs
    y, st = deb.perturbations.solve_grouped(blob[None], k, tau[None], 4, rtol=1e-4, atol=1e-4, throw=False,
                                            return_stats=True, **DIMS)
    assert (st["status"][:4] == 0).all() and (st["status"][4:] == 4).all()
    assert np.isnan(y[4:]).all() and np.isfinite(y[:4]).all()
    assert len(set(map(tuple, st["steps"][:4]))) == 1
