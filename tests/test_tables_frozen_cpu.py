"""Frozen RECFAST step sequences (deb_evolve_background_frozen_host) and the
cancellation-free Saha roots: the theta +- eps table sets of a gradient are
a smooth function of theta, as the reference's jax.jacfwd through its
RECFAST diffeqsolve differentiates the nominal steps
(thermodynamics_recfast.py:283-298).  Host code only; the GPU form of the
same producer is checked against this one in test_gpu_tables.py.
"""
import ctypes
import math

import numpy as np
import pytest

from discoeb_gb300 import _native, recfast, tables as tb, tables_gpu
from discoeb_gb300.gradient import perturbed_params
from discoeb_gb300.workloads import fiducial_mnu_param, sample_cosmologies

N = 256
CAP = tables_gpu.STEP_CAP_PER_SAMPLE * N


def _xe(t):
    return t[:, tb.HDR_LEN + N: tb.HDR_LEN + 2 * N]


def _sets(p, rs):
    pert = perturbed_params(p, rel_step=rs)
    return [p] + [q for (_, _, a, b) in pert for q in (a, b)], np.array([e for (_, e, _, _) in pert])


def _steps(nset):
    return np.zeros((nset, 3 * N + 1 + 2 * CAP))


def test_leaders_equal_the_adaptive_producer_and_twins_equal_their_leader():
    p = fiducial_mnu_param()
    sets, _ = _sets(p, 1e-4)
    sets = sets + [p]                           # a follower with the leader's own parameters
    lead = np.concatenate([tables_gpu.follow_nominal(1, 12), [0]]).astype(np.int32)
    st = _steps(len(sets))
    tf, sf = tables_gpu.evolve_background_tables_host(sets, 15, leader=lead, steps=st)
    ta, sa = tables_gpu.evolve_background_tables_host(sets, 15)
    assert (sf == 0).all() and (sa == 0).all()
    np.testing.assert_array_equal(tf[0], ta[0])
    np.testing.assert_array_equal(tf[-1], tf[0])
    # the record: monotone interval offsets, step ends inside their intervals, the last at the interval's end
    a_th = tables_gpu.grid(N, 15)[2 * tables_gpu.NUM_NU + 2 * tables_gpu.NQ_BG + 30:][:N + 1]
    off = st[0, :N + 1].astype(int)
    assert off[0] == 0 and (np.diff(off) >= 0).all() and 0 < off[-1] <= CAP
    ends = st[0, 3 * N + 1:3 * N + 1 + 2 * off[-1]:2]
    for i in np.nonzero(np.diff(off))[0]:
        e = ends[off[i]:off[i + 1]]
        assert (np.diff(e) > 0).all() and e[0] > a_th[i] and e[-1] == a_th[i + 1]
    # the library's own record buffer gives the same blobs
    tn, _ = tables_gpu.evolve_background_tables_host(sets, 15, leader=lead)
    np.testing.assert_array_equal(tn, tf)


def test_frozen_quotients_are_smooth_where_the_adaptive_ones_jump():
    """A sampled cosmology whose Omega_b and h sets at eps = 1e-4 take other
    adaptive step counts than the nominal set: there the adaptive quotients
    of x_e at eps = 1e-4 and 1e-5 differ by more than the derivative itself,
    the frozen ones by < 1e-6 of it (the w0 / wa rows of x_e are tiny and
    carry rounding noise over eps, hence their looser bars)."""
    p = sample_cosmologies(16, seed=7)[0][10]
    sets, _ = _sets(p, 1e-4)
    st = _steps(len(sets))
    tables_gpu.evolve_background_tables_host(sets, 3, leader=np.full(len(sets), -1, np.int32), steps=st)
    flips = [s for s in range(1, len(sets)) if st[s, N] != st[0, N]]
    assert len(flips) >= 2, flips
    q = {}
    for rs in (1e-4, 1e-5):
        sets, eps = _sets(p, rs)
        for mode in ("frozen", "adaptive"):
            lead = tables_gpu.follow_nominal(1, len(sets) - 1) if mode == "frozen" else None
            t, s = tables_gpu.evolve_background_tables_host(sets, 3, leader=lead)
            assert (s == 0).all()
            x = _xe(t)
            q[rs, mode] = (x[1::2] - x[2::2]) / (2 * eps[:, None])
    rel = {m: np.abs(q[1e-4, m] - q[1e-5, m]).max(axis=1) / np.abs(q[1e-5, m]).max(axis=1)
           for m in ("frozen", "adaptive")}
    assert rel["adaptive"][1] > 0.1 and rel["adaptive"][2] > 0.1, rel["adaptive"]
    np.testing.assert_array_less(rel["frozen"], [1e-6, 1e-6, 1e-6, 1e-6, 1e-4, 1e-3])


def test_fiducial_quotients_agree_across_eps():
    p = fiducial_mnu_param()
    q = []
    for rs in (1e-4, 1e-5, 1e-6):
        sets, eps = _sets(p, rs)
        t, s = tables_gpu.evolve_background_tables_host(sets, 3, leader=tables_gpu.follow_nominal(1, len(sets) - 1))
        assert (s == 0).all()
        x = _xe(t)
        q.append((x[1::2] - x[2::2]) / (2 * eps[:, None]))
    sc = np.abs(q[0]).max(axis=1)
    np.testing.assert_array_less(np.abs(q[0] - q[1]).max(axis=1) / sc, [1e-7, 1e-6, 1e-6, 1e-5, 1e-4, 1e-3])
    np.testing.assert_array_less(np.abs(q[1] - q[2]).max(axis=1) / sc, [1e-7, 1e-5, 1e-5, 1e-4, 1e-3, 1e-2])


def test_small_record_falls_back_to_adaptive_and_says_so():
    p = fiducial_mnu_param()
    sets, _ = _sets(p, 1e-4)
    st = np.zeros((len(sets), 3 * N + 1 + 2 * 40))          # room for 40 steps of ~600
    t, s = tables_gpu.evolve_background_tables_host(sets, 3, leader=tables_gpu.follow_nominal(1, 12), steps=st)
    assert (s & 2).all() and not (s & 1).any()
    ta, _ = tables_gpu.evolve_background_tables_host(sets, 3)
    np.testing.assert_array_equal(t[0], ta[0])
    assert np.isfinite(t).all()


def test_leader_checks():
    p = fiducial_mnu_param()
    with pytest.raises(ValueError):
        tables_gpu.evolve_background_tables_host([p, p, p], 3, leader=[-1, 0, 1])    # follows a follower
    with pytest.raises(ValueError):
        tables_gpu.evolve_background_tables_host([p, p], 3, leader=[-1, 2])          # out of range
    with pytest.raises(ValueError):
        tables_gpu.evolve_background_tables_host([p, p], 3, leader=[-1])             # one per set
    # through the C ABI the library refuses such a leader per set and runs the set adaptive
    L = _native.load()
    pm = np.ascontiguousarray(tables_gpu.param_matrix([p, p, p]))
    consts, grd = tables_gpu.constants(), tables_gpu.grid(N, 3)
    bl = tables_gpu.blob_len(N, 3)
    tabs = np.zeros((3, bl))
    status = np.zeros(3, np.int32)
    lead = np.array([-1, 0, 1], np.int32)
    cfg = tables_gpu.DebBgCfg(N, tables_gpu.NUM_NU, tables_gpu.NQ_BG, 3, 128, tables_gpu.AMIN, 1e-3, 1e-6)
    c = lambda a: ctypes.c_void_p(a.ctypes.data)
    rc = L.deb_evolve_background_frozen_host(ctypes.byref(cfg), c(pm), 3, c(lead), c(consts), c(grd), None, 0,
                                             c(tabs), bl, c(status), 1)
    assert rc == 0 and status.tolist() == [0, 0, 4]
    np.testing.assert_array_equal(tabs[2], tabs[0])
    assert L.deb_evolve_background_frozen_host(ctypes.byref(cfg), c(pm), 3, None, c(consts), c(grd), None, 0,
                                               c(tabs), bl, c(status), 1) != 0


@pytest.mark.parametrize("b,c", [(1e9, 1e9), (3e6, 3e6 * 1.08), (2.5e5, 4.0), (0.5, 2.0), (-3.0, 1.5), (0.0, 2.0)])
def test_saha_root_without_cancellation(b, c):
    """The root of x^2 + b x - c: residual at rounding level in either regime,
    where the direct (sqrt(b^2 + 4c) - b) / 2 loses ~b * 1e-16 absolute."""
    r = recfast.quad_root(b, c)
    assert r > 0
    assert abs((r + b) * r - c) <= 4e-16 * max(c, abs(b * r))
    if b > 1e5:
        direct = 0.5 * (math.sqrt(b * b + 4.0 * c) - b)
        assert abs((direct + b) * direct - c) > abs((r + b) * r - c)
