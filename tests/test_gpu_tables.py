"""GPU table producer against the host producer (same algorithm, FP64).

Both sides run the RECFAST branch of evolve_background from the same grids
and constants; they differ by the rounding of exp / log / pow and of sums,
which the adaptive ionisation integration carries forward.  Bars: header
scalars 1e-12 relative; spline values and second derivatives 1e-8 of each
array's largest magnitude; the FP32 knots bit for bit; P(k) of the solver on
either set of tables 1e-9 relative in the median (1e-5 at most).
"""
import numpy as np
import pytest

import discoeb_gb300 as deb
import discoeb_gb300.background as bg
import discoeb_gb300.tables as tb
from discoeb_gb300 import tables_gpu
from discoeb_gb300.workloads import fiducial_mnu_param, lcdm_massless_param, reference_test_param, sample_cosmologies

pytestmark = pytest.mark.gpu

FID = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=17, nqmax=15)


def _params():
    sampled, _ = sample_cosmologies(3, seed=5)
    return [lcdm_massless_param(), fiducial_mnu_param(), reference_test_param()] + sampled


@pytest.fixture(scope="module")
def both():
    ps = _params()
    host = np.stack([tb.pack_cosmology(bg.evolve_background(param=p), 15) for p in ps])
    dev, tau, st = tables_gpu.evolve_background_tables(ps, 15, aexp_out=[0.5, 1.0])
    return ps, host, dev.cpu().numpy(), tau.cpu().numpy(), st.cpu().numpy()


def test_status_and_layout(both):
    ps, host, dev, _, st = both
    assert (st == 0).all()
    assert dev.shape == host.shape
    np.testing.assert_array_equal(dev[:, 19:29], host[:, 19:29])     # nq, sizes, length, magic, derived offset


def test_header_scalars(both):
    _, host, dev, _, _ = both
    np.testing.assert_allclose(dev[:, :19], host[:, :19], rtol=1e-12, atol=0)


# largest difference allowed, relative to each array's largest magnitude: the
# RECFAST outputs (x_e, c_s^2 a; splines 0, 1, 6) come from an adaptive
# rtol 1e-3 integration in which a rounding-level difference (exp / pow of
# the two math libraries) can move one accept/reject decision near err = 1,
# and that moves the result by a fraction of the tolerance; the background
# tables (neutrino densities, tau(a)) carry rounding only.  Second
# derivatives and polynomial coefficients amplify knot-to-knot differences.
RECFAST_SPLINES = (0, 1, 6)


def _bars(s):
    return (1e-5, 1e-3) if s in RECFAST_SPLINES else (1e-10, 1e-8)


def _scale(h):
    """Each row's largest magnitude; a row that is zero throughout (e.g. the
    massive-neutrino tables of a cosmology without massive neutrinos) is
    measured against the largest magnitude of the whole array, and an array
    that is zero everywhere against 1, so that it must match absolutely."""
    s = np.abs(h).max(axis=1, keepdims=True)
    glob = float(np.abs(h).max())
    return np.where(s > 0, s, glob if glob > 0 else 1.0)


def test_splines_and_derived_sections(both):
    _, host, dev, _, _ = both
    sizes = host[0, 20:27].astype(int)
    worst = {}
    p = 32
    for si, n in enumerate(sizes):
        for part in range(3):   # x, y, S
            h, d = host[:, p:p + n], dev[:, p:p + n]
            worst[(si, "xyS"[part])] = float((np.abs(d - h) / _scale(h)).max())
            p += n
    nq = int(host[0, 19])
    np.testing.assert_array_equal(dev[:, p:p + 2 * nq], host[:, p:p + 2 * nq])
    p += 2 * nq
    for si, n in enumerate(sizes):
        cf_h, cf_d = host[:, p:p + 4 * (n - 1)].reshape(-1, n - 1, 4), dev[:, p:p + 4 * (n - 1)].reshape(-1, n - 1, 4)
        worst[(si, "c")] = float((np.abs(cf_d - cf_h) / _scale(cf_h.reshape(cf_h.shape[0], -1))[:, :, None]).max())
        p += 4 * (n - 1)
        m = (n + 1) // 2
        if si in (0, 1, 2, 3, 5):   # knots on the fixed log a / a grids: identical FP32 roundings
            np.testing.assert_array_equal(dev[:, p:p + m].view(np.float32), host[:, p:p + m].view(np.float32))
        p += m
    assert p == host.shape[1]
    assert all(np.isfinite(v) for v in worst.values()), worst
    bad = {k: v for k, v in worst.items() if v > (_bars(k[0])[0] if k[1] in "xy" else _bars(k[0])[1])}
    print({f"{k[0]}{k[1]}": f"{v:.1e}" for k, v in worst.items()})
    assert not bad, bad


def test_tau_of_a(both):
    ps, host, _, tau, _ = both
    for i, p in enumerate(ps):
        ref = tb.tau_of_a(bg.evolve_background(param=p), [0.5, 1.0])
        np.testing.assert_allclose(tau[i], ref, rtol=1e-10)


def test_power_spectrum_from_gpu_tables_equals_host_tables(both):
    ps, host, dev, tau, _ = both
    k = np.geomspace(1e-4, 10.0, 8)
    nc = len(ps)
    kk, com = np.tile(k, nc), np.repeat(np.arange(nc, dtype=np.int32), k.size)
    tau_h = np.stack([tb.tau_of_a(bg.evolve_background(param=p), [0.5, 1.0]) for p in ps])
    yh = deb.solve(host, kk, tau_h, com, rtol=1e-5, atol=1e-5, **FID)
    yd = deb.solve(dev, kk, tau, com, rtol=1e-5, atol=1e-5, **FID)
    rel = np.abs(yd[:, :, 4] ** 2 / yh[:, :, 4] ** 2 - 1.0)
    # x_e tables that agree to ~1e-6 leave P(k) equal to ~1e-8; a mode whose
    # accept/reject decision sits within that of err = 1 takes another step
    # sequence: at the end time that moves it by its own discretisation error
    # (< 1e-5 at rtol 1e-5), at the interior output a = 0.5 by the difference of
    # the linear in-step interpolants of the two sequences (SaveAt, 1e-3)
    assert np.median(rel) < 1e-7, float(np.median(rel))
    assert rel[:, 1].max() < 1e-5 and rel[:, 0].max() < 1e-3, (float(rel[:, 1].max()), float(rel[:, 0].max()))


def test_gradient_from_gpu_tables_matches_host_tables():
    """d ln P / d theta with every theta +- eps table set produced on the GPU
    equals the one from the library's producer on the host cores to 1e-6 of
    each parameter's largest derivative: both follow the nominal set's RECFAST
    steps and branches (deb_evolve_background_frozen), so the quotients see
    the two producers' rounding, not their step decisions.  The Python
    producer integrates every set adaptively; against it the bar stays 1e-3."""
    small = dict(lmaxg=8, lmaxgp=8, lmaxr=10, lmaxnu=8, nqmax=3)
    p = fiducial_mnu_param()
    kw = dict(aexp_out=[1.0], kmin=1e-3, kmax=1.0, num_k=6, rtol=1e-5, atol=1e-5, max_steps=8000, **small)
    Ph, Dh, _ = deb.evolve_perturbations_grad(params=p, tables="python", processes=4, **kw)
    Pg, Dg, _ = deb.evolve_perturbations_grad(params=p, tables="gpu", **kw)
    Pn, Dn, _ = deb.evolve_perturbations_grad(params=p, tables="native", **kw)
    scale = np.abs(Dn).max(axis=(0, 1))
    np.testing.assert_allclose(Pg, Pn, rtol=1e-9)
    assert (np.abs(Dg - Dn) <= 1e-6 * scale).all(), (np.abs(Dg - Dn).max(axis=(0, 1)) / scale).tolist()
    np.testing.assert_allclose(Pn, Ph, rtol=1e-5)
    assert (np.abs(Dn - Dh) <= 1e-3 * scale + 1e-12).all(), (np.abs(Dn - Dh).max(axis=(0, 1)) / scale).tolist()


def test_gradient_at_a_small_wa():
    """w_a = 1e-3: its eps is 1e-4 of the scale 0.1 (EPS_SCALE), not of w_a
    itself, and with the frozen RECFAST steps the d ln P / d theta of the GPU
    tables equals the host tables' to 1e-6 of each parameter's largest
    derivative, by replay and by adjoint, and the two methods agree to 1e-6."""
    small = dict(lmaxg=8, lmaxgp=8, lmaxr=10, lmaxnu=8, nqmax=3)
    p = fiducial_mnu_param()
    p["w_DE_a"] = 1e-3
    kw = dict(aexp_out=[1.0], kmin=1e-3, kmax=1.0, num_k=6, rtol=1e-6, atol=1e-9, max_steps=20000, **small)
    D = {(t, m): deb.evolve_perturbations_grad(params=p, tables=t, method=m, **kw)[1]
         for t in ("gpu", "native") for m in ("replay", "adjoint")}
    scale = np.abs(D["native", "replay"]).max(axis=(0, 1))
    for a, b in ((("gpu", "replay"), ("native", "replay")), (("gpu", "adjoint"), ("native", "adjoint")),
                 (("native", "adjoint"), ("native", "replay"))):
        err = np.abs(D[a] - D[b]).max(axis=(0, 1)) / scale
        assert (err <= 1e-6).all(), (a, b, err.tolist())
