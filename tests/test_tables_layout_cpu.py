"""Host side of the GPU table producer: constants order, grids and blob length (no GPU)."""
import os
import re

import numpy as np

from discoeb_gb300 import recfast, tables, tables_gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _enum(name):
    txt = open(os.path.join(ROOT, "include", "discoeb_gb300.h")).read()
    body = re.search(r"enum %s \{(.*?)\};" % name, txt, re.S).group(1)
    return [x.split("=")[0].strip() for x in body.replace("\n", " ").split(",") if x.strip()]


def test_constants_follow_the_header_order():
    names = _enum("deb_tables_const")
    assert names[-1] == "DEB_TC_COUNT"
    py = list(tables_gpu.CONST_NAMES) + ["PI", "SQRT_PI", "C2OK"]
    assert len(py) == len(names) - 1 == tables_gpu.constants().shape[0]
    norm = lambda s: s.replace("DEB_TC_", "").replace("_", "").upper()
    alias = {"GN": "GN", "MH": "MH", "ME": "ME", "CLIGHT": "C", "KB": "KB", "T0": "T0", "T1": "T1"}
    for a, b in zip(py, names[:-1]):
        assert alias.get(norm(a), norm(a)) == norm(b), (a, b)
    assert tables_gpu.constants()[names.index("DEB_TC_CR")] == recfast.CR


def test_params_follow_the_header_order():
    names = _enum("deb_bg_param")
    assert names[-1] == "DEB_BG_NPARAM" and len(names) - 1 == len(tables_gpu.PARAM_KEYS)
    m = tables_gpu.param_matrix([dict(Omegam=0.3, Omegab=0.05, H0=70.0, Tcmb=2.7255, YHe=0.248, Neff=3.046, Nmnu=0,
                                      mnu=0.0, w_DE_0=-0.9, w_DE_a=0.0, A_s=2e-9, n_s=0.96)])
    assert m.shape == (1, len(tables_gpu.PARAM_KEYS))
    assert m[0, tables_gpu.PARAM_KEYS.index("cs2_DE")] == 1.0 and m[0, tables_gpu.PARAM_KEYS.index("k_p")] == 0.05


def test_grid_and_blob_length_match_the_host_producer():
    g = tables_gpu.grid(256, 15)
    assert g.shape[0] == 2 * tables_gpu.NUM_NU + 2 * tables_gpu.NQ_BG + 2 * 15 + 257 + 256
    a_th = g[2 * 512 + 16 + 30:2 * 512 + 16 + 30 + 257]
    np.testing.assert_array_equal(a_th, recfast.adaptive_sampling(1e-9, 1.01, 257))
    assert tables_gpu.blob_len(256, 15) == tables.blob_length([256, 256, 512, 512, 256, 256, 256], 15)


def test_producer_code_on_the_host_equals_the_python_producer():
    """The GPU producer's per-set code (deb_tables_core.cuh) built for the host
    against the Python producer (background.py + recfast.py): same algorithm,
    same math library, so agreement to rounding (1e-10 of each array's
    largest value; second derivatives 1e-9)."""
    import sys

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from native import harness as H
    from discoeb_gb300 import background as bg
    from discoeb_gb300.workloads import fiducial_mnu_param, lcdm_massless_param, sample_cosmologies

    ps = [lcdm_massless_param(), fiducial_mnu_param()] + sample_cosmologies(1, seed=5)[0]
    dev, st = H.tables(ps, 15)
    host = np.stack([tables.pack_cosmology(bg.evolve_background(param=p), 15) for p in ps])
    assert (st == 0).all() and dev.shape == host.shape
    np.testing.assert_array_equal(dev[:, 19:32], host[:, 19:32])
    np.testing.assert_allclose(dev[:, :19], host[:, :19], rtol=1e-13, atol=1e-300)
    sizes = host[0, 20:27].astype(int)
    p = 32
    for n in sizes:
        for part in range(3):
            h, d = host[:, p:p + n], dev[:, p:p + n]
            scale = np.abs(h).max(axis=1, keepdims=True)
            assert (np.abs(d - h) <= (1e-9 if part == 2 else 1e-10) * scale).all(), (n, part)
            p += n
    p += 2 * int(host[0, 19])
    np.testing.assert_array_equal(dev[:, 32 + 3 * sizes.sum():p], host[:, 32 + 3 * sizes.sum():p])


def test_library_host_producer_equals_the_python_producer():
    """deb_evolve_background_host (the producer's code compiled into the CUDA
    library's host side, worker threads over the sets) against the Python
    producer, and tau(a) read back from the blobs."""
    from discoeb_gb300 import background as bg
    from discoeb_gb300.workloads import fiducial_mnu_param, sample_cosmologies

    ps = [fiducial_mnu_param()] + sample_cosmologies(3, seed=9)[0]
    got, st = tables_gpu.evolve_background_tables_host(ps, 15, nthreads=3)
    assert (st == 0).all()
    evolved = [bg.evolve_background(param=p) for p in ps]
    ref = np.stack([tables.pack_cosmology(e, 15) for e in evolved])
    np.testing.assert_array_equal(got[:, 19:32], ref[:, 19:32])
    np.testing.assert_allclose(got[:, :19], ref[:, :19], rtol=1e-13, atol=1e-300)
    sizes = ref[0, 20:27].astype(int)
    p = 32
    for n in sizes:   # rounding only: values 1e-10 of each array's largest, second derivatives 1e-9
        for part in range(3):
            h, d = ref[:, p:p + n], got[:, p:p + n]
            assert (np.abs(d - h) <= (1e-9 if part == 2 else 1e-10) * np.abs(h).max(axis=1, keepdims=True)).all()
            p += n
    tau = tables.tau_of_a_blob(got, [0.25, 1.0])
    np.testing.assert_allclose(tau, np.stack([tables.tau_of_a(e, [0.25, 1.0]) for e in evolved]), rtol=1e-12)


import pytest  # noqa: E402


@pytest.mark.parametrize("nqmax", [3, 4, 5, 8, 15])
def test_library_host_producer_momentum_bins(nqmax):
    """The blob's momentum nodes for CAMB's 3/4/5-bin tables and for
    generalised Gauss-Laguerre, as the Python producer packs them."""
    from discoeb_gb300 import background as bg
    from discoeb_gb300.workloads import fiducial_mnu_param

    p = fiducial_mnu_param()
    got, st = tables_gpu.evolve_background_tables_host([p], nqmax, nthreads=1)
    ref = tables.pack_cosmology(bg.evolve_background(param=p), nqmax)
    assert st[0] == 0 and got.shape == (1, ref.shape[0])
    sizes = ref[20:27].astype(int)
    p0 = 32 + 3 * int(sizes.sum())
    np.testing.assert_array_equal(got[0, p0:p0 + 2 * nqmax], ref[p0:p0 + 2 * nqmax])
    np.testing.assert_array_equal(got[0, 19:32], ref[19:32])


def test_native_evolve_background_gives_the_path_the_same_inputs():
    """evolve_background(producer="native") returns a param dict that packs
    to the same blob (to rounding) and has the same output times as the
    Python producer's."""
    from discoeb_gb300 import background as bg
    from discoeb_gb300.workloads import reference_test_param

    p = reference_test_param()
    fast = bg.evolve_background(param=p, producer="native")
    slow = bg.evolve_background(param=p)
    bf, bs = tables.pack_cosmology(fast, 5), tables.pack_cosmology(slow, 5)
    np.testing.assert_array_equal(bf[19:32], bs[19:32])
    scale = np.abs(bs).max()
    assert np.abs(bf - bs).max() <= 1e-9 * scale
    np.testing.assert_allclose(tables.tau_of_a(fast, [0.1, 1.0]), tables.tau_of_a(slow, [0.1, 1.0]), rtol=1e-12)
    for key in ("OmegaDE", "taumin", "amnu", "adotrad", "grhom"):
        np.testing.assert_allclose(fast[key], slow[key], rtol=1e-13)
    np.testing.assert_allclose(fast["xe"], slow["xe"], rtol=1e-9)
    np.testing.assert_allclose(fast["cs2"], slow["cs2"], rtol=1e-8)
