"""Named workloads: cosmologies, k-grids, hierarchy sizes and tolerances.

Each workload is named by what it is.  Common fixed inputs follow the
reference's tests: Tcmb=2.7255, YHe=0.248, Omegak=0, cs2_DE=1, k_p=0.05.
"""
from __future__ import annotations

import math

import numpy as np

TCMB = 2.7255
YHE = 0.248


def reference_test_param() -> dict:
    """Cosmology of the reference's tests (``tests/test_perturbations.py:11-57``)."""
    tnu = (4.0 / 11.0) ** (1.0 / 3.0)
    return dict(Omegam=0.3099, Omegab=0.0488911, w_DE_0=-0.99, w_DE_a=0.0, cs2_DE=1.0, Omegak=0.0,
                A_s=2.1064e-09, n_s=0.96822, H0=67.742, Tcmb=TCMB, YHe=YHE,
                Neff=3.046 - 1 * (tnu / ((4.0 / 11.0) ** (1.0 / 3.0))) ** 4, Nmnu=1, mnu=0.06, k_p=0.05)


def lcdm_massless_param(w0: float = -0.999) -> dict:
    """Flat LCDM, 3.046 massless neutrinos, no massive species.

    w0 = -1 exactly makes the reference's DE-velocity equation divide by
    1 + w = 0 (``perturbations.py:368``), so the default is -0.999.
    """
    return dict(Omegam=0.3099, Omegab=0.0486, w_DE_0=w0, w_DE_a=0.0, cs2_DE=1.0, Omegak=0.0,
                A_s=2.1e-9, n_s=0.9667, H0=67.74, Tcmb=TCMB, YHe=YHE, Neff=3.046, Nmnu=0, mnu=0.0, k_p=0.05)


def fiducial_mnu_param() -> dict:
    """LCDM + one 0.06 eV neutrino (2.046 + 1) + w0=-0.9, wa=0.1 fluid."""
    p = lcdm_massless_param()
    p.update(w_DE_0=-0.9, w_DE_a=0.1, Neff=2.046, Nmnu=1, mnu=0.06)
    return p


def sample_cosmologies(n: int, seed: int = 1234, min_abs_1pw: float = 1e-3):
    """n parameter vectors, uniform in the ranges below, drawn in this order.

    Omegam [.25,.35], Omegab [.04,.055], h [.6,.75], n_s [.92,1],
    ln(1e10 A_s) [2.9,3.2], m_nu [.06,.3] eV, w0 [-1.2,-.8], wa [-.3,.3].
    Draws whose w(a) = w0 + wa (1 - a) comes within ``min_abs_1pw`` of -1 on
    a in [0, 1] are rejected and redrawn (the DE equations divide by 1 + w;
    w is linear in a, so the end points decide).  Returns (params, rejected).
    """
    rng = np.random.default_rng(seed)
    out, rejected = [], 0
    while len(out) < n:
        Om, Ob, h, ns, lnAs, mnu, w0, wa = (
            rng.uniform(0.25, 0.35), rng.uniform(0.04, 0.055), rng.uniform(0.6, 0.75), rng.uniform(0.92, 1.0),
            rng.uniform(2.9, 3.2), rng.uniform(0.06, 0.3), rng.uniform(-1.2, -0.8), rng.uniform(-0.3, 0.3))
        e0, e1 = 1.0 + w0 + wa, 1.0 + w0
        if e0 * e1 <= 0.0 or min(abs(e0), abs(e1)) < min_abs_1pw:
            rejected += 1
            continue
        out.append(dict(Omegam=Om, Omegab=Ob, w_DE_0=w0, w_DE_a=wa, cs2_DE=1.0, Omegak=0.0,
                        A_s=math.exp(lnAs) * 1e-10, n_s=ns, H0=100.0 * h, Tcmb=TCMB, YHe=YHE,
                        Neff=2.046, Nmnu=1, mnu=mnu, k_p=0.05))
    return out, rejected


# Hierarchy sizes and tolerances per workload.
LCDM_64K = dict(kmin=1e-4, kmax=1.0, num_k=64, aexp_out=[1.0], lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=8, nqmax=3,
                rtol=1e-3, atol=1e-6)
FIDUCIAL_256K = dict(kmin=1e-4, kmax=10.0, num_k=256, aexp_out=[1.0], lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=17,
                     nqmax=15, rtol=1e-5, atol=1e-5)
BATCHED_64C_512K = dict(ncosmo=64, kmin=1e-4, kmax=10.0, num_k=512, aexp_out=[1.0], lmaxg=12, lmaxgp=12, lmaxr=17,
                        lmaxnu=17, nqmax=15, rtol=1e-5, atol=1e-5)
GRADIENT_128K_8A = dict(kmin=1e-3, kmax=1.0, num_k=128, aexp_out=list(np.linspace(0.2, 1.0, 8)), lmaxg=12, lmaxgp=12,
                        lmaxr=17, lmaxnu=17, nqmax=15, rtol=1e-5, atol=1e-5)
