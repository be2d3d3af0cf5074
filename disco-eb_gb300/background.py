"""Host-side background cosmology: the input producer of the perturbation path.

Everything here runs once per cosmology on the host in FP64 and fills the
``param`` dict that :func:`perturbations.evolve_perturbations` consumes, with
the same keys the reference's ``evolve_background`` writes
(``src/discoeb/background.py:140-342``).  Only the keys the perturbation path
reads are produced (scalars, the ``*_of_loga`` and ``*_of_tau`` splines); the
optical-depth / visibility block (``background.py:307-335``) is not on the
path and is left out.
"""
from __future__ import annotations

import math

import numpy as np

from .spline import SplineInterpolation

# Fermi-Dirac normalisation 7 pi^4 / 120, ``background.py:23``.
FERMI_DIRAC_CONST = 5.682196976983475
# m_nu c^2 / (k_B T) conversion in K / eV, ``background.py:141``.
C2OK = 1.62581581e4

# CAMB's high-accuracy momentum nodes for 3, 4, 5 bins (``background.py:27-38``):
# these are published quadrature tables that have to be identical for parity.
_CAMB_NODES = {
    3: ([0.913201, 3.37517, 7.79184], [0.0687359, 3.31435, 2.29911]),
    4: ([0.7, 2.62814, 5.90428, 12.0], [0.0200251, 1.84539, 3.52736, 0.289427]),
    5: ([0.583165, 2.0, 4.0, 7.26582, 13.0], [0.0081201, 0.689407, 2.8063, 2.05156, 0.12681]),
}


def generalized_gauss_laguerre(n: int, alpha: float):
    """Nodes and weights of n-point generalised Gauss-Laguerre quadrature.

    Golub-Welsch: eigen-decomposition of the symmetric Jacobi matrix with
    diagonal 2i-1+alpha and off-diagonal sqrt(i(i+alpha)); weights are the
    squared first eigenvector components times Gamma(alpha+1)
    (``src/discoeb/util.py:82-123``).
    """
    i = np.arange(1, n + 1, dtype=np.float64)
    diag = 2.0 * i - 1.0 + alpha
    io = np.arange(1, n, dtype=np.float64)
    off = np.sqrt(io * (io + alpha))
    J = np.diag(diag) + np.diag(off, 1) + np.diag(off, -1)
    nodes, V = np.linalg.eigh(J)
    weights = V[0, :] ** 2 * math.gamma(alpha + 1.0)
    return nodes, weights


def get_neutrino_momentum_bins(nqmax: int):
    """Momentum nodes q and kernel weights w for massive neutrinos.

    ``background.py:13-44``: CAMB nodes for nqmax in {3,4,5}, otherwise
    generalised Gauss-Laguerre with alpha=1, all divided by 7 pi^4/120.
    """
    if nqmax in _CAMB_NODES:
        q = np.array(_CAMB_NODES[nqmax][0], dtype=np.float64)
        wc = np.array(_CAMB_NODES[nqmax][1], dtype=np.float64)
        dlfdlq = -q / (1.0 + np.exp(-q))
        w = wc / (-0.25 * dlfdlq)
    else:
        alpha = 1
        q, w = generalized_gauss_laguerre(nqmax, alpha)
        w = w * q**3 / (1.0 + np.exp(-q)) * q ** (-alpha)
    return q, w / FERMI_DIRAC_CONST


def nu_background(a, amnu: float, nq: int = 8):
    """rho_nu/rho_nu0 and p_nu/p_nu0 of one massive flavour (``background.py:47-68``)."""
    a = np.atleast_1d(np.asarray(a, dtype=np.float64))
    q, w = get_neutrino_momentum_bins(nq)
    v = 1.0 / np.sqrt(1.0 + (a[:, None] * amnu / q[None, :]) ** 2)
    rhonu = (w[None, :] / v).sum(axis=1)
    pnu = (w[None, :] * v / 3.0).sum(axis=1)
    ppnu = (w[None, :] * v**3 / 3.0).sum(axis=1)
    return rhonu, pnu, ppnu


def romberg(f, a: float, b: float, divmax: int = 6) -> float:
    """Romberg integration of a vectorised f over [a, b].

    Textbook Romberg (trapezoid sums on 2^i panels, Richardson table of depth
    ``divmax``), the algorithm of ``jax_cosmo.scipy.integrate.romb`` with its
    default ``divmax=6`` that the reference calls at ``background.py:182`` and
    ``thermodynamics_recfast.py:484``.
    """
    rng = b - a
    R = [rng * 0.5 * (float(f(np.array([a]))[0]) + float(f(np.array([b]))[0]))]
    for i in range(1, divmax + 1):
        npan = 2 ** (i - 1)
        h = rng / npan
        mids = a + h * (np.arange(npan) + 0.5)
        t = 0.5 * R[0] + 0.5 * h * float(np.sum(f(mids)))
        newR = [t]
        for j in range(1, i + 1):
            fac = 4.0**j
            newR.append((fac * newR[j - 1] - R[j - 1]) / (fac - 1.0))
        R = newR
    return R[divmax]


def rho_de(a, w0: float, wa: float):
    """w0/wa dark-energy density in units of today's (``background.py:75``)."""
    return a ** (-3.0 * (1.0 + w0 + wa)) * np.exp(3.0 * (a - 1.0) * wa)


def dtauda(a, param):
    """d tau / d a from the Friedmann equation (``background.py:71-80``)."""
    a = np.asarray(a, dtype=np.float64)
    rhonu = np.exp(param["logrhonu_of_loga_spline"].evaluate(np.log(a)))
    grho2 = (
        param["grhom"] * param["Omegam"] * a
        + (param["grhog"] + param["grhor"] * (param["Neff"] + param["Nmnu"] * rhonu))
        + param["grhom"] * param["OmegaDE"] * rho_de(a, param["w_DE_0"], param["w_DE_a"]) * a**4
        + param["grhom"] * param["Omegak"] * a**2
    )
    return np.sqrt(3.0 / grho2)


def dadtau(a, param):
    """d a / d tau (``background.py:83-92``)."""
    return 1.0 / dtauda(a, param)


def get_aprimeoa(*, param, aexp):
    """Conformal Hubble rate a'/a (``background.py:100-122``)."""
    a = np.asarray(aexp, dtype=np.float64)
    rhonu = np.exp(param["logrhonu_of_loga_spline"].evaluate(np.log(a)))
    grho = (
        param["grhom"] * param["Omegam"] / a
        + (param["grhog"] + param["grhor"] * (param["Neff"] + param["Nmnu"] * rhonu)) / a**2
        + param["grhom"] * param["OmegaDE"] * rho_de(a, param["w_DE_0"], param["w_DE_a"]) * a**2
        + param["grhom"] * param["Omegak"]
    )
    return np.sqrt(grho / 3.0)


def setup_background_evolution(*, amin: float, amax: float, param: dict) -> dict:
    """Densities, neutrino tables, closure and tau range (``background.py:140-188``)."""
    num_neutrino = 512
    param["amin"] = amin
    param["amax"] = amax
    param["grhom"] = 3.33795017e-11 * param["H0"] ** 2
    param["grhog"] = 1.49594245e-13 * param["Tcmb"] ** 4
    param["grhor"] = 3.39739477e-14 * param["Tcmb"] ** 4
    param["adotrad"] = math.sqrt((param["grhog"] + param["grhor"] * (param["Neff"] + param["Nmnu"])) / 3.0)
    param["amnu"] = param["mnu"] * C2OK / param["Tcmb"]

    a = np.geomspace(amin * 0.9, amax * 1.1, num_neutrino)
    loga = np.log(a)
    param["a"] = a
    rhonu, pnu, ppnu = nu_background(a, param["amnu"])
    param["logrhonu_of_loga_spline"] = SplineInterpolation(loga, np.log(rhonu))
    param["logpnu_of_loga_spline"] = SplineInterpolation(loga, np.log(pnu))
    param["logppseudonu_of_loga_spline"] = SplineInterpolation(loga, np.log(ppnu))

    rhonu0 = float(np.exp(param["logrhonu_of_loga_spline"].evaluate(0.0)))
    param["Omegamnu"] = param["grhor"] * rhonu0 / param["grhom"]
    Omegar = (param["Neff"] + param["Nmnu"] * rhonu0) * param["grhor"] / param["grhom"]
    Omegag = param["grhog"] / param["grhom"]
    param["OmegaDE"] = 1.0 - param["Omegak"] - Omegar - Omegag - param["Omegam"]

    param["taumin"] = amin / param["adotrad"]
    param["taumax"] = param["taumin"] + romberg(lambda x: dtauda(x, param), amin, amax)
    return param


def evolve_background(*, param: dict, thermo_module: str = "RECFAST", num_thermo: int = 256,
                      producer: str = "python", recfast_stage_times: bool = False, **_unused) -> dict:
    """Background + RECFAST thermal history, filling the splines the path reads.

    Mirrors ``evolve_background`` (``background.py:191-305``) for
    ``thermo_module='RECFAST'``.  Produces ``tau_of_a``, ``a_of_tau``,
    ``xe_of_tau``, ``xe_of_loga`` and ``cs2a_of_loga`` splines plus the
    scalars written by :func:`setup_background_evolution`.
    ``producer="native"`` builds the same tables with the library's compiled
    producer (~100x faster; the dict then carries what the perturbation path
    reads, see ``tables_gpu.param_from_blob``).
    ``recfast_stage_times=True`` (Python producer only) integrates the
    ionisation history with GRK4A's stages at their own times instead of the
    reference's all-stages-at-t0 step (``ode_integrators_stiff.py:192-200``):
    the accurate solution of the same equations, not the reference's tables.
    """
    from .recfast import evaluate_thermo

    if thermo_module != "RECFAST":
        raise NotImplementedError("only thermo_module='RECFAST' is produced on the host")
    if producer == "native":
        from .tables_gpu import evolve_backgrounds_native

        return evolve_backgrounds_native([param], num_thermo=num_thermo)[0]
    if producer != "python":
        raise ValueError(f"producer must be 'python' or 'native', not {producer!r}")
    if recfast_stage_times and producer != "python":
        raise ValueError("recfast_stage_times needs producer='python'")
    param = dict(param)
    param.setdefault("Omegak", 0.0)
    amin, amax = 1e-9, 1.01
    param = setup_background_evolution(amin=amin, amax=amax, param=param)
    tau, aexp, cs2, Tm, mu, xe, xeHI, xeHeI, xeHeII = evaluate_thermo(param=param, num_thermo=num_thermo,
                                                                     stage_times=recfast_stage_times)
    param["aexp"] = aexp
    param["tau"] = tau
    param["xe"] = xe
    param["xeHI"] = xeHI
    param["xeHeI"] = xeHeI
    param["xeHeII"] = xeHeII
    param["cs2"] = cs2
    param["Tm"] = Tm
    param["tau_of_a_spline"] = SplineInterpolation(aexp, tau)
    param["a_of_tau_spline"] = SplineInterpolation(tau, aexp)
    param["xe_of_tau_spline"] = SplineInterpolation(tau, xe)
    param["cs2a_of_tau_spline"] = SplineInterpolation(tau, aexp * cs2)
    param["xe_of_loga_spline"] = SplineInterpolation(np.log(aexp), xe)
    param["cs2a_of_loga_spline"] = SplineInterpolation(np.log(aexp), aexp * cs2)
    return param
