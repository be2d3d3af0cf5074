"""RECFAST thermal history on the host (FP64): the x_e(a), c_s^2(a) tables.

Restates ``src/discoeb/thermodynamics_recfast.py`` (itself an adaptation of
RECFAST by Seager, Sasselov & Scott 1999/2000 with the Wong, Moss & Scott 2008
fudges).  The physical constants, fitting parameters and the three-equation
ionisation system are the published RECFAST model and have to be identical
for the tables to agree; the code around them is written for plain Python
scalars so that the 3x3 Jacobian can be taken by complex-step differentiation
(exact to rounding, like the reference's ``jacfwd``).

Integration per sampling interval uses the reference's GRK4A Rosenbrock
method (Kaps & Rentrop 1979, ``ode_integrators_stiff.py:78-223``) under a
diffrax-style I-controller with the defaults the reference inherits
(``thermodynamics_recfast.py:283-300``).  Only x_e, T_m and c_s^2 leave this
module; the dx/dz closed forms of the Saha branches feed nothing on the
perturbation path and are not evaluated.
"""
from __future__ import annotations

import cmath
import math

import numpy as np

from .background import get_aprimeoa, dtauda, romberg

# --- physical constants (thermodynamics_recfast.py:38-53) ---------------------
G_N = 6.67430e-11
M_H = 1.67353284e-27
M_E = 9.1093837015e-31
MHE_MH = 3.97146570884
C_LIGHT = 2.99792458e08
H_PLANCK = 6.62607015e-34
K_B = 1.380649e-23
SIGMA_T = 6.6524587321e-29
A_RAD = 4 * 5.670374419e-8 / C_LIGHT
BIG_H = 3.2407792902755102e-18
DENS_FAC = 11.223810928601939
E_ION_HE12S = 6.314878282674e5

# --- atomic data (thermodynamics_recfast.py:57-84) ----------------------------
LAMBDA_H = 8.2245809
LAMBDA_HE = 51.3
L_H_ION = 1.096787737e7
L_H_ALPHA = 8.225916453e6
L_HE1_ION = 1.98310772e7
L_HE2_ION = 4.389088863e7
L_HE_2S = 1.66277434e7
L_HE_2P = 1.71134891e7
A2P_S = 1.798287e9
A2P_T = 177.58
L_HE_2PT = 1.690871466e7
L_HE_2ST = 1.5985597526e7
L_HE2ST_ION = 3.8454693845e6
SIGMA_HE_2PS = 1.436289e-22
SIGMA_HE_2PT = 1.484872e-22
AGAUSS1, AGAUSS2 = -0.14, 0.05
ZGAUSS1, ZGAUSS2 = 7.28, 6.75
WGAUSS1, WGAUSS2 = 0.18, 0.33
H_FRAC = 1.0e-3

LALPHA = 1.0 / L_H_ALPHA
LALPHA_HE = 1.0 / L_HE_2P
CDB = H_PLANCK * C_LIGHT * (L_H_ION - L_H_ALPHA) / K_B
CDB_HE = H_PLANCK * C_LIGHT * (L_HE1_ION - L_HE_2S) / K_B
CB1 = H_PLANCK * C_LIGHT * L_H_ION / K_B
CR = 2.0 * math.pi * (M_E / H_PLANCK) * (K_B / H_PLANCK)
CK = LALPHA**3 / (8.0 * math.pi)
CK_HE = LALPHA_HE**3 / (8.0 * math.pi)
CL = C_LIGHT * H_PLANCK / (K_B * LALPHA)
CL_HE = C_LIGHT * H_PLANCK / (K_B / L_HE_2S)
CT = (8.0 / 3.0) * (SIGMA_T / (M_E * C_LIGHT)) * A_RAD
BFACT = H_PLANCK * C_LIGHT * (L_HE_2P - L_HE_2S) / K_B
CL_PST = H_PLANCK * C_LIGHT * (L_HE_2PT - L_HE_2ST) / K_B
HCL_HE2ST_KB = H_PLANCK * C_LIGHT * L_HE_2ST / K_B
HCL_HE2ST_ION_KB = H_PLANCK * C_LIGHT * L_HE2ST_ION / K_B

A_PPB, B_PPB, C_PPB, D_PPB = 4.309, -0.6166, 0.6703, 0.5300
A_VF = 10.0 ** (-16.744)
B_VF = 0.711
T_0 = 10 ** 0.477121
T_1 = 10 ** 5.114
A_TRIP = 10.0 ** (-16.306)
B_TRIP = 0.761
FU = 1.105

# GRK4A coefficients (Kaps & Rentrop 1979, ``ode_integrators_stiff.py:131-150``).
_G = 0.395
_G21, _G31, _G32 = -0.767672395484, -0.851675323742, 0.522967289188
_G41, _G42, _G43 = 0.288463109545, 0.880214273381e-1, -0.337389840627
_A21, _A31, _A32 = 0.438, 0.796920457938, 0.730795420615e-1
_CH1, _CH2, _CH3 = 0.346325833758, 0.285693175712, 0.367980990530
_C1, _C2, _C3, _C4 = 0.199293275701, 0.482645235674, 0.680614886256e-1, 0.25


def _re(x):
    return x.real if isinstance(x, complex) else x


def ionization_rhs(a, y, P, aH):
    """d(x_H, x_He, T_m)/da (``thermodynamics_recfast.py:124-281``).

    ``y`` may hold complex numbers (complex-step Jacobian); every branch
    condition is taken on the real part.  ``aH`` is the conformal Hubble rate
    at ``a`` (it does not depend on y).
    """
    cx = any(isinstance(v, complex) for v in y)
    ex = cmath.exp if cx else math.exp
    sq = cmath.sqrt if cx else math.sqrt
    z = 1.0 / a - 1.0
    H = P["H0"] / 100.0
    HO = H * BIG_H
    mu_H = 1.0 / (1.0 - P["YHe"])
    fHe = P["YHe"] / (MHE_MH * (1.0 - P["YHe"]))
    Nnow = DENS_FAC * H * H * P["Omegab"] / mu_H
    x_H, x_He, T2 = y
    x = x_H + fHe * x_He
    Tmat = T2 if _re(T2) >= 0 else -T2
    zt = 1.0 + z
    n = Nnow * zt**3
    n_He = fHe * n
    Trad = P["Tcmb"] * zt
    Hz = (1e-5 * aH) / a * C_LIGHT * BIG_H

    Tm4 = Tmat / 1e4
    CRT15 = (CR * Tmat) ** 1.5
    Rdown = 1e-19 * A_PPB * Tm4**B_PPB / (1.0 + C_PPB * Tm4**D_PPB)
    Rup = Rdown * CRT15 * ex(-CDB / Tmat)
    sq0 = sq(Tmat / T_0)
    sq1 = sq(Tmat / T_1)
    Rdown_He = A_VF / (sq0 * (1.0 + sq0) ** (1.0 - B_VF) * (1.0 + sq1) ** (1.0 + B_VF))
    Rup_He = 4.0 * Rdown_He * CRT15 * ex(-CDB_HE / Tmat)
    bt = BFACT / Tmat
    He_Boltz = ex(bt if _re(bt) < 680.0 else 680.0)
    Rdown_trip = A_TRIP / (sq0 * (1.0 + sq0) ** (1.0 - B_TRIP) * (1.0 + sq1) ** (1.0 + B_TRIP))
    Rup_trip = Rdown_trip * ex(-HCL_HE2ST_ION_KB / Tmat) * CRT15 * (4.0 / 3.0)
    lz = math.log(zt)
    K = CK / Hz * (1.0 + AGAUSS1 * math.exp(-(((lz - ZGAUSS1) / WGAUSS1) ** 2))
                   + AGAUSS2 * math.exp(-(((lz - ZGAUSS2) / WGAUSS2) ** 2)))
    omxHe = 1.0 - x_He
    omxH = 1.0 - x_H
    nHe1 = n_He * omxHe
    Hzz = Hz * zt

    xHe_r = _re(x_He)
    xH_r = _re(x_H)
    he_edge = (xHe_r < 5e-9) or (xHe_r > 0.98)

    # Peebles K factor for HeI singlets, three cases (recfast :206-214)
    if he_edge:
        K_He = CK_HE / Hz
    else:
        tauHe_s = A2P_S * CK_HE * 3.0 * nHe1 / Hz
        pHe_s = (1.0 - ex(-tauHe_s)) / tauHe_s
        if xH_r < 0.9999999:
            Dop = sq(2.0 * K_B * Tmat / (M_H * MHE_MH * C_LIGHT**2))
            Dop_2p = C_LIGHT * L_HE_2P * Dop
            g2Ps = (3.0 * A2P_S * fHe * omxHe * C_LIGHT**2) / (
                math.sqrt(math.pi) * SIGMA_HE_2PS * 8.0 * math.pi * Dop_2p * omxH * (C_LIGHT * L_HE_2P) ** 2)
            AHcon = A2P_S / (1.0 + 0.36 * g2Ps**0.86)
            K_He = 1.0 / ((A2P_S * pHe_s + AHcon) * 3.0 * nHe1)
        else:
            K_He = 1.0 / (A2P_S * pHe_s * 3.0 * nHe1)

    timeTh = (1.0 / (CT * Trad**4)) * (1.0 + x + fHe) / x
    timeH = 2.0 / (3.0 * HO * zt**1.5)

    # hydrogen
    if xH_r > 0.99:
        f0 = 0.0 * x_H
    else:
        rate = x * x_H * n * Rdown - Rup * omxH * ex(-CL / Tmat)
        if xH_r > 0.985:
            f0 = rate / Hzz
        else:
            KLn = K * LAMBDA_H * n * omxH
            den = 1.0 / FU + KLn / FU + K * Rup * n * omxH
            f0 = rate * (1.0 + KLn) / (Hzz * den)

    # helium
    if xHe_r < 1e-8:
        f1 = 0.0 * x_He
    else:
        rate_He = x * x_He * n * Rdown_He - Rup_He * omxHe * ex(-CL_HE / Tmat)
        KHL = K_He * LAMBDA_HE * nHe1 * He_Boltz
        Hden = 1.0 + K_He * (LAMBDA_HE + Rup_He) * nHe1 * He_Boltz
        f1 = rate_He * (1.0 + KHL) / (Hzz * Hden)
        if not he_edge:
            tauHe_t = A2P_T * nHe1 * 3.0 / (8.0 * math.pi * Hz * L_HE_2PT**3)
            pHe_t = (1.0 - ex(-tauHe_t)) / tauHe_t
            ePSt = ex(-CL_PST / Tmat)
            if xH_r > 0.99999:
                CfHe_t = A2P_T * pHe_t * ePSt
            else:
                Dop = sq(2.0 * K_B * Tmat / (M_H * MHE_MH * C_LIGHT**2))
                Dop_2Pt = C_LIGHT * L_HE_2PT * Dop
                g2Pt = (3.0 * A2P_T * fHe * omxHe * C_LIGHT**2) / (
                    math.sqrt(math.pi) * SIGMA_HE_2PT * 8.0 * math.pi * Dop_2Pt * omxH * (C_LIGHT * L_HE_2PT) ** 2)
                AHcon_t = A2P_T / (1.0 + 0.66 * g2Pt**0.9) / 3.0
                CfHe_t = (A2P_T * pHe_t + AHcon_t) * ePSt
            CfHe_t = CfHe_t / (Rup_trip + CfHe_t)
            trip = x * x_He * n * Rdown_trip - omxHe * 3.0 * Rup_trip * ex(-HCL_HE2ST_KB / Tmat)
            f1 = f1 + trip * CfHe_t / Hzz

    # matter temperature
    if _re(timeTh) < H_FRAC * timeH:
        f2 = Tmat / zt
    else:
        f2 = CT * Trad**4 * x / (1.0 + x + fHe) * (Tmat - Trad) / Hzz + 2.0 * Tmat / zt

    dzda = -1.0 / a**2
    return [f0 * dzda, f1 * dzda, f2 * dzda]


def _jac3(a, y, P, aH):
    """3x3 Jacobian d f / d y by complex step (exact to rounding)."""
    h = 1e-30
    J = np.zeros((3, 3))
    for j in range(3):
        yc = [complex(v) for v in y]
        yc[j] += 1j * h
        fc = ionization_rhs(a, yc, P, aH)
        for i in range(3):
            J[i, j] = (fc[i].imag if isinstance(fc[i], complex) else 0.0) / h
    return J


def _grk4a_step(t0, dt, y0, P, aH):
    """One GRK4A step with all stages at t0 (``ode_integrators_stiff.py:117-223``)."""
    f = lambda y: np.array(ionization_rhs(t0, list(y), P, aH), dtype=np.float64) * dt
    J = _jac3(t0, list(y0), P, aH) * dt
    A = np.eye(3) - _G * J
    Ainv = np.linalg.inv(A)
    k1 = Ainv @ f(y0)
    Jk1 = J @ k1
    k2 = Ainv @ (f(y0 + _A21 * k1) + _G21 * Jk1)
    Jk2 = J @ k2
    f2 = f(y0 + _A31 * k1 + _A32 * k2)
    k3 = Ainv @ (f2 + _G31 * Jk1 + _G32 * Jk2)
    Jk3 = J @ k3
    k4 = Ainv @ (f2 + _G41 * Jk1 + _G42 * Jk2 + _G43 * Jk3)
    y1 = y0 + _C1 * k1 + _C2 * k2 + _C3 * k3 + _C4 * k4
    err = (_C1 - _CH1) * k1 + (_C2 - _CH2) * k2 + (_C3 - _CH3) * k3 + _C4 * k4
    return y1, err


# Stage abscissae and summed gammas of GRK4A for the non-autonomous form
# (Kaps & Rentrop 1979; Hairer & Wanner, Solving ODEs II, IV.7):
# alpha_i = sum_j alpha_ij, gamma_i = gamma + sum_j gamma_ij.
_ALPHA2, _ALPHA3 = _A21, _A31 + _A32
_GAM1 = _G
_GAM2 = _G + _G21
_GAM3 = _G + _G31 + _G32
_GAM4 = _G + _G41 + _G42 + _G43


def _grk4a_step_timed(t0, dt, y0, P, aH_of):
    """One GRK4A step of the non-autonomous problem: stage i at
    t0 + alpha_i dt, plus the gamma_i dt^2 df/dt terms (df/dt by a central
    difference in a).  Not the reference's step (which keeps every stage at
    t0); used to measure what that choice costs."""
    f = lambda t, y: np.array(ionization_rhs(t, list(y), P, aH_of(t)), dtype=np.float64) * dt
    J = _jac3(t0, list(y0), P, aH_of(t0)) * dt
    ht = 1e-7 * t0
    ft = (f(t0 + ht, y0) - f(t0 - ht, y0)) * (dt / (2.0 * ht))
    Ainv = np.linalg.inv(np.eye(3) - _G * J)
    k1 = Ainv @ (f(t0, y0) + _GAM1 * ft)
    Jk1 = J @ k1
    k2 = Ainv @ (f(t0 + _ALPHA2 * dt, y0 + _A21 * k1) + _G21 * Jk1 + _GAM2 * ft)
    Jk2 = J @ k2
    f2 = f(t0 + _ALPHA3 * dt, y0 + _A31 * k1 + _A32 * k2)
    k3 = Ainv @ (f2 + _G31 * Jk1 + _G32 * Jk2 + _GAM3 * ft)
    Jk3 = J @ k3
    k4 = Ainv @ (f2 + _G41 * Jk1 + _G42 * Jk2 + _G43 * Jk3 + _GAM4 * ft)
    y1 = y0 + _C1 * k1 + _C2 * k2 + _C3 * k3 + _C4 * k4
    err = (_C1 - _CH1) * k1 + (_C2 - _CH2) * k2 + (_C3 - _CH3) * k3 + _C4 * k4
    return y1, err


def solve_ionization(astart, aend, ystart, P, aH_of, rtol=1e-3, atol=1e-6, max_steps=128, stage_times=False):
    """Adaptive GRK4A from astart to aend (``thermodynamics_recfast.py:283-300``).

    I-controller of diffrax defaults (safety 0.9, factor in [0.2, 10],
    error order 3 as GRKT4 declares), RMS norm over the three components.
    Returns (x_H, x_He, T_m, dx_H/da, dx_He/da, dT_m/da) at aend.
    ``stage_times=True`` integrates the non-autonomous problem properly
    (:func:`_grk4a_step_timed`) instead of the reference's step.
    """
    t0 = astart
    t1 = min(astart + abs(astart) * 1e-3, aend)
    y = np.array(ystart[:3], dtype=np.float64)
    steps = 0
    while t0 < aend and steps < max_steps:
        dt = t1 - t0
        if stage_times:
            y1, err = _grk4a_step_timed(t0, dt, y, P, aH_of)
        else:
            y1, err = _grk4a_step(t0, dt, y, P, aH_of(t0))
        y1c = y if np.isnan(y1).any() else y1
        sc = err / (atol + rtol * np.maximum(np.abs(y), np.abs(y1c)))
        e = math.sqrt(float(np.mean(sc * sc)))
        keep = e < 1.0
        inv = math.inf if e == 0.0 else 1.0 / e
        fac = 0.9 * inv ** (1.0 / 3.0)
        fac = min(max(fac, 1.0 if keep else 0.2), 10.0)
        if keep:
            y = y1
            t0 = t1
        t1 = t0 + dt * fac
        if t1 > aend - 1e-10:
            t1 = aend
        steps += 1
    dy = ionization_rhs(aend, list(y), P, aH_of(aend))
    return np.concatenate([y, np.array(dy, dtype=np.float64)])


def saha_heii(a, P):
    """HeII -> HeIII Saha fraction (``thermodynamics_recfast.py:302-321``)."""
    fHe = P["fHe"]
    Hfac = 1.0 / (1.0e06 * 3.0856775807e13)
    mu_H = 1.0 / (1.0 - P["YHe"])
    rho_c = 3.0 * (P["H0"] * Hfac) ** 2 / (8.0 * math.pi * G_N)
    NH = rho_c * P["Omegab"] / (M_H * mu_H) / a**3
    T = P["Tcmb"] / a
    betaE = E_ION_HE12S / T
    A = 1.0 + fHe
    B = 1.0 + 2.0 * fHe
    R = (2.0 * math.pi * M_E * K_B / H_PLANCK**2 * T) ** 1.5 / NH * math.exp(-betaE)
    if R > 1e5:
        return fHe * (1.0 - B / R + (1.0 + 5.0 * fHe + 6.0 * fHe**2) / R**2)
    return quad_root(R - A, R * B) - A


def quad_root(b: float, c: float) -> float:
    """The positive root of x^2 + b x - c = 0 (c >= 0), (sqrt(b^2 + 4c) - b) / 2,
    the form of the Saha fractions; as 2c / (sqrt(b^2 + 4c) + b) when b > 0,
    the same number without the cancellation of the direct form (~b * 1e-16
    absolute, noise that a difference quotient over parameter sets divides
    by 2 eps)."""
    s = math.sqrt(b * b + 4.0 * c)
    return 2.0 * c / (s + b) if b > 0.0 else 0.5 * (s - b)


def adaptive_sampling(a0: float, a1: float, N: int) -> np.ndarray:
    """Scale-factor samples clustered on recombination (``thermodynamics_recfast.py:324-360``)."""
    n1 = max(8, int(N * 0.05))
    n2 = max(8, int(N * 0.10))
    n3 = int(N * 0.50)
    n4 = N - n1 - n2 - n3
    ab1 = max(1.0 / 3001.0, a0)
    ab2 = 1.0 / 1401.0
    ab3 = 1.0 / 601.0
    return np.concatenate([
        np.geomspace(a0, ab1, n1, endpoint=False),
        np.geomspace(ab1, ab2, n2, endpoint=False),
        np.geomspace(ab2, ab3, n3, endpoint=False),
        np.geomspace(ab3, a1, n4),
    ])


def compute_thermal_history(*, a0, a1, N, param, rtol=1e-3, atol=1e-6, stage_times=False):
    """Ionisation history sampled on N adaptive points (``thermodynamics_recfast.py:362-452``)."""
    a = adaptive_sampling(a0, a1, N + 1)
    H = param["H0"] / 100.0
    HO = H * BIG_H
    mu_H = 1.0 / (1.0 - param["YHe"])
    Nnow = 3.0 * HO * HO * param["Omegab"] / (8.0 * math.pi * G_N * mu_H * M_H)
    fHe = param["YHe"] / (MHE_MH * (1.0 - param["YHe"]))
    Tcmb = param["Tcmb"]
    aH_of = lambda aa: float(get_aprimeoa(param=param, aexp=aa))
    out = np.zeros((6, N))
    for i in range(N):
        astart, aend = a[i], a[i + 1]
        zstart = 1.0 / astart - 1.0
        zend = 1.0 / aend - 1.0
        if i > 0:
            y_prev = out[:, i - 1]
        else:
            y_prev = np.array([1.0, 1.0, Tcmb * (1.0 + zstart), 0.0, 0.0, -Tcmb * (1.0 + zstart)])
        if zend > 3500.0:
            new = np.array([1.0, 1.0, Tcmb * (1.0 + zend), 0.0, 0.0, -Tcmb * (1.0 + zend)])
        elif i > 0 and y_prev[1] > 0.99:
            rhs = math.exp(1.5 * math.log(CR * Tcmb / (1.0 + zend)) - H_PLANCK * C_LIGHT * L_HE1_ION / K_B / (Tcmb * (1.0 + zend))) / Nnow * 4.0
            xHe0 = quad_root(rhs - 1.0, (1.0 + fHe) * rhs)
            new = np.array([1.0, (xHe0 - 1.0) / fHe, Tcmb * (1.0 + zend), 0.0, 0.0, -Tcmb * (1.0 + zend)])
        elif i > 0 and y_prev[0] > 0.99:
            rhs = math.exp(1.5 * math.log(CR * Tcmb / (1.0 + zend)) - CB1 / (Tcmb * (1.0 + zend))) / Nnow
            xH0 = quad_root(rhs, rhs)
            new = solve_ionization(astart, aend, y_prev, param, aH_of, rtol, atol, stage_times=stage_times)
            new[0] = xH0
            new[3] = 0.0
        else:
            new = solve_ionization(astart, aend, y_prev, param, aH_of, rtol, atol, stage_times=stage_times)
        out[:, i] = new
    return out, a[1:]


def evaluate_thermo(*, param: dict, num_thermo: int = 256, stage_times: bool = False):
    """x_e, T_m, c_s^2 and tau on the sampled scale factors (``thermodynamics_recfast.py:455-501``)."""
    param["fHe"] = param["YHe"] / (MHE_MH * (1.0 - param["YHe"]))
    y, a = compute_thermal_history(a0=param["amin"], a1=param["amax"], N=num_thermo, param=param,
                                   stage_times=stage_times)
    xeHI = y[0]
    xeHeI = y[1]
    xeHeII = np.array([saha_heii(ai, param) for ai in a])
    xe = xeHI + param["fHe"] * xeHeI + xeHeII
    mu = 1.0 / (1.0 + (1.0 / MHE_MH - 1.0) * param["YHe"] + (1.0 - param["YHe"]) * xe)
    Tm = y[2]
    dTmda = y[5]
    daTmda = Tm + a * dTmda
    cs2 = K_B / M_H / C_LIGHT**2 / mu * Tm * (4.0 - daTmda / Tm) / 3.0
    tau = np.empty_like(a)
    tau[0] = param["taumin"]
    f = lambda x: dtauda(x, param)
    for i in range(1, a.shape[0]):
        tau[i] = tau[i - 1] + romberg(f, a[i - 1], a[i])
    return tau, a, cs2, Tm, mu, xe, xeHI, xeHeI, xeHeII
