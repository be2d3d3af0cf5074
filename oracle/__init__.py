"""CPU oracle for the perturbation hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may import this package; the library never does.  It wraps
``discoeb_oracle.cpp`` (an FP64 restatement of the reference algorithm with a
forward-mode dense Jacobian and partial-pivot dense LU, file:line citations
in that file) through ctypes.

Parity pin: checked against the reference's own golden vectors
(``tests/resources/CLASS_data.json`` P_bc(k) at a=0.01 and
``RECFAST_DISCO_EB_data.json`` x_e(a), both at the reference's 5e-3) by the
tests in ``tests/test_oracle_golden.py``.  At the 1e-4 level the reference
(JAX + diffrax) cannot run here, so finer parity with the live reference is
unpinned.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libdiscoeb_oracle.so")
_lib = None

STATUS_NAMES = {0: "OK", 1: "MAX_STEPS", 2: "DT_UNDERFLOW", 3: "NONFINITE", 4: "BAD_INPUT"}


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "discoeb_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.check_call(["bash", os.path.join(_HERE, "build.sh")])
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        dp = ctypes.POINTER(ctypes.c_double)
        ip = ctypes.POINTER(ctypes.c_int)
        L.oracle_solve.argtypes = [dp, ctypes.c_int, ctypes.c_int, dp, ip, ctypes.c_int, dp, ctypes.c_int, ip, dp,
                                   ctypes.c_int, ctypes.c_int, dp, ip, ctypes.c_int]
        L.oracle_solve_grouped.argtypes = [dp, ctypes.c_int, ctypes.c_int, dp, ip, ctypes.c_int, dp, ctypes.c_int, ip,
                                           dp, ctypes.c_int, ctypes.c_int, dp, ip, ctypes.c_int]
        L.oracle_rhs.argtypes = [dp, ip, ctypes.c_double, ctypes.c_double, dp, dp]
        L.oracle_jacobian.argtypes = [dp, ip, ctypes.c_double, ctypes.c_double, dp, dp, dp]
        L.oracle_initial.argtypes = [dp, ip, ctypes.c_double, ctypes.c_double, dp, dp]
        L.oracle_outputs.argtypes = [dp, ip, ctypes.c_double, dp, dp]
        L.oracle_spline_eval.argtypes = [dp, ctypes.c_int, dp, ctypes.c_int, dp]
        L.oracle_n_vars.argtypes = [ctypes.c_int] * 5
        _lib = L
    return _lib


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


def n_vars(lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax) -> int:
    return 7 + (lmaxg + 1) + (lmaxgp + 1) + (lmaxr + 1) + nqmax * (lmaxnu + 1) + 2


def solve(tables, kmodes, tau_out, *, cosmo_of_mode=None, lmaxg=11, lmaxgp=11, lmaxr=11, lmaxnu=8, nqmax=3,
          rtol=1e-4, atol=1e-4, pcoeff=0.25, icoeff=0.80, dcoeff=0.0, factormax=20.0, factormin=0.3,
          max_steps=2048, return_full=False, error_order=5.0, safety=0.9, hist_on_reject=False, nthreads=0,
          step_to_outputs=False):
    """Run the oracle.  Returns (y [nmode, nout, 20|n], stats [nmode, 3])."""
    tables = np.ascontiguousarray(np.atleast_2d(tables), dtype=np.float64)
    kmodes = np.ascontiguousarray(kmodes, dtype=np.float64)
    tau_out = np.ascontiguousarray(np.atleast_2d(tau_out), dtype=np.float64)
    nmode = kmodes.shape[0]
    ncosmo = tables.shape[0]
    nout = tau_out.shape[1]
    if cosmo_of_mode is None:
        cosmo_of_mode = np.zeros(nmode, dtype=np.int32)
    cosmo_of_mode = np.ascontiguousarray(cosmo_of_mode, dtype=np.int32)
    dims = np.array([lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax], dtype=np.int32)
    cfg = np.array([rtol, atol, pcoeff, icoeff, dcoeff, factormax, factormin, error_order, safety,
                    1.0 if hist_on_reject else 0.0, 1.0 if step_to_outputs else 0.0], dtype=np.float64)
    n = n_vars(lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax)
    osz = n if return_full else 20
    y = np.empty((nmode, nout, osz), dtype=np.float64)
    stats = np.zeros((nmode, 3), dtype=np.int32)
    rc = lib().oracle_solve(_p(tables), ncosmo, tables.shape[1], _p(kmodes), _p(cosmo_of_mode, ctypes.c_int), nmode,
                            _p(tau_out), nout, _p(dims, ctypes.c_int), _p(cfg), int(max_steps),
                            1 if return_full else 0, _p(y), _p(stats, ctypes.c_int), int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle_solve returned {rc}")
    return y, stats


def solve_grouped(tables, kmodes, tau_out, batch_size, *, cosmo_of_mode=None, lmaxg=11, lmaxgp=11, lmaxr=11,
                  lmaxnu=8, nqmax=3, rtol=1e-4, atol=1e-4, pcoeff=0.25, icoeff=0.80, dcoeff=0.0, factormax=20.0,
                  factormin=0.3, max_steps=2048, error_order=5.0, safety=0.9, hist_on_reject=False, nthreads=0):
    """The reference's batched variant (groups of batch_size consecutive modes
    sharing one start time and one step sequence).  Returns (y [nmode, nout,
    20], stats [nmode, 3])."""
    tables = np.ascontiguousarray(np.atleast_2d(tables), dtype=np.float64)
    kmodes = np.ascontiguousarray(kmodes, dtype=np.float64)
    tau_out = np.ascontiguousarray(np.atleast_2d(tau_out), dtype=np.float64)
    nmode, nout = kmodes.shape[0], tau_out.shape[1]
    com = np.ascontiguousarray(np.zeros(nmode) if cosmo_of_mode is None else cosmo_of_mode, dtype=np.int32)
    dims = np.array([lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax], dtype=np.int32)
    cfg = np.array([rtol, atol, pcoeff, icoeff, dcoeff, factormax, factormin, error_order, safety,
                    1.0 if hist_on_reject else 0.0, 0.0], dtype=np.float64)
    y = np.empty((nmode, nout, 20), dtype=np.float64)
    stats = np.zeros((nmode, 3), dtype=np.int32)
    rc = lib().oracle_solve_grouped(_p(tables), tables.shape[0], tables.shape[1], _p(kmodes), _p(com, ctypes.c_int),
                                    nmode, _p(tau_out), nout, _p(dims, ctypes.c_int), _p(cfg), int(max_steps),
                                    int(batch_size), _p(y), _p(stats, ctypes.c_int), int(nthreads))
    if rc != 0:
        raise RuntimeError(f"oracle_solve_grouped returned {rc}")
    return y, stats


def _dims(d):
    return np.array(d, dtype=np.int32)


def rhs(blob, dims, k, tau, y):
    y = np.ascontiguousarray(y, dtype=np.float64)
    f = np.empty_like(y)
    rc = lib().oracle_rhs(_p(np.ascontiguousarray(blob)), _p(_dims(dims), ctypes.c_int), k, tau, _p(y), _p(f))
    assert rc == 0
    return f


def jacobian(blob, dims, k, tau, y):
    y = np.ascontiguousarray(y, dtype=np.float64)
    n = y.shape[0]
    J = np.empty((n, n))
    dT = np.empty(n)
    rc = lib().oracle_jacobian(_p(np.ascontiguousarray(blob)), _p(_dims(dims), ctypes.c_int), k, tau, _p(y), _p(J), _p(dT))
    assert rc == 0
    return J, dT


def initial(blob, dims, k, tau_out_min):
    n = n_vars(*dims)
    y0 = np.empty(n)
    t = np.zeros(1)
    rc = lib().oracle_initial(_p(np.ascontiguousarray(blob)), _p(_dims(dims), ctypes.c_int), k, tau_out_min, _p(t), _p(y0))
    assert rc == 0
    return float(t[0]), y0


def outputs(blob, dims, k, y):
    o = np.empty(20)
    rc = lib().oracle_outputs(_p(np.ascontiguousarray(blob)), _p(_dims(dims), ctypes.c_int), k,
                              _p(np.ascontiguousarray(y, dtype=np.float64)), _p(o))
    assert rc == 0
    return o


def spline_eval(blob, which, x):
    x = np.ascontiguousarray(np.atleast_1d(x), dtype=np.float64)
    o = np.empty_like(x)
    rc = lib().oracle_spline_eval(_p(np.ascontiguousarray(blob)), int(which), _p(x), x.shape[0], _p(o))
    assert rc == 0
    return o
