"""ctypes wrapper of the test-only host build of the kernel core (core_harness.cpp)."""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SRC = os.path.join(_HERE, "core_harness.cpp")
_TSRC = os.path.join(_HERE, "tables_harness.cpp")
_ASRC = os.path.join(_HERE, "adjoint_harness.cpp")
_ACORE = os.path.join(_HERE, "..", "..", "disco-eb_gb300", "csrc", "deb_adjoint.cuh")
_TCORE = os.path.join(_HERE, "..", "..", "disco-eb_gb300", "csrc", "deb_tables_core.cuh")
_INC = os.path.join(_HERE, "..", "..", "include")
_CORE = os.path.join(_HERE, "..", "..", "disco-eb_gb300", "csrc", "deb_core.cuh")
_LIB = os.path.join(_HERE, "_build", "libcore_harness.so")
_lib = None
dp = ctypes.POINTER(ctypes.c_double)
ip = ctypes.POINTER(ctypes.c_int)


def lib():
    global _lib
    if _lib is None:
        os.makedirs(os.path.dirname(_LIB), exist_ok=True)
        deps = (_SRC, _CORE, _TSRC, _TCORE, _ASRC, _ACORE)
        if not os.path.exists(_LIB) or os.path.getmtime(_LIB) < max(os.path.getmtime(d) for d in deps):
            subprocess.check_call(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-I", _INC, "-o", _LIB, _SRC, _TSRC,
                                   _ASRC])
        L = ctypes.CDLL(_LIB)
        L.h_rhs.argtypes = [dp, ctypes.c_int, ip, ctypes.c_double, ctypes.c_double, dp, dp, dp]
        L.h_solve_W.argtypes = [dp, ctypes.c_int, ip, ctypes.c_double, ctypes.c_double, dp, ctypes.c_double, dp, dp, ctypes.c_int]
        L.h_spline.argtypes = [dp, ctypes.c_int, ctypes.c_int, dp, ctypes.c_int, dp, ip]
        L.h_solve_rr.argtypes = [dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, dp, ip, ctypes.c_int, dp, ctypes.c_int, ip,
                                 dp, ctypes.c_int, dp, ctypes.c_int, ip, ctypes.c_int, ctypes.c_int, dp, ip]
        L.h_start.argtypes = [dp, ctypes.c_int, ip, ctypes.c_double, dp, dp]
        L.h_solve.argtypes = [dp, ctypes.c_int, ctypes.c_int, dp, ip, ctypes.c_int, dp, ctypes.c_int, ip, dp, ctypes.c_int,
                              ctypes.c_int, ctypes.c_int, dp, ip]
        ci, cd = ctypes.c_int, ctypes.c_double
        L.h_solve_grouped.argtypes = [dp, ci, ci, dp, ip, ci, dp, ci, ip, dp, ci, ci, dp, ip]
        L.h_tables.argtypes = [dp, ci, dp, dp, ci, ci, ci, ci, ci, cd, cd, cd, dp, ci, ip]
        L.h_adj_phi.argtypes = [dp, ci, ip, cd, cd, dp, dp, dp]
        L.h_adj_jt.argtypes = [dp, ci, ip, cd, cd, dp, dp, dp, ci]
        L.h_adj_solve_wt.argtypes = [dp, ci, ip, cd, cd, dp, cd, dp, dp]
        L.h_adj_outputs.argtypes = [dp, ci, ip, cd, cd, dp, dp, dp]
        L.h_adjoint.argtypes = [dp, ci, ci, cd, dp, ci, ip, dp, ci, ci, dp, dp, dp, dp, ip, dp]
        L.h_adj_solve_m.argtypes = [dp, ci, ip, cd, cd, dp, cd, dp, dp, ci]
        L.h_adj_outputs_pair.argtypes = [dp, ci, ip, cd, dp, dp, dp]
        L.h_step_adj.argtypes = [dp, ci, ci, ip, cd, cd, cd, dp, dp, dp, dp, dp, dp, dp]
        _lib = L
    return _lib


def tables(params, nqmax, num_thermo=256, rtol=1e-3, atol=1e-6, max_steps=128):
    """Table blobs of the GPU producer's code run on the host (one lane)."""
    from discoeb_gb300 import tables_gpu as tg

    pm = np.ascontiguousarray(tg.param_matrix(params))
    consts, grid = tg.constants(), tg.grid(num_thermo, nqmax)
    L = tg.blob_len(num_thermo, nqmax)
    out = np.zeros((pm.shape[0], L))
    st = np.zeros(pm.shape[0], dtype=np.int32)
    rc = lib().h_tables(_p(pm), pm.shape[0], _p(consts), _p(grid), num_thermo, tg.NUM_NU, tg.NQ_BG, nqmax, max_steps,
                        tg.AMIN, rtol, atol, _p(out), L, _p(st, ctypes.c_int))
    assert rc == 0, rc
    return out, st


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _d(dims):
    return np.array(dims, dtype=np.int32)


def rhs(blob, dims, k, tau, y):
    y = np.ascontiguousarray(y, dtype=np.float64)
    f, jc0 = np.empty_like(y), np.empty_like(y)
    rc = lib().h_rhs(_p(blob), blob.shape[0], _p(_d(dims), ctypes.c_int), k, tau, _p(y), _p(f), _p(jc0))
    assert rc == 0, rc
    return f, jc0


def solve_W(blob, dims, k, tau, y, dt, b, dense=False):
    y = np.ascontiguousarray(y, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty_like(b)
    rc = lib().h_solve_W(_p(blob), blob.shape[0], _p(_d(dims), ctypes.c_int), k, tau, _p(y), dt, _p(b), _p(x), int(dense))
    assert rc == 0, rc
    return x


def solve(tables, kmodes, tau_out, *, cosmo_of_mode=None, lmaxg=11, lmaxgp=11, lmaxr=11, lmaxnu=8, nqmax=3, rtol=1e-4,
          atol=1e-4, pcoeff=0.25, icoeff=0.80, dcoeff=0.0, factormax=20.0, factormin=0.3, max_steps=2048,
          return_full=False, error_order=5.0, safety=0.9, hist_on_reject=False, dense=False, step_to_outputs=False):
    tables = np.ascontiguousarray(np.atleast_2d(tables), dtype=np.float64)
    kmodes = np.ascontiguousarray(kmodes, dtype=np.float64)
    tau_out = np.ascontiguousarray(np.atleast_2d(tau_out), dtype=np.float64)
    nmode, nout = kmodes.shape[0], tau_out.shape[1]
    com = np.ascontiguousarray(np.zeros(nmode) if cosmo_of_mode is None else cosmo_of_mode, dtype=np.int32)
    dims = _d([lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax])
    cfg = np.array([rtol, atol, pcoeff, icoeff, dcoeff, factormax, factormin, error_order, safety,
                    1.0 if hist_on_reject else 0.0, 1.0 if step_to_outputs else 0.0])
    n = 7 + (lmaxg + 1) + (lmaxgp + 1) + (lmaxr + 1) + nqmax * (lmaxnu + 1) + 2
    y = np.empty((nmode, nout, n if return_full else 20))
    st = np.zeros((nmode, 3), dtype=np.int32)
    rc = lib().h_solve(_p(tables), tables.shape[0], tables.shape[1], _p(kmodes), _p(com, ctypes.c_int), nmode, _p(tau_out),
                       nout, _p(dims, ctypes.c_int), _p(cfg), int(max_steps), int(return_full), int(dense), _p(y),
                       _p(st, ctypes.c_int))
    assert rc == 0, rc
    return y, st


def spline(blob, which, x):
    x = np.ascontiguousarray(np.atleast_1d(x), dtype=np.float64)
    out = np.empty_like(x)
    idx = np.empty(x.shape, dtype=np.int32)
    rc = lib().h_spline(_p(blob), blob.shape[0], int(which), _p(x), x.shape[0], _p(out), _p(idx, ctypes.c_int))
    assert rc == 0, rc
    return out, idx


def solve_rr(tables, nset, kmodes, tau_out, *, rec=None, nrec=None, record=False, replay=False, cosmo_of_mode=None,
             lmaxg=11, lmaxgp=11, lmaxr=11, lmaxnu=8, nqmax=3, rtol=1e-4, atol=1e-4, max_steps=2048,
             step_to_outputs=False):
    """Record (nset = 1) or replay (nset table sets per cosmology) like the kernel."""
    tables = np.ascontiguousarray(np.atleast_2d(tables), dtype=np.float64)
    kmodes = np.ascontiguousarray(kmodes, dtype=np.float64)
    tau_out = np.ascontiguousarray(np.atleast_2d(tau_out), dtype=np.float64)
    nmode, nout = kmodes.shape[0], tau_out.shape[1]
    ncosmo = tables.shape[0] // nset
    com = np.ascontiguousarray(np.zeros(nmode) if cosmo_of_mode is None else cosmo_of_mode, dtype=np.int32)
    dims = _d([lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax])
    cfg = np.array([rtol, atol, 0.25, 0.80, 0.0, 20.0, 0.3, 5.0, 0.9, 0.0, 1.0 if step_to_outputs else 0.0])
    rec_len = max_steps + 1
    if rec is None:
        rec = np.zeros((nmode, rec_len))
        nrec = np.zeros(nmode, dtype=np.int32)
    y = np.empty((nset * nmode, nout, 20))
    st = np.zeros((nset * nmode, 3), dtype=np.int32)
    rc = lib().h_solve_rr(_p(tables), ncosmo, nset, tables.shape[1], _p(kmodes), _p(com, ctypes.c_int), nmode, _p(tau_out),
                          nout, _p(dims, ctypes.c_int), _p(cfg), int(max_steps), _p(rec), rec_len,
                          _p(nrec, ctypes.c_int), int(record), int(replay), _p(y), _p(st, ctypes.c_int))
    assert rc == 0, rc
    return y, st, rec, nrec


def solve_grouped(tables, kmodes, tau_out, batch_size, *, cosmo_of_mode=None, lmaxg=11, lmaxgp=11, lmaxr=11, lmaxnu=8,
                  nqmax=3, rtol=1e-4, atol=1e-4, pcoeff=0.25, icoeff=0.80, dcoeff=0.0, factormax=20.0, factormin=0.3,
                  max_steps=2048):
    """The kernel's group driver on the host: y [nmode, nout, 20], stats [nmode, 3]."""
    tables = np.ascontiguousarray(np.atleast_2d(tables), dtype=np.float64)
    kmodes = np.ascontiguousarray(kmodes, dtype=np.float64)
    tau_out = np.ascontiguousarray(np.atleast_2d(tau_out), dtype=np.float64)
    nmode, nout = kmodes.shape[0], tau_out.shape[1]
    com = np.ascontiguousarray(np.zeros(nmode) if cosmo_of_mode is None else cosmo_of_mode, dtype=np.int32)
    cfg = np.array([rtol, atol, pcoeff, icoeff, dcoeff, factormax, factormin, 5.0, 0.9, 0.0, 0.0])
    y = np.empty((nmode, nout, 20))
    st = np.zeros((nmode, 3), dtype=np.int32)
    rc = lib().h_solve_grouped(_p(tables), tables.shape[0], tables.shape[1], _p(kmodes), _p(com, ctypes.c_int), nmode,
                               _p(tau_out), nout, _p(_d([lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax]), ctypes.c_int), _p(cfg),
                               int(max_steps), int(batch_size), _p(y), _p(st, ctypes.c_int))
    assert rc == 0, rc
    return y, st


# ---------------------------------------------------------------- adjoint pieces (deb_adjoint.cuh on the host)
def adj_phi(blob, dims, k, tau, x, y):
    """[phi(B(x, y)), x^T f, d phi/da, x^T df/da, d phi/dtau]"""
    out = np.zeros(5)
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    rc = lib().h_adj_phi(_p(blob), blob.shape[0], _p(_d(dims), ctypes.c_int), k, tau, _p(x), _p(y), _p(out))
    assert rc == 0, rc
    return out


def adj_jt(blob, dims, k, tau, x, y, der=False):
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.ascontiguousarray(y, dtype=np.float64)
    z = np.zeros_like(y)
    rc = lib().h_adj_jt(_p(blob), blob.shape[0], _p(_d(dims), ctypes.c_int), k, tau, _p(x), _p(y), _p(z), int(der))
    assert rc == 0, rc
    return z


def adj_solve_wt(blob, dims, k, tau, y, dt, b):
    y = np.ascontiguousarray(y, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    z = np.zeros_like(b)
    rc = lib().h_adj_solve_wt(_p(blob), blob.shape[0], _p(_d(dims), ctypes.c_int), k, tau, _p(y), dt, _p(b), _p(z))
    assert rc == 0, rc
    return z


def adj_outputs(blob, dims, k, a, s):
    s = np.ascontiguousarray(s, dtype=np.float64)
    r, dr = np.zeros(20), np.zeros(20)
    rc = lib().h_adj_outputs(_p(blob), blob.shape[0], _p(_d(dims), ctypes.c_int), k, a, _p(s), _p(r), _p(dr))
    assert rc == 0, rc
    return r, dr


def adjoint(tables, eps, k, tau_out, dims, gy, rtol=1e-5, atol=1e-5, max_steps=20000, ck_cap=32, step_to_outputs=False,
            pcoeff=0.25, icoeff=0.80, dcoeff=0.0, factormax=20.0, factormin=0.3, debug=False, full_info=False):
    """One mode: record (with checkpoints) on tables[0], then the adjoint of
    the cotangent gy [nout, 20]; tables [1 + 2 npar, L] (nominal, then +eps,
    -eps per parameter), tau_out [1 + 2 npar, nout].  Returns (gtheta [npar],
    y_out [nout, 20], (status, accepted, ck_stride, rejected), adjoint status)."""
    tables = np.ascontiguousarray(tables, dtype=np.float64)
    tau_out = np.ascontiguousarray(tau_out, dtype=np.float64)
    npar = (tables.shape[0] - 1) // 2
    nout = tau_out.shape[1]
    cfg = np.array([rtol, atol, pcoeff, icoeff, dcoeff, factormax, factormin, 5.0, 0.9, 0.0,
                    1.0 if step_to_outputs else 0.0])
    gth = np.zeros(npar)
    y = np.zeros((nout, 20))
    info = np.zeros(4, dtype=np.int32)
    eps = np.ascontiguousarray(eps, dtype=np.float64)
    gy = np.ascontiguousarray(gy, dtype=np.float64)
    n = 7 + (dims[0] + 1) + (dims[1] + 1) + (dims[2] + 1) + dims[4] * (dims[3] + 1) + 2
    dbg = np.zeros(n + 1 + nout + max_steps + 1) if debug else None
    rc = lib().h_adjoint(_p(tables), npar, tables.shape[1], k, _p(tau_out), nout, _p(_d(dims), ctypes.c_int), _p(cfg),
                         max_steps, ck_cap, _p(eps), _p(gy), _p(gth), _p(y), _p(info, ctypes.c_int),
                         None if dbg is None else _p(dbg))
    if debug:
        return gth, y, tuple(int(v) for v in info[:3]), rc, dict(lam0=dbg[:n], dts=dbg[n], dto=dbg[n + 1:n + 1 + nout],
                                                             rec=dbg[n + 1 + nout:n + 2 + nout + int(info[1])])
    return gth, y, tuple(int(v) for v in info[:3]) + ((int(info[3]),) if full_info else ()), rc


def step_adj(tables, eps, dims, k, t0, dt, y0, lam=None):
    """One step on tables[0]: y1; with lam also (ybar0, [tbar0, dtbar], thbar)."""
    tables = np.ascontiguousarray(tables, dtype=np.float64)
    npar = (tables.shape[0] - 1) // 2
    y0 = np.ascontiguousarray(y0, dtype=np.float64)
    y1 = np.zeros_like(y0)
    yb, tb, th = np.zeros_like(y0), np.zeros(2), np.zeros(max(npar, 1))
    eps = np.ascontiguousarray(eps, dtype=np.float64)
    lp = None if lam is None else np.ascontiguousarray(lam, dtype=np.float64)
    rc = lib().h_step_adj(_p(tables), npar, tables.shape[1], _p(_d(dims), ctypes.c_int), k, t0, dt, _p(y0), _p(eps),
                          None if lp is None else _p(lp), _p(y1), _p(yb), _p(tb), _p(th))
    assert rc == 0, rc
    return y1 if lam is None else (y1, yb, tb, th[:npar])


def adj_solve_m(blob, dims, k, tau, y, dt, b, trans):
    y = np.ascontiguousarray(y, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    z = np.zeros_like(b)
    rc = lib().h_adj_solve_m(_p(blob), blob.shape[0], _p(_d(dims), ctypes.c_int), k, tau, _p(y), dt, _p(b), _p(z),
                             int(trans))
    assert rc == 0, rc
    return z


def adj_outputs_pair(blob, dims, k, y):
    """(fields as the forward kernel converts y, fields as the adjoint does)"""
    y = np.ascontiguousarray(y, dtype=np.float64)
    rk, rs = np.zeros(20), np.zeros(20)
    rc = lib().h_adj_outputs_pair(_p(blob), blob.shape[0], _p(_d(dims), ctypes.c_int), k, _p(y), _p(rk), _p(rs))
    assert rc == 0, rc
    return rk, rs
