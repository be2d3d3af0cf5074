"""The library's table producer (``deb_evolve_background`` on the GPU,
``deb_evolve_background_host`` on the host cores).

The RECFAST branch of ``evolve_background`` (``src/discoeb/background.py:140-342``
with ``thermodynamics_recfast.py:124-501``) for many parameter sets at once,
written straight into the table blobs the solver reads.  The algorithm is the
one of :mod:`background` / :mod:`recfast`: the same sampling grids, quadrature
nodes and constants are passed to the compiled code from those modules, so
its tables agree with theirs to rounding.

:func:`evolve_background_tables` (GPU, one warp per set: parameter dicts in,
``[nset, blob_len]`` device tables out, optionally ``tau_of_a`` at given scale
factors) and :func:`evolve_background_tables_host` (the same code on worker
threads, numpy blobs out).  One RECFAST history is a long sequential chain of
small FP64 steps: a CPU core builds a set in ~2 ms, one GPU lane in ~130 ms,
so the host producer is the faster one for the set counts of a gradient call.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np

from . import _native
from . import background as _bg
from . import recfast as _rf
from . import tables as _tables

# order of deb_tables_const in include/discoeb_gb300.h
CONST_NAMES = (
    "G_N", "M_H", "M_E", "MHE_MH", "C_LIGHT", "H_PLANCK", "K_B", "BIG_H", "DENS_FAC", "E_ION_HE12S", "LAMBDA_H",
    "LAMBDA_HE", "L_HE1_ION", "L_HE_2P", "A2P_S", "A2P_T", "L_HE_2PT", "SIGMA_HE_2PS", "SIGMA_HE_2PT", "AGAUSS1",
    "AGAUSS2", "ZGAUSS1", "ZGAUSS2", "WGAUSS1", "WGAUSS2", "H_FRAC", "CDB", "CDB_HE", "CB1", "CR", "CK", "CK_HE",
    "CL", "CL_HE", "CT", "BFACT", "CL_PST", "HCL_HE2ST_KB", "HCL_HE2ST_ION_KB", "A_PPB", "B_PPB", "C_PPB", "D_PPB",
    "A_VF", "B_VF", "T_0", "T_1", "A_TRIP", "B_TRIP", "FU", "_G", "_G21", "_G31", "_G32", "_G41", "_G42", "_G43",
    "_A21", "_A31", "_A32", "_CH1", "_CH2", "_CH3", "_C1", "_C2", "_C3", "_C4")
# order of deb_bg_param
PARAM_KEYS = ("Omegam", "Omegab", "H0", "Tcmb", "YHe", "Neff", "Nmnu", "mnu", "w_DE_0", "w_DE_a", "cs2_DE", "A_s",
              "n_s", "k_p", "Omegak")
PARAM_DEFAULTS = {"cs2_DE": 1.0, "k_p": 0.05, "Omegak": 0.0}

AMIN, AMAX = 1e-9, 1.01      # evolve_background's range (background.py:191-200)
NUM_NU, NQ_BG = 512, 8       # neutrino table points and momentum bins (background.py:158, 47)


class DebBgCfg(ctypes.Structure):
    _fields_ = [("num_thermo", ctypes.c_int), ("num_nu", ctypes.c_int), ("nq_bg", ctypes.c_int), ("nqmax", ctypes.c_int),
                ("max_steps", ctypes.c_int), ("amin", ctypes.c_double), ("rtol", ctypes.c_double),
                ("atol", ctypes.c_double)]


def constants() -> np.ndarray:
    """The RECFAST constants, fitting parameters and GRK4A coefficients of the
    host producer, plus pi, sqrt(pi) and the neutrino mass conversion."""
    vals = [float(getattr(_rf, n)) for n in CONST_NAMES] + [math.pi, math.sqrt(math.pi), _bg.C2OK]
    return np.array(vals, dtype=np.float64)


def grid(num_thermo: int, nqmax: int) -> np.ndarray:
    """Parameter-independent inputs: neutrino table scale factors and logs,
    both momentum quadratures, the RECFAST sampling and its logs."""
    a_nu = np.geomspace(AMIN * 0.9, AMAX * 1.1, NUM_NU)
    q_bg, w_bg = _bg.get_neutrino_momentum_bins(NQ_BG)
    q, w = _bg.get_neutrino_momentum_bins(nqmax)
    a_th = _rf.adaptive_sampling(AMIN, AMAX, num_thermo + 1)
    return np.ascontiguousarray(np.concatenate([a_nu, np.log(a_nu), q_bg, w_bg, q, w, a_th, np.log(a_th[1:])]))


def param_matrix(params) -> np.ndarray:
    rows = []
    for p in params:
        rows.append([float(p["H0"]) if k == "H0" else float(p.get(k, PARAM_DEFAULTS.get(k, np.nan))) for k in PARAM_KEYS])
    m = np.array(rows, dtype=np.float64)
    if np.isnan(m).any():
        missing = [k for j, k in enumerate(PARAM_KEYS) if np.isnan(m[:, j]).any()]
        raise KeyError(f"parameter set(s) missing {missing}")
    return m


def blob_len(num_thermo: int, nqmax: int) -> int:
    return _tables.blob_length([num_thermo, num_thermo, NUM_NU, NUM_NU, num_thermo, num_thermo, num_thermo], nqmax)


_static = {}
# GRK4A step ends recorded per RECFAST sample for the frozen form (the
# histories at rtol 1e-3 take a few per sample)
STEP_CAP_PER_SAMPLE = 16


def _leader_array(leader, nset):
    """Checked leader indices (-1: adaptive; j: follow set j's steps)."""
    ld = np.ascontiguousarray(np.asarray(leader, dtype=np.int32))
    if ld.shape != (nset,):
        raise ValueError(f"leader must have one entry per set ({nset}), got shape {ld.shape}")
    fol = ld >= 0
    if (ld < -1).any() or (ld[fol] >= nset).any() or (ld[ld[fol]] >= 0).any():
        raise ValueError("a leader must be -1 or the index of a set whose own leader is -1")
    return ld


def follow_nominal(ncosmo: int, nper: int):
    """Leader indices for the layout [ncosmo nominal sets, then nper
    perturbed sets per cosmology]: the nominal sets adaptive, each perturbed
    set on its cosmology's nominal step sequence."""
    return np.concatenate([np.full(ncosmo, -1, np.int32), np.repeat(np.arange(ncosmo, dtype=np.int32), nper)])


def evolve_background_tables(params, nqmax: int, *, num_thermo: int = 256, aexp_out=None, rtol: float = 1e-3,
                             atol: float = 1e-6, max_steps: int = 128, stream=None, out=None, tau_out=None,
                             leader=None):
    """Table blobs of every parameter set on the current CUDA device.

    ``params``: list of dicts with the keys ``evolve_background`` reads.
    Returns ``(tables [nset, blob_len], tau [nset, nout] or None, status
    [nset])`` as torch tensors on the device (stream-ordered, no host sync);
    ``out`` / ``tau_out`` may pass preallocated buffers.  A nonzero status
    (``DEB_BG_*`` bits) means an interval of the ionisation history used up
    its step budget or a frozen step record was incomplete.  ``leader`` (one
    int per set, see :func:`follow_nominal`) puts sets on the recorded step
    sequence of another set (``deb_evolve_background_frozen``).
    """
    import torch

    L = _native.load()
    dev = torch.device("cuda", torch.cuda.current_device())
    s = stream if stream is not None else torch.cuda.current_stream()
    key = (dev.index, num_thermo, nqmax)
    if key not in _static:
        _static[key] = (torch.as_tensor(constants()).to(dev), torch.as_tensor(grid(num_thermo, nqmax)).to(dev))
    consts, grd = _static[key]
    pm = torch.as_tensor(param_matrix(params)).to(dev, non_blocking=True)
    nset = pm.shape[0]
    bl = blob_len(num_thermo, nqmax)
    rc_len = L.deb_tables_blob_len(num_thermo, NUM_NU, nqmax)
    if rc_len != bl:
        raise RuntimeError(f"blob length mismatch: host {bl}, library {rc_len}")
    tabs = out if out is not None else torch.empty((nset, bl), dtype=torch.float64, device=dev)
    status = torch.empty((nset,), dtype=torch.int32, device=dev)
    cfg = DebBgCfg(num_thermo, NUM_NU, NQ_BG, nqmax, max_steps, AMIN, rtol, atol)
    c = lambda t: ctypes.c_void_p(t.data_ptr())
    with torch.cuda.stream(s):
        if leader is None:
            _native.check(L.deb_evolve_background(ctypes.byref(cfg), c(pm), nset, c(consts), c(grd), c(tabs), bl,
                                                  c(status), ctypes.c_void_p(s.cuda_stream)), "deb_evolve_background")
        else:
            ld = torch.as_tensor(_leader_array(leader, nset)).to(dev, non_blocking=True)
            cap = STEP_CAP_PER_SAMPLE * num_thermo
            steps = torch.empty((nset, 3 * num_thermo + 1 + 2 * cap), dtype=torch.float64, device=dev)
            _native.check(L.deb_evolve_background_frozen(ctypes.byref(cfg), c(pm), nset, c(ld), c(consts), c(grd),
                                                         c(steps), cap, c(tabs), bl, c(status),
                                                         ctypes.c_void_p(s.cuda_stream)),
                          "deb_evolve_background_frozen")
        tau = None
        if aexp_out is not None:
            aexp = torch.as_tensor(np.atleast_1d(np.asarray(aexp_out, dtype=np.float64))).to(dev)
            tau = tau_out if tau_out is not None else torch.empty((nset, aexp.shape[0]), dtype=torch.float64, device=dev)
            _native.check(L.deb_tau_of_a(c(tabs), nset, bl, c(aexp), int(aexp.shape[0]), c(tau),
                                         ctypes.c_void_p(s.cuda_stream)), "deb_tau_of_a")
    return tabs, tau, status


def evolve_background_tables_host(params, nqmax: int, *, num_thermo: int = 256, rtol: float = 1e-3,
                                  atol: float = 1e-6, max_steps: int = 128, nthreads: int = 0, out=None,
                                  leader=None, steps=None):
    """The same producer on the host cores (``deb_evolve_background_host``):
    ``[nset, blob_len]`` numpy blobs (written into ``out``, e.g. pinned
    memory, when given) and the status per set.  One CPU core builds a set
    in a few milliseconds; worker threads split the sets.  ``leader`` as in
    :func:`evolve_background_tables` (``deb_evolve_background_frozen_host``);
    ``steps``, a float64 array ``[nset, 3 num_thermo + 1 + 2 cap]``,
    receives the leaders' step records (layout of
    ``deb_evolve_background_frozen``)."""
    L = _native.load()
    pm = np.ascontiguousarray(param_matrix(params))
    nset = pm.shape[0]
    bl = blob_len(num_thermo, nqmax)
    key = ("host", num_thermo, nqmax)
    if key not in _static:
        _static[key] = (constants(), grid(num_thermo, nqmax))
    consts, grd = _static[key]
    tabs = out if out is not None else np.empty((nset, bl), dtype=np.float64)
    if tabs.shape != (nset, bl) or tabs.dtype != np.float64 or not tabs.flags.c_contiguous:
        raise ValueError(f"out must be a C-contiguous float64 array of shape {(nset, bl)}")
    status = np.zeros(nset, dtype=np.int32)
    cfg = DebBgCfg(num_thermo, NUM_NU, NQ_BG, nqmax, max_steps, AMIN, rtol, atol)
    p = lambda a: ctypes.c_void_p(a.ctypes.data)
    if leader is None:
        _native.check(L.deb_evolve_background_host(ctypes.byref(cfg), p(pm), nset, p(consts), p(grd), p(tabs), bl,
                                                   p(status), int(nthreads)), "deb_evolve_background_host")
    else:
        ld = _leader_array(leader, nset)
        cap = 0
        if steps is not None:
            if steps.dtype != np.float64 or steps.ndim != 2 or steps.shape[0] != nset or not steps.flags.c_contiguous:
                raise ValueError("steps must be a C-contiguous float64 array [nset, 3 num_thermo + 1 + 2 cap]")
            cap = (steps.shape[1] - 3 * num_thermo - 1) // 2
        _native.check(L.deb_evolve_background_frozen_host(ctypes.byref(cfg), p(pm), nset, p(ld), p(consts), p(grd),
                                                          p(steps) if steps is not None else None, cap, p(tabs),
                                                          bl, p(status), int(nthreads)),
                      "deb_evolve_background_frozen_host")
    return tabs, status


def param_from_blob(inputs: dict, blob: np.ndarray) -> dict:
    """A ``param`` dict as ``evolve_background`` returns it, read back from a
    produced blob: the input keys, the scalars the perturbation path reads,
    ``adotrad``, the seven splines (fields ``_x_``, ``_y_``, ``_S_full_``; the
    second derivatives are the producer's) and the ``a``, ``aexp``, ``tau``,
    ``xe``, ``cs2`` arrays.  The ionisation fractions by species, T_m, mu,
    ``taumax`` and the splines the path does not read are not in a blob and
    are not set."""
    from .spline import SplineInterpolation

    b = np.asarray(blob, dtype=np.float64)
    out = dict(inputs)
    out.setdefault("Omegak", 0.0)
    for i, key in enumerate(_tables.SCALAR_KEYS):
        out[key] = float(b[i])
    out["adotrad"] = math.sqrt((out["grhog"] + out["grhor"] * (out["Neff"] + out["Nmnu"])) / 3.0)
    sizes = b[_tables.H_NSPL0:_tables.H_NSPL0 + 7].astype(int)
    p = _tables.HDR_LEN
    for key, n in zip(_tables.SPLINE_KEYS, sizes):
        sp = SplineInterpolation.__new__(SplineInterpolation)
        sp._x_, sp._y_, sp._S_full_ = b[p:p + n].copy(), b[p + n:p + 2 * n].copy(), b[p + 2 * n:p + 3 * n].copy()
        sp._n_ = int(n)
        out[key] = sp
        p += 3 * n
    out["aexp"] = out["tau_of_a_spline"]._x_.copy()
    out["tau"] = out["tau_of_a_spline"]._y_.copy()
    out["xe"] = out["xe_of_tau_spline"]._y_.copy()
    out["cs2"] = out["cs2a_of_loga_spline"]._y_ / out["aexp"]
    out["a"] = np.exp(out["logrhonu_of_loga_spline"]._x_)
    out["amin"], out["amax"] = AMIN, AMAX
    return out


def evolve_backgrounds_native(params, *, num_thermo: int = 256, nthreads: int = 0):
    """``evolve_background`` of many parameter dicts by the library's
    producer on the host cores (a few milliseconds per set); returns the
    ``param`` dicts of :func:`param_from_blob`."""
    blobs, status = evolve_background_tables_host(params, 3, num_thermo=num_thermo, nthreads=nthreads)
    if (status != 0).any():
        raise RuntimeError(f"{int((status != 0).sum())} parameter set(s): an ionisation interval ran out of steps")
    return [param_from_blob(p, b) for p, b in zip(params, blobs)]
