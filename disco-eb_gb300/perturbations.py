"""Reference-facing API of the perturbation hot path (GPU only).

Mirrors ``discoeb.perturbations`` (``src/discoeb/perturbations.py``):

* :func:`evolve_perturbations` -- same keyword-only signature and the same
  ``(y, kmodes, param)`` return as ``perturbations.py:926-997``;
* :func:`evolve_perturbations_batched` -- signature of
  ``perturbations.py:1000-1061``, returns ``(y, kmodes)``;
* :func:`get_power` -- ``perturbations.py:1101-1123``;
* :func:`evolve_perturbations_multi` -- many cosmologies in one launch (no
  reference counterpart; the reference handles one ``param`` per call).

All integration runs in the CUDA library through the C ABI; ``param`` is
packed into the FP64 table blob (:mod:`tables`) and uploaded.  When a mode
fails (max_steps reached, non-finite state) the call raises RuntimeError like
diffrax does with ``throw=True``, unless ``throw=False``.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from . import autotune as _autotune
from . import tables as _tables

_plans: dict = {}


def _torch():
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("discoeb_gb300 needs a CUDA device; none is available")
    return torch


def nvar(lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax) -> int:
    """Number of ODE variables (``perturbations.py:739``)."""
    return 7 + (lmaxg + 1) + (lmaxgp + 1) + (lmaxr + 1) + nqmax * (lmaxnu + 1) + 2


def _dims(lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax, nout, return_full, linear_solver, exec_mode="auto"):
    ls = {"structured": _native.DEB_SOLVE_STRUCTURED, "dense": _native.DEB_SOLVE_DENSE}[linear_solver]
    return _native.DebDims(lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax, nout, 1 if return_full else 0, ls,
                           _native.EXEC_MODES[exec_mode])


def _cfg(rtol, atol, pcoeff, icoeff, dcoeff, factormax, factormin, max_steps, safety=0.9, error_order=5.0,
         hist_on_reject=False, step_to_outputs=False):
    return _native.DebSolverCfg(rtol, atol, pcoeff, icoeff, dcoeff, factormax, factormin, safety, error_order,
                                int(max_steps), 1 if hist_on_reject else 0, 1 if step_to_outputs else 0)


# Attempted steps per mode peak near k = 0.15 / Mpc (tens of steps at
# k = 1e-4, ~1500 at the peak, a few hundred at k = 1-10 for the
# fiducial-like cosmologies); the first launch of a problem hands modes out
# in order of distance from that peak.
K_STEP_PEAK = 0.15


def schedule_order(kmodes: np.ndarray, cost=None) -> np.ndarray:
    """Queue order (a permutation), most expensive modes first: by measured
    cost (e.g. attempted steps of an earlier launch) when given, else by
    |ln(k / K_STEP_PEAK)|."""
    if cost is not None:
        return np.argsort(-np.asarray(cost, dtype=np.float64), kind="stable").astype(np.int32)
    k = np.asarray(kmodes, dtype=np.float64)
    ok = np.isfinite(k) & (k > 0)
    key = np.full(k.shape, np.inf)          # invalid k (rejected by the kernel) last
    key[ok] = np.abs(np.log(k[ok] / K_STEP_PEAK))
    return np.argsort(key, kind="stable").astype(np.int32)


def launch_ordered(plan, order, nmode: int, fn):
    """Run fn() (one launch on plan) with queue order ``order`` (device int32
    tensor or None) set for that launch only."""
    L = _native.load()
    if order is not None:
        _native.check(L.deb_plan_set_order(plan.ptr, ctypes.c_void_p(order.data_ptr()), int(nmode)), "deb_plan_set_order")
    try:
        return fn()
    finally:
        if order is not None:
            L.deb_plan_set_order(plan.ptr, None, 0)


def get_plan(dims: _native.DebDims, nmode: int, launch=None) -> _native.Plan:
    """Cached plan for these hierarchy sizes with room for >= nmode modes.

    ``launch`` = (stage vectors, modes-per-SM cap) overrides the launch shape;
    by default the shape :mod:`autotune` chose for these sizes is used, else
    the library's default."""
    torch = _torch()
    if launch is None:
        launch = _autotune.chosen(dims)
    key = (torch.cuda.current_device(), dims.lmaxg, dims.lmaxgp, dims.lmaxr, dims.lmaxnu, dims.nqmax, dims.nout,
           dims.return_full, dims.linear_solver, dims.exec_mode, launch)
    p = _plans.get(key)
    # an automatic plan is re-made when the batch size moves it across the
    # lane/warp threshold (the execution mode is fixed at plan creation)
    if p is None or p.max_modes < nmode or (dims.exec_mode == 0 and p.max_modes > 4 * max(nmode, 1)):
        _plans.pop(key, None)
        p = _native.Plan(dims, max(nmode, 1), launch)
        _plans[key] = p
    return p


class DeviceProblem:
    """Device-resident inputs/outputs of one launch, reusable across launches.

    ``tables`` [ncosmo, blob_len], ``kmodes`` [nmode], ``cosmo_of_mode``
    [nmode], ``tau_out`` [ncosmo, nout] -- numpy or torch; moved to the
    current CUDA device once.  :meth:`launch` enqueues ``deb_forward`` on a
    stream without synchronising.
    """

    def __init__(self, tables, kmodes, tau_out, cosmo_of_mode=None, *, lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax,
                 return_full=False, linear_solver="structured", exec_mode="auto"):
        torch = _torch()
        dev = torch.device("cuda", torch.cuda.current_device())
        as_t = lambda a, dt: (a if torch.is_tensor(a) else torch.as_tensor(np.ascontiguousarray(a))).to(dev, dt).contiguous()
        self.tables = as_t(np.atleast_2d(tables) if not torch.is_tensor(tables) else tables, torch.float64)
        self.k = as_t(kmodes, torch.float64)
        self.tau_out = as_t(np.atleast_2d(tau_out) if not torch.is_tensor(tau_out) else tau_out, torch.float64)
        self.nmode = int(self.k.shape[0])
        self.ncosmo = int(self.tables.shape[0])
        self.blob_len = int(self.tables.shape[1])
        self.nout = int(self.tau_out.shape[1])
        if cosmo_of_mode is None:
            self.cosmo = None
        else:
            self.cosmo = as_t(cosmo_of_mode, torch.int32)
        self.dims = _dims(lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax, self.nout, return_full, linear_solver, exec_mode)
        self.n = nvar(lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax)
        self.osz = self.n if return_full else 20
        self.y = torch.empty((self.nmode, self.nout, self.osz), dtype=torch.float64, device=dev)
        self.status = torch.empty((self.nmode,), dtype=torch.int32, device=dev)
        self.steps = torch.empty((self.nmode, 2), dtype=torch.int32, device=dev)
        self.plan = get_plan(self.dims, self.nmode)
        self.device = dev
        host_k = self.k.cpu().numpy() if self.nmode else np.zeros(0)
        self.order = torch.as_tensor(schedule_order(host_k)).to(dev) if self.nmode else None

    def reorder_by_steps(self):
        """Hand modes out longest-first by the attempted steps of the last
        launch (synchronises; results do not depend on the order)."""
        torch = _torch()
        torch.cuda.synchronize()
        st = self.steps.cpu().numpy()
        self.order = torch.as_tensor(schedule_order(None, st[:, 0] + st[:, 1])).to(self.device)
        torch.cuda.synchronize()

    def launch(self, cfg: _native.DebSolverCfg, stream=None):
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream()
        L = _native.load()
        rc = launch_ordered(self.plan, self.order, self.nmode, lambda: L.deb_forward(
            self.plan.ptr, ctypes.c_void_p(self.tables.data_ptr()), self.ncosmo, self.blob_len,
            ctypes.c_void_p(self.k.data_ptr()), ctypes.c_void_p(self.cosmo.data_ptr() if self.cosmo is not None else 0),
            self.nmode, ctypes.c_void_p(self.tau_out.data_ptr()), ctypes.byref(cfg), ctypes.c_void_p(self.y.data_ptr()),
            ctypes.c_void_p(self.status.data_ptr()), ctypes.c_void_p(self.steps.data_ptr()), ctypes.c_void_p(s.cuda_stream)))
        _native.check(rc, "deb_forward")

    def tune(self, cfg: _native.DebSolverCfg, candidates=_autotune.CANDIDATES):
        """Time this problem's launch for each candidate launch shape
        (:mod:`autotune`), keep the fastest plan; returns {shape: ms}."""
        if self.dims.exec_mode == _native.EXEC_MODES["lane"] or self.nmode == 0:
            return {}
        L = _native.load()

        def launch(plan, s):
            _native.check(launch_ordered(plan, self.order, self.nmode, lambda: L.deb_forward(
                plan.ptr, ctypes.c_void_p(self.tables.data_ptr()), self.ncosmo, self.blob_len,
                ctypes.c_void_p(self.k.data_ptr()),
                ctypes.c_void_p(self.cosmo.data_ptr() if self.cosmo is not None else 0), self.nmode,
                ctypes.c_void_p(self.tau_out.data_ptr()), ctypes.byref(cfg), ctypes.c_void_p(self.y.data_ptr()),
                ctypes.c_void_p(self.status.data_ptr()), ctypes.c_void_p(self.steps.data_ptr()),
                ctypes.c_void_p(s.cuda_stream))), "deb_forward")

        best, times = _autotune.tune(self.dims, self.nmode, launch, candidates)
        self.plan = get_plan(self.dims, self.nmode, best)
        return times

    def capture(self, cfg: _native.DebSolverCfg, idx: int = 4):
        """Capture the whole solve (queue reset, the persistent launch and
        get_power) as one CUDA graph; :meth:`replay` re-runs it on the
        current stream with whatever the input buffers hold and returns the
        graph's P(k) buffer [nmode, nout].  Runs the solve once eagerly
        first (its y, status and steps are left in place) and returns that
        run's P(k); the capture itself executes nothing."""
        torch = _torch()
        self.launch(cfg)                  # untimed launch outside the capture
        P = self.power(idx)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            s = torch.cuda.current_stream()
            self.launch(cfg, s)
            self.graph_P = self.power(idx, s)
        self.graph = g
        return P

    def replay(self):
        self.graph.replay()
        return self.graph_P

    def power(self, idx: int, stream=None):
        """P(k) of field ``idx`` for every mode and output, on the device."""
        torch = _torch()
        s = stream if stream is not None else torch.cuda.current_stream()
        P = torch.empty((self.nmode, self.nout), dtype=torch.float64, device=self.device)
        rc = _native.load().deb_get_power(ctypes.c_void_p(self.tables.data_ptr()), self.ncosmo, self.blob_len,
                                          ctypes.c_void_p(self.k.data_ptr()),
                                          ctypes.c_void_p(self.cosmo.data_ptr() if self.cosmo is not None else 0),
                                          self.nmode, self.nout, ctypes.c_void_p(self.y.data_ptr()), self.osz, int(idx),
                                          ctypes.c_void_p(P.data_ptr()), ctypes.c_void_p(s.cuda_stream))
        _native.check(rc, "deb_get_power")
        return P


def _check_status(status: np.ndarray, kmodes: np.ndarray, throw: bool):
    bad = np.nonzero(status != 0)[0]
    if bad.size and throw:
        names = [f"k={kmodes[i]:.4g}:{_native.MODE_STATUS.get(int(status[i]), status[i])}" for i in bad[:8]]
        raise RuntimeError(f"{bad.size} mode(s) failed: " + ", ".join(names) + (" ..." if bad.size > 8 else ""))


def solve(tables, kmodes, tau_out, cosmo_of_mode=None, *, lmaxg=11, lmaxgp=11, lmaxr=11, lmaxnu=8, nqmax=3,
          rtol=1e-4, atol=1e-4, pcoeff=0.25, icoeff=0.80, dcoeff=0.0, factormax=20.0, factormin=0.3, max_steps=2048,
          return_full=False, linear_solver="structured", throw=True, return_stats=False, output="numpy",
          error_order=5.0, safety=0.9, hist_on_reject=False, exec_mode="auto", step_to_outputs=False):
    """Integrate modes of packed cosmologies on the GPU; y [nmode, nout, 20|nvar]."""
    torch = _torch()
    prob = DeviceProblem(tables, kmodes, tau_out, cosmo_of_mode, lmaxg=lmaxg, lmaxgp=lmaxgp, lmaxr=lmaxr, lmaxnu=lmaxnu,
                         nqmax=nqmax, return_full=return_full, linear_solver=linear_solver, exec_mode=exec_mode)
    cfg = _cfg(rtol, atol, pcoeff, icoeff, dcoeff, factormax, factormin, max_steps, safety, error_order, hist_on_reject,
               step_to_outputs)
    prob.launch(cfg)
    status = prob.status.cpu().numpy()
    _check_status(status, np.asarray(kmodes if not torch.is_tensor(kmodes) else kmodes.cpu()), throw)
    y = prob.y if output == "torch" else prob.y.cpu().numpy()
    if return_stats:
        return y, {"status": status, "steps": prob.steps.cpu().numpy()}
    return y


def evolve_perturbations(*, param, aexp_out, kmin: float, kmax: float, num_k: int, lmaxg: int = 11, lmaxgp: int = 11,
                         lmaxr: int = 11, lmaxnu: int = 8, nqmax: int = 3, rtol: float = 1e-4, atol: float = 1e-4,
                         pcoeff: float = 0.25, icoeff: float = 0.80, dcoeff: float = 0.0, factormax: float = 20.0,
                         factormin: float = 0.3, max_steps: int = 2048, return_full: bool = False, dologk: bool = True,
                         throw: bool = True, linear_solver: str = "structured", output: str = "numpy"):
    """Evolve the synchronous-gauge perturbations of all k-modes on the GPU.

    Same arguments and return value as ``perturbations.py:926-997``:
    ``y`` is ``[num_k, nout, 20]`` (``[num_k, nout, nvar]`` with
    ``return_full``), ``kmodes`` the geomspace (or linspace) grid, and
    ``param`` is updated in place with lmax*/nqmax/nout/tau_out.
    """
    kmodes = np.geomspace(kmin, kmax, num_k) if dologk else np.linspace(kmin, kmax, num_k)
    aexp_out = np.atleast_1d(np.asarray(aexp_out, dtype=np.float64))
    tau_out = _tables.tau_of_a(param, aexp_out)
    blob = _tables.pack_cosmology(param, nqmax)
    y = solve(blob[None, :], kmodes, tau_out[None, :], None, lmaxg=lmaxg, lmaxgp=lmaxgp, lmaxr=lmaxr, lmaxnu=lmaxnu,
              nqmax=nqmax, rtol=rtol, atol=atol, pcoeff=pcoeff, icoeff=icoeff, dcoeff=dcoeff, factormax=factormax,
              factormin=factormin, max_steps=max_steps, return_full=return_full, linear_solver=linear_solver,
              throw=throw, output=output)
    param["lmaxg"] = lmaxg
    param["lmaxgp"] = lmaxgp
    param["lmaxr"] = lmaxr
    param["lmaxnu"] = lmaxnu
    param["nqmax"] = nqmax
    param["nout"] = aexp_out.shape[0]
    param["tau_out"] = tau_out
    return y, kmodes, param


def solve_grouped(tables, kmodes, tau_out, batch_size: int, cosmo_of_mode=None, *, lmaxg=11, lmaxgp=11, lmaxr=11,
                  lmaxnu=8, nqmax=3, rtol=1e-4, atol=1e-4, pcoeff=0.25, icoeff=0.80, dcoeff=0.0, factormax=20.0,
                  factormin=0.3, max_steps=2048, throw=True, return_stats=False, output="numpy"):
    """Groups of ``batch_size`` consecutive modes sharing one start time and one
    step sequence (``deb_forward_grouped``); y [nmode, nout, 20]."""
    torch = _torch()
    dev = torch.device("cuda", torch.cuda.current_device())
    as_t = lambda a, dt: (a if torch.is_tensor(a) else torch.as_tensor(np.ascontiguousarray(a))).to(dev, dt).contiguous()
    tabs = as_t(np.atleast_2d(tables) if not torch.is_tensor(tables) else tables, torch.float64)
    k = as_t(kmodes, torch.float64)
    tau = as_t(np.atleast_2d(tau_out) if not torch.is_tensor(tau_out) else tau_out, torch.float64)
    nmode, nout = int(k.shape[0]), int(tau.shape[1])
    if nmode % batch_size:
        raise ValueError("the number of modes must be divisible by batch_size")
    com = as_t(np.zeros(nmode, dtype=np.int32) if cosmo_of_mode is None else cosmo_of_mode, torch.int32)
    dims = _dims(lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax, nout, False, "structured", "warp")
    key = ("grouped", torch.cuda.current_device(), lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax, nout, int(batch_size))
    plan = _plans.get(key)
    if plan is None or plan.max_modes < nmode:
        plan = _native.Plan(dims, max(nmode, 1), batch_size=int(batch_size))
        _plans[key] = plan
    cfg = _cfg(rtol, atol, pcoeff, icoeff, dcoeff, factormax, factormin, max_steps)
    y = torch.empty((nmode, nout, 20), dtype=torch.float64, device=dev)
    status = torch.empty((nmode,), dtype=torch.int32, device=dev)
    steps = torch.empty((nmode, 2), dtype=torch.int32, device=dev)
    c = lambda t: ctypes.c_void_p(t.data_ptr())
    _native.check(_native.load().deb_forward_grouped(plan.ptr, c(tabs), int(tabs.shape[0]), int(tabs.shape[1]), c(k),
                                                     c(com), nmode, c(tau), ctypes.byref(cfg), c(y), c(status), c(steps),
                                                     ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)),
                  "deb_forward_grouped")
    st = status.cpu().numpy()
    _check_status(st, k.cpu().numpy(), throw)
    out = y if output == "torch" else y.cpu().numpy()
    if return_stats:
        return out, {"status": st, "steps": steps.cpu().numpy()}
    return out


def evolve_perturbations_batched(*, param, aexp_out, kmin: float, kmax: float, num_k: int, lmaxg: int = 11,
                                 lmaxgp: int = 11, lmaxr: int = 11, lmaxnu: int = 8, nqmax: int = 3, rtol: float = 1e-4,
                                 atol: float = 1e-4, pcoeff: float = 0.25, icoeff: float = 0.80, dcoeff: float = 0.0,
                                 factormax: float = 20.0, factormin: float = 0.3, max_steps: int = 2048,
                                 batch_size: int = 16, throw: bool = True, output: str = "numpy",
                                 grouped: bool = True):
    """Signature and semantics of ``perturbations.py:1000-1061``; returns ``(y, kmodes)``.

    As in the reference, ``batch_size`` consecutive modes (of the geomspace
    grid) form a group that starts at the group's smallest start time and
    takes one shared step sequence, controlled by one error norm over all its
    modes (``deb_forward_grouped``, one warp per group).  ``grouped=False``
    gives every mode its own start time and steps instead (the
    :func:`evolve_perturbations` semantics, the persistent per-mode kernel).
    ``batch_size`` must divide ``num_k`` as in the reference (1 to 32 here).
    """
    if num_k % batch_size != 0:
        raise ValueError("num_k must be divisible by batch_size")
    if not grouped:
        y, kmodes, _ = evolve_perturbations(param=dict(param), aexp_out=aexp_out, kmin=kmin, kmax=kmax, num_k=num_k,
                                            lmaxg=lmaxg, lmaxgp=lmaxgp, lmaxr=lmaxr, lmaxnu=lmaxnu, nqmax=nqmax,
                                            rtol=rtol, atol=atol, pcoeff=pcoeff, icoeff=icoeff, dcoeff=dcoeff,
                                            factormax=factormax, factormin=factormin, max_steps=max_steps,
                                            throw=throw, output=output)
        param["nout"] = np.atleast_1d(aexp_out).shape[0]
        return y, kmodes
    kmodes = np.geomspace(kmin, kmax, num_k)
    aexp_out = np.atleast_1d(np.asarray(aexp_out, dtype=np.float64))
    tau_out = _tables.tau_of_a(param, aexp_out)
    blob = _tables.pack_cosmology(param, nqmax)
    y = solve_grouped(blob[None, :], kmodes, tau_out[None, :], batch_size, None, lmaxg=lmaxg, lmaxgp=lmaxgp,
                      lmaxr=lmaxr, lmaxnu=lmaxnu, nqmax=nqmax, rtol=rtol, atol=atol, pcoeff=pcoeff, icoeff=icoeff,
                      dcoeff=dcoeff, factormax=factormax, factormin=factormin, max_steps=max_steps, throw=throw,
                      output=output)
    param["nout"] = aexp_out.shape[0]
    return y, kmodes


def evolve_perturbations_multi(*, params, aexp_out, kmin: float, kmax: float, num_k: int, lmaxg: int = 11,
                               lmaxgp: int = 11, lmaxr: int = 11, lmaxnu: int = 8, nqmax: int = 3, rtol: float = 1e-4,
                               atol: float = 1e-4, pcoeff: float = 0.25, icoeff: float = 0.80, dcoeff: float = 0.0,
                               factormax: float = 20.0, factormin: float = 0.3, max_steps: int = 2048,
                               return_full: bool = False, dologk: bool = True, throw: bool = True,
                               linear_solver: str = "structured", output: str = "numpy"):
    """All modes of many cosmologies in one persistent launch.

    Returns ``y [ncosmo, num_k, nout, 20]`` and ``kmodes``.
    """
    kmodes = np.geomspace(kmin, kmax, num_k) if dologk else np.linspace(kmin, kmax, num_k)
    aexp_out = np.atleast_1d(np.asarray(aexp_out, dtype=np.float64))
    tabs = _tables.pack_batch(params, nqmax)
    tau = np.stack([_tables.tau_of_a(p, aexp_out) for p in params])
    nc = len(params)
    kk = np.tile(kmodes, nc)
    com = np.repeat(np.arange(nc, dtype=np.int32), num_k)
    y = solve(tabs, kk, tau, com, lmaxg=lmaxg, lmaxgp=lmaxgp, lmaxr=lmaxr, lmaxnu=lmaxnu, nqmax=nqmax, rtol=rtol,
              atol=atol, pcoeff=pcoeff, icoeff=icoeff, dcoeff=dcoeff, factormax=factormax, factormin=factormin,
              max_steps=max_steps, return_full=return_full, linear_solver=linear_solver, throw=throw, output=output)
    return y.reshape(nc, num_k, aexp_out.shape[0], -1), kmodes


def get_power(*, k, y, idx: int, param: dict):
    """P(k) = 2 pi^2 A_s (k/k_p)^(n_s-1) k^-3 y[..., idx]^2 (``perturbations.py:1101-1123``).

    Evaluated on the GPU by ``deb_get_power``.  ``y`` may have shape
    ``[num_k, 20]`` or ``[num_k, nout, 20]`` (numpy or CUDA tensor); the
    result has ``y``'s shape without the last axis and the container type of
    ``y``.
    """
    torch = _torch()
    is_t = torch.is_tensor(y)
    dev = torch.device("cuda", torch.cuda.current_device())
    yt = (y if is_t else torch.as_tensor(np.asarray(y, dtype=np.float64))).to(dev, torch.float64).contiguous()
    kt = (k if torch.is_tensor(k) else torch.as_tensor(np.asarray(k, dtype=np.float64))).to(dev, torch.float64).contiguous()
    shape = tuple(yt.shape[:-1])
    nmode = int(kt.shape[0])
    nout = int(np.prod(shape[1:])) if len(shape) > 1 else 1
    if int(np.prod(shape)) != nmode * nout:
        raise ValueError("y must be [num_k, ..., nfields] with num_k == len(k)")
    hdr = np.zeros((1, _tables.HDR_LEN + 3 * 2 * 7 + 2), dtype=np.float64)
    hdr[0, 16] = float(param["A_s"])
    hdr[0, 17] = float(param["n_s"])
    hdr[0, 18] = float(param.get("k_p", 0.05))
    ht = torch.as_tensor(hdr).to(dev)
    P = torch.empty((nmode, nout), dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream()
    rc = _native.load().deb_get_power(ctypes.c_void_p(ht.data_ptr()), 1, hdr.shape[1], ctypes.c_void_p(kt.data_ptr()),
                                      ctypes.c_void_p(0), nmode, nout, ctypes.c_void_p(yt.data_ptr()), int(yt.shape[-1]),
                                      int(idx), ctypes.c_void_p(P.data_ptr()), ctypes.c_void_p(s.cuda_stream))
    _native.check(rc, "deb_get_power")
    P = P.reshape(shape)
    return P if is_t else P.cpu().numpy()
