"""d log P(k, a) / d theta on the GPU: tangents of the recorded step sequence.

The reference obtains gradients with ``jax.jacfwd`` through
``evolve_background`` and ``evolve_perturbations`` (notebooks'
``compute_matter_power``; ``DirectAdjoint`` at ``perturbations.py:765``).
diffrax's PID controller stops gradients through its step-size factor, so
every step length is dt0 = tau_start / 4 times frozen factors: under jacfwd
the step times scale with tau_start(theta) (whose derivative flows through
the start-time bisection's final midpoint), and steps ending on an output
time follow tau_out(theta).

Here that quantity is computed by central differences of exactly that map:
``deb_forward_record`` runs the nominal solve and stores every mode's
tau_start and accepted step times, then one ``deb_replay`` launch integrates
all (mode, theta_p +- eps_p) pairs on those steps, rescaled by each set's
own tau_start, with the perturbed tables.  The difference quotient equals
the tangent of that map to O(eps^2) (eps = 1e-4 relative by default); the
map has no step-size decision, so there is no step-selection noise.  ``A_s``
and ``n_s`` enter only ``get_power`` (``perturbations.py:1123``): their
derivatives are analytic.  :class:`PowerSpectrum` wraps the pair as a
``torch.autograd.Function``.
"""
from __future__ import annotations

import ctypes
import multiprocessing as mp
import os

import numpy as np

from . import _native
from . import background as _bg
from . import perturbations as _pt
from . import tables as _tables

THETA = ("Omegam", "Omegab", "h", "n_s", "A_s", "mnu", "w_DE_0", "w_DE_a")
ANALYTIC = ("n_s", "A_s")


def _get(param, name):
    return param["H0"] / 100.0 if name == "h" else param[name]


def _with(param, name, value):
    q = dict(param)
    if name == "h":
        q["H0"] = 100.0 * value
    else:
        q[name] = value
    return q


def _evolve(param):
    return _bg.evolve_background(param=param)


def evolve_backgrounds(params, processes=None, producer: str = "python"):
    """Host table production for many parameter dicts: the Python producer in
    a process pool (spawn), or the library's compiled producer on worker
    threads (``producer="native"``, a few ms per set)."""
    if producer == "native":
        from .tables_gpu import evolve_backgrounds_native

        return evolve_backgrounds_native(list(params))
    processes = processes if processes is not None else min(len(params), os.cpu_count() or 1)
    if processes <= 1 or len(params) <= 1:
        return [_evolve(p) for p in params]
    with mp.get_context("spawn").Pool(processes) as pool:
        return pool.map(_evolve, params)


# Parameters whose values cross zero take eps relative to this scale at least
# (w_a is drawn from [-0.3, 0.3]: eps = 1e-4 |w_a| would be 1e-7 at w_a = 1e-3,
# where the quotient of the solve divides its rounding by 2e-7)
EPS_SCALE = {"w_DE_a": 0.1}


def perturbed_params(cosmo, theta=THETA, rel_step=1e-4):
    """[(name, eps, param_plus, param_minus)] for the ODE parameters of theta:
    eps = rel_step * max(|theta|, EPS_SCALE[name])."""
    out = []
    for name in theta:
        if name in ANALYTIC:
            continue
        v = float(_get(cosmo, name))
        sc = max(abs(v), EPS_SCALE.get(name, 0.0))
        eps = rel_step * sc if sc != 0.0 else rel_step
        out.append((name, eps, _with(cosmo, name, v + eps), _with(cosmo, name, v - eps)))
    return out


TABLE_NAMES = ("tab0", "tau0", "tabs", "taus")
SMALL_NAMES = ("k", "com", "eps", "eps_c", "inv_As", "lnk")


def _host_inputs(plist, backgrounds, pert, kmodes, aexp_out, nqmax):
    """Packed host arrays of one gradient problem: k, cosmology index, eps per
    parameter, 1/A_s and ln(k/k_p) per mode, and -- unless ``backgrounds``
    is ``"gpu"`` -- the table blobs and output times of every set."""
    nc, num_k = len(plist), kmodes.shape[0]
    com = np.repeat(np.arange(nc, dtype=np.int32), num_k)
    kp = np.array([p.get("k_p", 0.05) for p in plist], dtype=np.float64)[com]
    As = np.array([p["A_s"] for p in plist], dtype=np.float64)[com]
    k = np.tile(kmodes, nc)
    h = dict(k=k, com=com,
             eps=np.ascontiguousarray(np.array([[e for (_, e, _, _) in pp] for pp in pert], dtype=np.float64)[com].T),
             eps_c=np.array([[e for (_, e, _, _) in pp] for pp in pert], dtype=np.float64),
             inv_As=(1.0 / As)[:, None], lnk=np.log(k / kp)[:, None])
    if _native_tables(backgrounds):
        from . import tables_gpu

        sets = [q for pp in pert for (_, _, a, b) in pp for q in (a, b)]
        tabs_all, _ = tables_gpu.evolve_background_tables_host(
            list(plist) + sets, nqmax, leader=tables_gpu.follow_nominal(nc, len(sets) // nc))
        h.update(tab0=tabs_all[:nc], tau0=_tables.tau_of_a_blob(tabs_all[:nc], aexp_out),
                 tabs=tabs_all[nc:], taus=_tables.tau_of_a_blob(tabs_all[nc:], aexp_out))
    elif not _gpu_tables(backgrounds):
        nominal = [b[0] for b in backgrounds]
        sets = [b[1:] for b in backgrounds]
        h.update(tab0=_tables.pack_batch(nominal, nqmax),
                 tau0=np.stack([_tables.tau_of_a(b, aexp_out) for b in nominal]),
                 tabs=_tables.pack_batch([q for st in sets for q in st], nqmax),
                 taus=np.stack([_tables.tau_of_a(q, aexp_out) for st in sets for q in st]))
    return h


def _gpu_tables(backgrounds):
    return isinstance(backgrounds, str) and backgrounds == "gpu"


def _native_tables(backgrounds):
    return isinstance(backgrounds, str) and backgrounds == "native"


def _device_tables(plist, pert, aexp_out, nqmax, out=None):
    """Tables and output times of the nominal and every theta +- eps set,
    produced on the GPU from the parameter dicts in one producer launch (its
    time is one set's latency, whatever the number of sets).  The sets are
    laid out nominal rows first, then the perturbed rows of cosmology c at
    c * nset + s, so tab0 and tabs are the two contiguous halves of one
    buffer.  ``out`` = (tables, tau) of an earlier call fills those buffers."""
    from . import tables_gpu

    sets = [q for pp in pert for (_, _, a, b) in pp for q in (a, b)]
    o = out or (None, None)
    nc = len(plist)
    tabs_all, tau_all, st = tables_gpu.evolve_background_tables(list(plist) + sets, nqmax, aexp_out=aexp_out,
                                                                out=o[0], tau_out=o[1],
                                                                leader=tables_gpu.follow_nominal(nc, len(sets) // nc))
    return dict(tables_all=tabs_all, tau_all=tau_all, tab0=tabs_all[:nc], tau0=tau_all[:nc], tabs=tabs_all[nc:],
                taus=tau_all[nc:]), st


def choose_method(method, nout, npar, lmax, linear_solver):
    """'adjoint' (one reverse sweep per output time and mode, ~3-5 forward
    steps of work each) or 'replay' (2 npar forward solves of the recorded
    steps): 'auto' takes the adjoint while nout seeds cost less than the
    2 npar replays, and when the hierarchy and solver allow it."""
    ok = linear_solver == "structured" and min(lmax) >= 5
    if method == "auto":
        return "adjoint" if ok and 4 * nout <= 2 * npar else "replay"
    if method not in ("adjoint", "replay"):
        raise ValueError(f"method must be 'auto', 'adjoint' or 'replay', not {method!r}")
    if method == "adjoint" and not ok:
        raise ValueError("the adjoint needs the structured solver and lmaxg, lmaxgp, lmaxr >= 5")
    return method


def seg_cap_for(max_steps, ck_cap):
    """Largest checkpoint stride a record with ck_cap slots can reach."""
    return max(1, -(-2 * int(max_steps) // int(ck_cap)))


# Checkpoint stride the adjoint plans allow (its segment buffer holds this many
# states per warp); every mode keeps at least 2 max_steps / SEG_CAP slots so that
# thinning stays within it, whatever its step count.
SEG_CAP = 64


def checkpoint_caps(nrec, max_steps, margin=1.25, extra=16):
    """Per-mode checkpoint slots fitted to recorded step counts: room for a
    state after every step with margin for other parameters of similar
    step counts (stride 1: the adjoint recomputes nothing), at least
    2 max_steps / SEG_CAP (a mode that outgrows its slots thins them, and
    its stride stays within the plan's segment buffer), even."""
    seg_floor = -(-2 * int(max_steps) // SEG_CAP)
    caps = np.maximum(np.ceil(np.asarray(nrec, dtype=np.float64) * margin).astype(np.int64) + extra, seg_floor)
    caps += caps & 1
    offs = np.concatenate([[0], np.cumsum(caps)[:-1]])
    return caps.astype(np.int32), offs.astype(np.int64), int(caps.sum()), seg_floor


_adj_plans: dict = {}


def adjoint_plan(dims, items, seg_cap):
    """Cached adjoint plan (deb_plan_create_adjoint) for >= items work items."""
    import torch

    key = (torch.cuda.current_device(), dims.lmaxg, dims.lmaxgp, dims.lmaxr, dims.lmaxnu, dims.nqmax, dims.nout,
           int(seg_cap))
    p = _adj_plans.get(key)
    if p is None or p.max_modes < items:
        _adj_plans.pop(key, None)
        p = _native.Plan(dims, max(int(items), 1), adjoint_seg_cap=int(seg_cap))
        _adj_plans[key] = p
    return p


class GradientProblem:
    """Device-resident inputs, buffers and plan of one gradient launch pair.

    ``backgrounds``: per cosmology the evolved ``param`` dicts
    [nominal, theta_1 + eps_1, theta_1 - eps_1, ...] (see
    :func:`perturbed_params`), or ``"native"`` / ``"gpu"``: the tables of all
    those sets are then produced from ``plist`` and ``pert`` by the
    library's table producer on the host cores or on the GPU
    (:mod:`tables_gpu`).  :meth:`run` enqueues the recorded nominal
    solve, the replay of every perturbed set, ``get_power`` and the
    difference quotients on one stream, without synchronising;
    :meth:`capture` records that sequence once as a CUDA graph and
    :meth:`replay` re-runs it; :meth:`load` copies the inputs of another
    problem of the same shape into the same device buffers (through pinned
    host memory), so one captured graph serves many calls.

    With ``method="adjoint"`` the record keeps checkpoints and :meth:`run`
    sweeps one adjoint per (output, mode) instead of the replay;
    :meth:`fit_checkpoints` lays the checkpoint slots out per mode.  Problems
    of one shape share the cached plans (their device workspaces and work
    queues): run them on one stream, or give each its own ``plan`` /
    ``adj_plan``.
    """

    def __init__(self, plist, backgrounds, pert, kmodes, aexp_out, *, lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax, rtol, atol,
                 pcoeff=0.25, icoeff=0.80, dcoeff=0.0, factormax=20.0, factormin=0.3, max_steps=2048, idx=4,
                 theta=THETA, step_to_outputs=False, launch=None, linear_solver="structured", method="auto",
                 ck_cap=32, jacobian=True):
        import torch

        self.theta = tuple(theta)
        self.nc = len(plist)
        self.kmodes = np.asarray(kmodes, dtype=np.float64)
        self.num_k = self.kmodes.shape[0]
        aexp_out = np.atleast_1d(np.asarray(aexp_out, dtype=np.float64))
        self.aexp_out = aexp_out
        self.nqmax = nqmax
        self.nout = aexp_out.shape[0]
        self.npar = len(pert[0])
        self.nset = 2 * self.npar
        self.idx = idx
        h = _host_inputs(plist, backgrounds, pert, self.kmodes, aexp_out, nqmax)
        self.host_k, self.host_com = h["k"], h["com"]
        self.nmode = self.host_k.shape[0]
        dev = torch.device("cuda", torch.cuda.current_device())
        self.device = dev
        # pinned staging copies of every per-call host input, and their device twins
        self.gpu_tables = _gpu_tables(backgrounds)
        self.table_source = backgrounds if isinstance(backgrounds, str) else "dicts"
        self._names = SMALL_NAMES + (() if self.gpu_tables else TABLE_NAMES)
        self._pinned = {n: torch.from_numpy(np.ascontiguousarray(h[n])).pin_memory() for n in self._names}
        self._dev = {n: self._pinned[n].to(dev) for n in self._names}
        if self.gpu_tables:
            dt, self._table_status = _device_tables(plist, pert, aexp_out, nqmax)
            self._dev.update(dt)
        self.blob_len = int(self._dev["tab0"].shape[1])
        self.d_tab0, self.d_tabs = self._dev["tab0"], self._dev["tabs"]
        self.d_k, self.d_com = self._dev["k"], self._dev["com"]
        self.d_tau0, self.d_taus = self._dev["tau0"], self._dev["taus"]
        self.eps_m = self._dev["eps"][:, :, None]     # [npar, nmode, 1]
        self.d_inv_As, self.d_lnk = self._dev["inv_As"], self._dev["lnk"]
        self.rec_len = int(max_steps) + 1
        nm, ns, no = self.nmode, self.nset, self.nout
        self.d_rec = torch.empty((nm, self.rec_len), dtype=torch.float64, device=dev)
        self.d_nrec = torch.empty((nm,), dtype=torch.int32, device=dev)
        self.d_y0 = torch.empty((nm, no, 20), dtype=torch.float64, device=dev)
        self.d_st0 = torch.empty((nm,), dtype=torch.int32, device=dev)
        self.d_steps = torch.empty((nm, 2), dtype=torch.int32, device=dev)
        self.method = choose_method(method, no, self.npar, (lmaxg, lmaxgp, lmaxr), linear_solver)
        if self.method == "replay":
            self.d_ys = torch.empty((ns * nm, no, 20), dtype=torch.float64, device=dev)
            self.d_sts = torch.empty((ns * nm,), dtype=torch.int32, device=dev)
        self.d_P = torch.empty((nm, no), dtype=torch.float64, device=dev)
        self.d_dl = torch.empty((nm, no, len(self.theta)), dtype=torch.float64, device=dev)
        self.ode_names = [n for (n, _, _, _) in pert[0]]
        self.dims = _pt._dims(lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax, no, False, linear_solver, "warp")
        self.plan = _pt.get_plan(self.dims, (ns if self.method == "replay" else 1) * nm, launch)
        self.cfg = _pt._cfg(rtol, atol, pcoeff, icoeff, dcoeff, factormax, factormin, max_steps,
                            step_to_outputs=step_to_outputs)
        self.order = torch.as_tensor(_pt.schedule_order(self.host_k)).to(dev, torch.int32)
        self.graph = None
        self._copied = None
        if self.method == "adjoint":
            n = _pt.nvar(lmaxg, lmaxgp, lmaxr, lmaxnu, nqmax)
            # uniform slots until fit_checkpoints() lays them out by step counts
            self.ck_cap = max(int(ck_cap), -(-2 * int(max_steps) // SEG_CAP))
            self.ck_cap += self.ck_cap & 1
            self.d_ckpt = torch.empty((nm, self.ck_cap, n), dtype=torch.float64, device=dev)
            self.d_ckoff = self.d_ckcap = None
            self.max_steps = int(max_steps)
            self.d_ckstride = torch.empty((nm,), dtype=torch.int32, device=dev)
            # the Jacobian takes one cotangent seed per output time (seed o is
            # d ln P(k, a_o) / d y); a vector-Jacobian product takes one
            self.nseed = no if jacobian else 1
            nsd = self.nseed
            self.d_gy = torch.zeros((nsd, nm, no, 20), dtype=torch.float64, device=dev)
            self.d_gth = torch.empty((nsd, nm, self.npar), dtype=torch.float64, device=dev)
            self.d_ast = torch.empty((nsd * nm,), dtype=torch.int32, device=dev)
            self.eps_c = self._dev["eps_c"]     # [ncosmo, npar], reloaded by load()
            self.adj_plan = adjoint_plan(self.dims, nsd * nm, SEG_CAP)

    def load(self, plist, backgrounds, pert, stream=None):
        """Copy the inputs of another set of cosmologies of the same shape
        (same count, k-grid, output times count, table lengths) into this
        problem's device buffers: host packing, then one pinned host-to-device
        copy per input array on ``stream``; with GPU tables the producer
        writes the new tables into the same buffers.  Returns the bytes
        copied from the host."""
        import torch

        if (backgrounds if isinstance(backgrounds, str) else "dicts") != self.table_source:
            raise ValueError(f"load: the problem was built with {self.table_source} tables")
        h = _host_inputs(plist, backgrounds, pert, self.kmodes, self.aexp_out, self.nqmax)
        s = stream if stream is not None else torch.cuda.current_stream()
        if self._copied is not None:
            self._copied.synchronize()   # the previous load's copies have left the pinned buffers
        nbytes = 0
        with torch.cuda.stream(s):
            for n in self._names:
                a = np.ascontiguousarray(h[n])
                if a.shape != tuple(self._pinned[n].shape):
                    raise ValueError(f"load: input {n} has shape {a.shape}, the problem was built for "
                                     f"{tuple(self._pinned[n].shape)}")
                self._pinned[n].numpy()[...] = a
                self._dev[n].copy_(self._pinned[n], non_blocking=True)
                nbytes += a.nbytes
            self._copied = torch.cuda.Event()
            self._copied.record(s)
            if self.gpu_tables:
                from . import tables_gpu

                _, self._table_status = _device_tables(plist, pert, self.aexp_out, self.nqmax,
                                                       out=(self._dev["tables_all"], self._dev["tau_all"]))
                nbytes += tables_gpu.param_matrix(plist).nbytes * (1 + self.nset)
        return nbytes

    def input_bytes(self) -> int:
        """Host bytes one call copies to the device: the packed tables and
        small per-mode arrays, or with GPU tables the parameter rows of
        every set plus the small arrays."""
        from . import tables_gpu

        n = sum(int(self._pinned[k].numel() * self._pinned[k].element_size()) for k in self._names)
        if self.gpu_tables:
            n += self.nc * (1 + self.nset) * len(tables_gpu.PARAM_KEYS) * 8
        return n

    def _record(self, plan, s):
        L = _native.load()
        c = lambda t: ctypes.c_void_p(t.data_ptr())
        co = lambda t: None if t is None else ctypes.c_void_p(t.data_ptr())
        if self.method == "adjoint":
            _native.check(_pt.launch_ordered(plan, self.order, self.nmode, lambda: L.deb_forward_record_ckpt(
                plan.ptr, c(self.d_tab0), self.nc, self.blob_len, c(self.d_k), c(self.d_com), self.nmode,
                c(self.d_tau0), ctypes.byref(self.cfg), c(self.d_y0), c(self.d_st0), c(self.d_steps), c(self.d_rec),
                self.rec_len, c(self.d_nrec), c(self.d_ckpt), self.ck_cap, co(self.d_ckoff), co(self.d_ckcap),
                c(self.d_ckstride), ctypes.c_void_p(s.cuda_stream))), "deb_forward_record_ckpt")
            return
        _native.check(_pt.launch_ordered(plan, self.order, self.nmode, lambda: L.deb_forward_record(
            plan.ptr, c(self.d_tab0), self.nc, self.blob_len, c(self.d_k), c(self.d_com), self.nmode,
            c(self.d_tau0), ctypes.byref(self.cfg), c(self.d_y0), c(self.d_st0), c(self.d_steps), c(self.d_rec),
            self.rec_len, c(self.d_nrec), ctypes.c_void_p(s.cuda_stream))), "deb_forward_record")

    def _adjoint(self, s, nseed):
        """deb_adjoint of the first nseed cotangent seeds in d_gy on stream s."""
        L = _native.load()
        c = lambda t: ctypes.c_void_p(t.data_ptr())
        _native.check(L.deb_adjoint(self.adj_plan.ptr, c(self.d_tab0), c(self.d_tabs), self.nc, self.npar,
                                    self.blob_len, c(self.eps_c), c(self.d_k), c(self.d_com), self.nmode,
                                    c(self.d_tau0), c(self.d_taus), c(self.d_rec), self.rec_len, c(self.d_nrec),
                                    c(self.d_ckpt), self.ck_cap,
                                    None if self.d_ckoff is None else c(self.d_ckoff), c(self.d_ckstride),
                                    c(self.d_gy), int(nseed),
                                    c(self.d_gth), c(self.d_ast), ctypes.c_void_p(s.cuda_stream)), "deb_adjoint")

    def fit_checkpoints(self, margin=1.25):
        """Lay the checkpoint slots out per mode from the last record's step
        counts (checkpoint_caps): afterwards every mode whose step count grows
        by less than the margin keeps a state after every step, and the
        adjoint recomputes no segment.  Synchronises; call it between runs,
        before a graph capture.  Returns the pool's bytes."""
        import torch

        if self.method != "adjoint":
            return 0
        if self.graph is not None or getattr(self, "_in_graph", False):
            raise RuntimeError("fit_checkpoints: a captured graph holds the current checkpoint buffers; "
                               "fit before capturing")
        torch.cuda.synchronize()
        nrec = self.d_nrec.cpu().numpy()
        caps, offs, total, _ = checkpoint_caps(nrec, self.max_steps, margin)
        n = self.d_ckpt.shape[-1]
        self.d_ckpt = None
        self.d_ckpt = torch.empty((total, n), dtype=torch.float64, device=self.device)
        self.d_ckcap = torch.as_tensor(caps).to(self.device)
        self.d_ckoff = torch.as_tensor(offs).to(self.device)
        return self.d_ckpt.numel() * 8

    def forward(self, stream=None):
        """The recorded nominal solve (with checkpoints when the method is the
        adjoint) and get_power, without gradients; returns P [nmode, nout]."""
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        self._record(self.plan, s)
        L = _native.load()
        c = lambda t: ctypes.c_void_p(t.data_ptr())
        _native.check(L.deb_get_power(c(self.d_tab0), self.nc, self.blob_len, c(self.d_k), c(self.d_com),
                                      self.nmode, self.nout, c(self.d_y0), 20, self.idx, c(self.d_P),
                                      ctypes.c_void_p(s.cuda_stream)), "deb_get_power")
        return self.d_P

    def vjp(self, gP, stream=None):
        """Gradient of sum_{k,a} gP P(k, a) over theta, per cosmology
        [ncosmo, len(theta)], by one adjoint sweep per mode (after
        :meth:`forward`; adjoint method only)."""
        import torch

        if self.method != "adjoint":
            raise RuntimeError("vjp needs a problem built with method='adjoint'")
        s = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            gP = gP.to(self.device, torch.float64).reshape(self.nmode, self.nout)
            w = gP * self.d_P
            self.d_gy[0].zero_()
            self.d_gy[0, :, :, self.idx] = 2.0 * w / self.d_y0[:, :, self.idx]
        self._adjoint(s, 1)
        with torch.cuda.stream(s):
            if getattr(self, "d_gvjp", None) is None:
                self.d_gvjp = torch.zeros((self.nc, len(self.theta)), dtype=torch.float64, device=self.device)
                self.d_com_l = self.d_com.long()
            g = self.d_gvjp
            g.zero_()
            for j, name in enumerate(self.theta):
                if name == "A_s":
                    v = (w * self.d_inv_As).sum(dim=1)
                elif name == "n_s":
                    v = (w * self.d_lnk).sum(dim=1)
                else:
                    v = self.d_gth[0, :, self.ode_names.index(name)]
                g[:, j].index_add_(0, self.d_com_l, v)
        return g

    def tune(self, candidates=None):
        """Choose the launch shape by timing the nominal recorded solve with
        each candidate (:mod:`autotune`); the replay uses the same kernel.
        Returns {shape: ms}."""
        from . import autotune

        best, times = autotune.tune(self.dims, self.nset * self.nmode, self._record,
                                    candidates or autotune.CANDIDATES)
        self.plan = _pt.get_plan(self.dims, self.nset * self.nmode, best)
        self.graph = None
        return times

    def run(self, stream=None, events=None):
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        L = _native.load()
        c = lambda t: ctypes.c_void_p(t.data_ptr())
        sp = ctypes.c_void_p(s.cuda_stream)
        if events:
            events[0].record(s)
        self._record(self.plan, s)
        if events:
            events[1].record(s)
        if self.method == "adjoint":
            if self.nseed != self.nout:
                raise RuntimeError("this problem was built for vector-Jacobian products (jacobian=False)")
            with torch.cuda.stream(s):
                # seed o: d ln P(k, a_o) / d y = 2 / y_idx at output o
                for o in range(self.nout):
                    self.d_gy[o, :, o, self.idx] = 2.0 / self.d_y0[:, o, self.idx]
            self._adjoint(s, self.nseed)
            if events:
                events[2].record(s)
            with torch.cuda.stream(s):
                dl_ode = self.d_gth.permute(2, 1, 0)        # [npar, nmode, nout]
        else:
            _native.check(L.deb_replay(self.plan.ptr, c(self.d_tabs), self.nc, self.nset, self.blob_len,
                                       c(self.d_k), c(self.d_com), self.nmode, c(self.d_taus), ctypes.byref(self.cfg),
                                       c(self.d_rec), self.rec_len, c(self.d_nrec), c(self.d_ys), c(self.d_sts), sp),
                          "deb_replay")
            if events:
                events[2].record(s)
            with torch.cuda.stream(s):
                ys = self.d_ys[..., self.idx].reshape(self.nset, self.nmode, self.nout)
                lp = torch.log(ys * ys)
                dl_ode = (lp[0::2] - lp[1::2]) / (2.0 * self.eps_m)
        with torch.cuda.stream(s):
            for j, name in enumerate(self.theta):
                if name == "A_s":
                    self.d_dl[:, :, j] = self.d_inv_As
                elif name == "n_s":
                    self.d_dl[:, :, j] = self.d_lnk
                else:
                    self.d_dl[:, :, j] = dl_ode[self.ode_names.index(name)]
        _native.check(L.deb_get_power(c(self.d_tab0), self.nc, self.blob_len, c(self.d_k), c(self.d_com),
                                      self.nmode, self.nout, c(self.d_y0), 20, self.idx, c(self.d_P), sp),
                      "deb_get_power")
        return self.d_P, self.d_dl

    def capture(self):
        """Capture :meth:`run` (record launch, replay launch, get_power and
        the difference quotients) as one CUDA graph.  Runs it once eagerly
        first; synchronises."""
        import torch

        self.run()
        torch.cuda.synchronize()
        if self.method == "adjoint" and self.d_ckoff is None:
            self.fit_checkpoints()
            self.run()
            torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run(torch.cuda.current_stream())
        self.graph = g
        return g

    def replay(self, stream=None):
        """Re-run the captured graph on ``stream`` (default: current)."""
        import torch

        if self.graph is None:
            self.capture()
        s = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            self.graph.replay()
        return self.d_P, self.d_dl

    def check(self):
        st0 = self.d_st0.cpu().numpy()
        sts = (self.d_ast if self.method == "adjoint" else self.d_sts).cpu().numpy()
        if (st0 != 0).any() or (sts != 0).any():
            raise RuntimeError(f"{int((st0 != 0).sum())} nominal / {int((sts != 0).sum())} replayed mode(s) failed")


_problems: dict = {}
_MAX_CACHED = 2


def _run_cached(plist, backgrounds, pert, kmodes, aexp_out, opts):
    """Run one gradient problem, reusing device buffers and the captured CUDA
    graph of an earlier call of the same shape: the first call of a shape
    runs eagerly, the second captures the graph (its eager run gives the
    results), later calls copy their inputs in and replay the graph."""
    import torch

    aexp = np.atleast_1d(np.asarray(aexp_out, dtype=np.float64))
    key = (torch.cuda.current_device(), len(plist), np.asarray(kmodes, dtype=np.float64).tobytes(), aexp.shape[0],
           tuple(sorted(opts.items())), tuple(n for (n, _, _, _) in pert[0]),
           backgrounds if isinstance(backgrounds, str) else "dicts")
    gp = _problems.get(key)
    if gp is not None:
        try:
            gp.load(plist, backgrounds, pert)
        except ValueError:      # table lengths differ: not the same shape after all
            gp = None
            _problems.pop(key, None)
    if gp is None:
        gp = GradientProblem(plist, backgrounds, pert, kmodes, aexp_out, **opts)
        gp.calls = 0
        while len(_problems) >= _MAX_CACHED:
            _problems.pop(next(iter(_problems)))
        _problems[key] = gp
    gp.calls += 1
    if gp.calls == 1:
        Pd, Dd = gp.run()
    elif gp.graph is None:
        gp.capture()
        Pd, Dd = gp.d_P, gp.d_dl
    else:
        Pd, Dd = gp.replay()
    return Pd, Dd, gp


def _problem_inputs(plist, *, kmin, kmax, num_k, dologk, theta, rel_step, tables, backgrounds, processes, opts):
    """k-grid, theta +- eps parameter sets and their tables' source for a
    gradient problem of the cosmologies ``plist``."""
    kmodes = np.geomspace(kmin, kmax, num_k) if dologk else np.linspace(kmin, kmax, num_k)
    pert = [perturbed_params(p, theta, rel_step) for p in plist]
    nset = 2 * len(pert[0])
    if tables not in ("native", "gpu", "python"):
        raise ValueError(f"tables must be 'native', 'gpu' or 'python', not {tables!r}")
    if backgrounds is None and tables in ("native", "gpu"):
        backgrounds = tables
    elif backgrounds is None:
        flat = []
        for p, pp in zip(plist, pert):
            flat.append(p)
            for (_, _, a, b) in pp:
                flat += [a, b]
        ev = evolve_backgrounds(flat, processes)
        backgrounds = [ev[i * (nset + 1):(i + 1) * (nset + 1)] for i in range(len(plist))]
    return kmodes, pert, backgrounds, opts


def evolve_perturbations_grad(*, params, aexp_out, kmin: float, kmax: float, num_k: int, lmaxg: int = 11,
                              lmaxgp: int = 11, lmaxr: int = 11, lmaxnu: int = 8, nqmax: int = 3, rtol: float = 1e-4,
                              atol: float = 1e-4, pcoeff: float = 0.25, icoeff: float = 0.80, dcoeff: float = 0.0,
                              factormax: float = 20.0, factormin: float = 0.3, max_steps: int = 2048, idx: int = 4,
                              theta=THETA, rel_step: float = 1e-4, dologk: bool = True, processes=None,
                              backgrounds=None, throw: bool = True, step_to_outputs: bool = False,
                              tables: str = "native", method: str = "auto"):
    """P(k, a) and d log P / d theta for one or many cosmologies.

    ``params``: input parameter dict(s) as given to ``evolve_background``
    (Omegam, Omegab, H0, mnu, w_DE_0, w_DE_a, A_s, n_s, ...).  Returns
    ``(P [ncosmo, num_k, nout], dlogP [ncosmo, num_k, nout, len(theta)],
    kmodes)``; with a single dict the cosmology axis is dropped.
    ``backgrounds`` may pass precomputed host tables: a list (per cosmology)
    of [nominal, +eps_1, -eps_1, +eps_2, ...] evolved ``param`` dicts.
    Without them the tables of all those sets come from the library's
    producer on the host cores (``tables="native"``, C++ threads, a few ms
    per set; the default), on the GPU in one launch (``tables="gpu"``), or
    from the Python producer in a process pool (``tables="python"``).
    With the reference's output semantics (linear interpolation inside the
    step) an interior output's derivative includes the slope of that
    interpolant; ``step_to_outputs=True`` lands steps on the output times.
    """
    single = isinstance(params, dict)
    plist = [params] if single else list(params)
    nc = len(plist)
    kmodes, pert, backgrounds, opts = _problem_inputs(
        plist, kmin=kmin, kmax=kmax, num_k=num_k, dologk=dologk, theta=theta, rel_step=rel_step, tables=tables,
        backgrounds=backgrounds, processes=processes,
        opts=dict(lmaxg=lmaxg, lmaxgp=lmaxgp, lmaxr=lmaxr, lmaxnu=lmaxnu, nqmax=nqmax, rtol=rtol, atol=atol,
                  pcoeff=pcoeff, icoeff=icoeff, dcoeff=dcoeff, factormax=factormax, factormin=factormin,
                  max_steps=max_steps, idx=idx, theta=tuple(theta), step_to_outputs=step_to_outputs, method=method))
    Pd, Dd, gp = _run_cached(plist, backgrounds, pert, kmodes, aexp_out, opts)
    if throw:
        gp.check()
    nout = gp.nout
    P = Pd.reshape(nc, num_k, nout).cpu().numpy()
    D = Dd.reshape(nc, num_k, nout, len(theta)).cpu().numpy()
    return (P[0], D[0], kmodes) if single else (P, D, kmodes)


class LoglikeProblem:
    """Device-resident Gaussian log-likelihood of P(k, a) and its gradient.

    ln L_c = -1/2 sum_{k,a} w_{k,a} (ln P_c(k, a) - lnP_data_c(k, a))^2 for
    every cosmology c, and d ln L_c / d theta by one adjoint sweep per mode
    (:meth:`GradientProblem.vjp`): the cotangent of P is
    -w (ln P - lnP_data) / P.  :meth:`run` enqueues the recorded solve with
    checkpoints, get_power, the likelihood and the adjoint on one stream;
    :meth:`capture` / :meth:`replay` as for :class:`GradientProblem`;
    :meth:`load` copies another call's tables and data into the same buffers.
    """

    def __init__(self, plist, backgrounds, pert, kmodes, aexp_out, lnP_data, weights, **opts):
        import torch

        opts = dict(opts)
        opts["method"] = "adjoint"
        opts["jacobian"] = False
        self.gp = GradientProblem(plist, backgrounds, pert, kmodes, aexp_out, **opts)
        gp = self.gp
        dev = gp.device
        self.shape = (gp.nc, gp.num_k, gp.nout)
        self._pdata = torch.zeros(self.shape, dtype=torch.float64).pin_memory()
        self.d_data = torch.empty((gp.nmode, gp.nout), dtype=torch.float64, device=dev)
        w = np.broadcast_to(np.asarray(weights, dtype=np.float64), (gp.num_k, gp.nout))
        self.d_w = torch.as_tensor(np.tile(w, (gp.nc, 1))).to(dev)
        self.d_lnL = torch.zeros((gp.nc,), dtype=torch.float64, device=dev)
        self.set_data(lnP_data)
        self.graph = None
        self.calls = 0

    def set_data(self, lnP_data, stream=None):
        import torch

        self._pdata.numpy()[...] = np.asarray(lnP_data, dtype=np.float64).reshape(self.shape)
        s = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            self.d_data.copy_(self._pdata.reshape(self.d_data.shape), non_blocking=True)
        return self._pdata.numel() * 8

    def run(self, stream=None):
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        return self.backward(self.gp.forward(s), s)

    def backward(self, P, stream=None):
        """The likelihood of the P a :meth:`GradientProblem.forward` left and
        its gradient by the adjoint sweep; returns (P, ln L, gradient)."""
        import torch

        gp = self.gp
        s = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            r = torch.log(P) - self.d_data
            gP = -self.d_w * r / P
            self.d_lnL.zero_()
            if getattr(self, "_com", None) is None:
                self._com = gp.d_com.long()
            self.d_lnL.index_add_(0, self._com, (-0.5 * self.d_w * r * r).sum(dim=1))
        g = gp.vjp(gP, s)
        return P, self.d_lnL, g

    def capture(self):
        import torch

        self.run()
        torch.cuda.synchronize()
        if self.gp.d_ckoff is None:
            self.gp.fit_checkpoints()
            self.run()
            torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.out = self.run(torch.cuda.current_stream())
        self.gp._in_graph = True
        self.graph = g
        return g

    def replay(self, stream=None):
        import torch

        if self.graph is None:
            self.capture()
        s = stream if stream is not None else torch.cuda.current_stream()
        with torch.cuda.stream(s):
            self.graph.replay()
        return self.out

    def load(self, plist, backgrounds, pert, lnP_data, stream=None):
        return self.gp.load(plist, backgrounds, pert, stream) + self.set_data(lnP_data, stream)

    def check(self):
        st0 = self.gp.d_st0.cpu().numpy()
        ast = self.gp.d_ast[:self.gp.nmode].cpu().numpy()
        if (st0 != 0).any() or (ast != 0).any():
            raise RuntimeError(f"{int((st0 != 0).sum())} forward / {int((ast != 0).sum())} adjoint mode(s) failed")


_ll_problems: dict = {}


def loglike_grad(*, params, lnP_data, weights, aexp_out, kmin: float, kmax: float, num_k: int, lmaxg: int = 11,
                 lmaxgp: int = 11, lmaxr: int = 11, lmaxnu: int = 8, nqmax: int = 3, rtol: float = 1e-4,
                 atol: float = 1e-4, pcoeff: float = 0.25, icoeff: float = 0.80, dcoeff: float = 0.0,
                 factormax: float = 20.0, factormin: float = 0.3, max_steps: int = 2048, idx: int = 4, theta=THETA,
                 rel_step: float = 1e-4, dologk: bool = True, processes=None, backgrounds=None, throw: bool = True,
                 step_to_outputs: bool = False, tables: str = "native", ck_cap: int = 32):
    """Gaussian log-likelihood of P(k, a) and its gradient over theta.

    ln L = -1/2 sum_{k,a} weights (ln P(k, a) - lnP_data)^2 per cosmology,
    with ``lnP_data`` [ncosmo, num_k, nout] (or [num_k, nout] for a single
    dict) and ``weights`` broadcastable to [num_k, nout] (e.g. N_k / 2, the
    inverse variance of ln P of a diagonal Gaussian covariance).  The gradient
    is one discrete-adjoint sweep per mode (``deb_adjoint``): its cost does
    not grow with the number of parameters or output times.  Returns
    ``(P [ncosmo, num_k, nout], lnL [ncosmo], grad [ncosmo, len(theta)],
    kmodes)``, the cosmology axis dropped for a single dict.  Repeated calls
    of the same shape replay a captured CUDA graph with the new inputs.
    """
    import torch

    single = isinstance(params, dict)
    plist = [params] if single else list(params)
    nc = len(plist)
    opts = dict(lmaxg=lmaxg, lmaxgp=lmaxgp, lmaxr=lmaxr, lmaxnu=lmaxnu, nqmax=nqmax, rtol=rtol, atol=atol,
                pcoeff=pcoeff, icoeff=icoeff, dcoeff=dcoeff, factormax=factormax, factormin=factormin,
                max_steps=max_steps, idx=idx, theta=tuple(theta), step_to_outputs=step_to_outputs, ck_cap=ck_cap)
    kmodes, pert, backgrounds, _ = _problem_inputs(plist, kmin=kmin, kmax=kmax, num_k=num_k, dologk=dologk,
                                                   theta=theta, rel_step=rel_step, tables=tables,
                                                   backgrounds=backgrounds, processes=processes, opts=None)
    aexp = np.atleast_1d(np.asarray(aexp_out, dtype=np.float64))
    data = np.asarray(lnP_data, dtype=np.float64).reshape(nc, num_k, aexp.shape[0])
    key = (torch.cuda.current_device(), nc, kmodes.tobytes(), aexp.tobytes(), tuple(sorted(opts.items())),
           np.asarray(weights, dtype=np.float64).tobytes(), backgrounds if isinstance(backgrounds, str) else "dicts")
    lp = _ll_problems.get(key)
    if lp is not None:
        try:
            lp.load(plist, backgrounds, pert, data)
        except ValueError:
            lp = None
            _ll_problems.pop(key, None)
    if lp is None:
        lp = LoglikeProblem(plist, backgrounds, pert, kmodes, aexp, data, weights, **opts)
        while len(_ll_problems) >= _MAX_CACHED:
            _ll_problems.pop(next(iter(_ll_problems)))
        _ll_problems[key] = lp
    lp.calls += 1
    if lp.calls == 1:
        P, lnL, g = lp.run()
    elif lp.graph is None:
        lp.capture()
        P, lnL, g = lp.out
    else:
        P, lnL, g = lp.replay()
    if throw:
        lp.check()
    P = P.reshape(nc, num_k, -1).cpu().numpy()
    lnL, g = lnL.cpu().numpy(), g.cpu().numpy()
    return (P[0], lnL[0], g[0], kmodes) if single else (P, lnL, g, kmodes)


def fisher_matrix(kmodes, dlogP, volume_mpc3: float):
    """F_ij = sum_{k,a} d_i lnP d_j lnP / sigma^2_lnP with sigma^2_lnP = 2 / N_k,
    N_k = V k^2 dk / (2 pi^2) (diagonal Gaussian covariance, one volume V per
    output time).  dlogP [num_k, nout, ntheta] -> [ntheta, ntheta]."""
    import torch

    k = np.asarray(kmodes, dtype=np.float64)
    edges = np.sqrt(k[1:] * k[:-1])
    dk = np.empty_like(k)
    dk[1:-1] = edges[1:] - edges[:-1]
    dk[0] = edges[0] - k[0] ** 2 / edges[0]
    dk[-1] = k[-1] ** 2 / edges[-1] - edges[-1]
    nk = volume_mpc3 * k**2 * dk / (2.0 * np.pi**2)
    w = torch.as_tensor(nk / 2.0, dtype=torch.float64, device="cuda")
    d = torch.as_tensor(np.asarray(dlogP, dtype=np.float64), device="cuda")
    F = torch.einsum("k,kai,kaj->ij", w, d, d)
    return F.cpu().numpy()


def _torch():
    import torch

    return torch


class PowerSpectrum:
    """``torch.autograd.Function`` from theta to P(k, a) for one cosmology.

    ``PowerSpectrum.apply(theta, base_params, options)`` with ``theta`` a
    float64 tensor [8] in the order of :data:`THETA` (h, not H0), overriding
    those entries of ``base_params``; ``options`` is a dict of the keyword
    arguments of :func:`evolve_perturbations_grad` (aexp_out, kmin, kmax,
    num_k, hierarchy sizes, tolerances, tables, ...).  Forward runs the
    recorded solve with checkpoints and returns P [num_k, nout] on theta's
    device; backward is one discrete-adjoint sweep per mode
    (``deb_adjoint``) with the cotangent grad_P, plus the analytic A_s and n_s
    terms (``perturbations.py:1123``) -- a vector-Jacobian product whose cost
    does not grow with the number of parameters or outputs.  Needs the
    structured solver and lmaxg, lmaxgp, lmaxr >= 5.
    """

    _fn = None

    @classmethod
    def apply(cls, theta, base_params, options):
        if cls._fn is None:
            torch = _torch()

            class _Fn(torch.autograd.Function):
                @staticmethod
                def forward(ctx, th, base, opts):
                    vals = th.detach().cpu().numpy().astype(np.float64)
                    if vals.shape != (len(THETA),):
                        raise ValueError(f"theta must have {len(THETA)} entries in the order {THETA}")
                    params = dict(base)
                    for name, v in zip(THETA, vals):
                        params = _with(params, name, float(v))
                    o = dict(opts)
                    pkw = {k: o.pop(k) for k in ("kmin", "kmax", "num_k") if k in o}
                    aexp_out = o.pop("aexp_out")
                    throw = o.pop("throw", True)
                    kmodes, pert, backgrounds, _ = _problem_inputs(
                        [params], kmin=pkw["kmin"], kmax=pkw["kmax"], num_k=pkw["num_k"],
                        dologk=o.pop("dologk", True), theta=THETA, rel_step=o.pop("rel_step", 1e-4),
                        tables=o.pop("tables", "native"), backgrounds=o.pop("backgrounds", None),
                        processes=o.pop("processes", None), opts=None)
                    o.pop("method", None)
                    gp = GradientProblem([params], backgrounds, pert, kmodes, aexp_out, theta=THETA,
                                         method="adjoint", jacobian=False, **o)
                    P = gp.forward()
                    if throw:
                        st0 = gp.d_st0.cpu().numpy()
                        if (st0 != 0).any():
                            raise RuntimeError(f"{int((st0 != 0).sum())} mode(s) failed")
                    ctx.gp = gp
                    ctx.dev = th.device
                    return P.detach().clone().to(th.device)

                @staticmethod
                def backward(ctx, gP):
                    g = ctx.gp.vjp(gP)
                    if (ctx.gp.d_ast[:ctx.gp.nmode] != 0).any():
                        raise RuntimeError("adjoint sweep failed for some modes")
                    return g[0].to(ctx.dev), None, None

            cls._fn = _Fn
        return cls._fn.apply(theta, base_params, options)
