"""Benchmark of the perturbation hot path on GB300.

Default workload ``large_4cosmo_1024k_n1098_64a_rtol1e-6_loglike`` (the
large batched adjoint configuration's per-cosmology work): 4 cosmologies
drawn uniformly over Omegam [.25,.35], Omegab [.04,.055], h [.6,.75],
n_s [.92,1], ln(1e10 A_s) [2.9,3.2], m_nu [.06,.3] eV, w0 [-1.2,-.8],
wa [-.3,.3] (w(a) = -1 crossings redrawn), each with 1024 log-spaced k in
[1e-5, 50] /Mpc, lmax 32 in every hierarchy and 30 momentum bins (nvar
1098), rtol = atol = 1e-6, 64 output times uniform in a over [0.2, 1] with
steps landing on them (diffrax step_ts; interpolated inside steps, P(k) at
this tolerance is off by up to 2 % at the lowest k).  A
"step" is, for every cosmology, P(k, a) at all 1024 x 64 points, the
Gaussian log-likelihood of a synthetic data vector (the cosmology's own
ln P with 5% seeded scatter, diagonal covariance 2 / N_k) and its gradient
over theta = (Omegam, Omegab, h, n_s, A_s, m_nu, w0, wa): one recorded solve
with checkpoints (4096 modes) and one discrete-adjoint sweep per mode,
captured as one CUDA graph.  ``value`` is cosmologies (P(k, a) plus the
8-parameter gradient) per second with the inputs resident on the device;
``e2e`` is the same through the public call ``loglike_grad`` from the
parameters (tables of all 13 parameter sets produced on the host cores inside
the call, data vector copied in, P, ln L and the gradient copied out).

Other workloads (``--workload``): the 8-output Jacobian of the fiducial
cosmology at nvar 323 (``fiducial_1cosmo_128k_8a_n323_rtol1e-5_grad``), 8
sampled cosmologies x 512 k at nvar 323 with the gradient
(``batched_8cosmo_512k_n323_rtol1e-5_grad``), 64 cosmologies x 512 k forward
only (``batched_64cosmo_512k_n323_rtol1e-5``), and smaller cases.

CPU figures, measured on the same sample of modes (every 64th mode of
cosmology 0's k-grid): the oracle (``oracle/``, the reference algorithm:
Rodas5 + PID + dense forward-mode Jacobian + dense LU, FP64, OpenMP over
modes) timed over a bounded number of steps per mode and scaled by the
workload's steps per cosmology solve; and the structured solver's host build
(the kernel's own code compiled for the CPU, threads over modes) run to
completion.  ``--impl reference`` prints the oracle's figure as the
reference arm: the reference's own JAX code is not installable here.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

_N323 = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=17, nqmax=15)
_N1098 = dict(lmaxg=32, lmaxgp=32, lmaxr=32, lmaxnu=32, nqmax=30)
_N80 = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=8, nqmax=3)
# cosmo: "sample" (seeded draws over the batched ranges), "fiducial" (LCDM + 0.06 eV nu + w0 -0.9, wa 0.1)
# or "lcdm" (flat LCDM, massless nu); names ending in _grad add the 8-parameter gradient; step_ts lands
# steps on every output time (diffrax PIDController(step_ts=...)), so interior outputs and their
# derivatives are step ends rather than in-step interpolants
WORKLOADS = {
    # the large batched adjoint configuration's per-cosmology work; objective "loglike": P(k, a) and the
    # gradient of a Gaussian log-likelihood by one adjoint sweep per mode
    # (steps land on the 64 outputs: with the reference's in-step linear interpolation, P(k) at rtol 1e-6
    # is off by up to 2 % at the lowest k against a tight solve; landing on them, by 2e-6)
    "large_4cosmo_1024k_n1098_64a_rtol1e-6_loglike": dict(
        cosmo="sample", ncosmo=4, num_k=1024, kmin=1e-5, kmax=50.0, dims=_N1098, rtol=1e-6, atol=1e-6,
        aexp=[float(a) for a in np.linspace(0.2, 1.0, 64)], objective="loglike", max_steps=8192, ck_cap=1024,
        step_ts=True),
    # profiling case of the same kernels: one cosmology, 128 k over the same range
    "large_1cosmo_128k_n1098_64a_rtol1e-6_loglike": dict(
        cosmo="sample", ncosmo=1, num_k=128, kmin=1e-5, kmax=50.0, dims=_N1098, rtol=1e-6, atol=1e-6,
        aexp=[float(a) for a in np.linspace(0.2, 1.0, 64)], objective="loglike", max_steps=8192, ck_cap=1024,
        step_ts=True),
    # counter-capture case of the same kernels: 1216 modes (every SM's 8 slots) at the lowest k, whose short
    # step sequences keep one adjoint launch near a second
    "profile_1cosmo_1216k_n1098_8a_rtol1e-6_loglike": dict(
        cosmo="sample", ncosmo=1, num_k=1216, kmin=1e-5, kmax=1e-4, dims=_N1098, rtol=1e-6, atol=1e-6,
        aexp=[float(a) for a in np.linspace(0.2, 1.0, 8)], objective="loglike", max_steps=2048, ck_cap=32),
    "batched_8cosmo_512k_n323_rtol1e-5_grad": dict(cosmo="sample", ncosmo=8, num_k=512, kmin=1e-4, kmax=10.0,
                                                   dims=_N323, rtol=1e-5, atol=1e-5, aexp=[1.0]),
    "fiducial_1cosmo_128k_8a_n323_rtol1e-5_grad": dict(cosmo="fiducial", ncosmo=1, num_k=128, kmin=1e-3, kmax=1.0,
                                                       dims=_N323, rtol=1e-5, atol=1e-5, step_ts=True,
                                                       aexp=[float(a) for a in np.linspace(0.2, 1.0, 8)]),
    "batched_64cosmo_512k_n323_rtol1e-5": dict(cosmo="sample", ncosmo=64, num_k=512, kmin=1e-4, kmax=10.0, dims=_N323,
                                               rtol=1e-5, atol=1e-5, aexp=[1.0]),
    "batched_8cosmo_512k_n323_rtol1e-5": dict(cosmo="sample", ncosmo=8, num_k=512, kmin=1e-4, kmax=10.0, dims=_N323,
                                              rtol=1e-5, atol=1e-5, aexp=[1.0]),
    "fiducial_1cosmo_256k_n323_rtol1e-5": dict(cosmo="fiducial", ncosmo=1, num_k=256, kmin=1e-4, kmax=10.0,
                                               dims=_N323, rtol=1e-5, atol=1e-5, aexp=[1.0]),
    "lcdm_1cosmo_64k_n80_rtol1e-3": dict(cosmo="lcdm", ncosmo=1, num_k=64, kmin=1e-4, kmax=1.0, dims=_N80, rtol=1e-3,
                                         atol=1e-6, aexp=[1.0]),
    "single_1cosmo_256k_n323_rtol1e-5": dict(cosmo="sample", ncosmo=1, num_k=256, kmin=1e-4, kmax=10.0, dims=_N323,
                                             rtol=1e-5, atol=1e-5, aexp=[1.0]),
    # profiling case: enough modes to fill every SM's slots, short enough for a counter capture
    "batched_2cosmo_512k_n323_rtol1e-5": dict(cosmo="sample", ncosmo=2, num_k=512, kmin=1e-4, kmax=10.0, dims=_N323,
                                              rtol=1e-5, atol=1e-5, aexp=[1.0]),
}
DEFAULT_WORKLOAD = "large_4cosmo_1024k_n1098_64a_rtol1e-6_loglike"
# the metric named by the project's benchmark contract; this build's solves are FP64 throughout (there is no
# mixed-precision form: the structured O(n) solve leaves no factorisation to run in lower precision), and
# the "plain FP64" comparison is the dense-LU form measured beside it (plain_fp64)
METRIC = "P(k)+dP/d\u03b8 solves/s on 1 GB300, batched mixed vs plain FP64, at \u22641e-4 rel error"
VOLUME_MPC3 = 1e9   # survey volume of the likelihood's diagonal covariance (N_k modes per k-bin)


def _dist():
    from discoeb_gb300.sharding import dist_env

    return dist_env()


def make_inputs(name, rank=0, world=1, seed=1234):
    from discoeb_gb300 import background, tables
    from discoeb_gb300.gradient import evolve_backgrounds, perturbed_params
    from discoeb_gb300.sharding import shard
    from discoeb_gb300.workloads import fiducial_mnu_param, lcdm_massless_param, sample_cosmologies

    wl = WORKLOADS[name]
    ncosmo, num_k, kmin, kmax, dims, rtol, atol = (wl["ncosmo"], wl["num_k"], wl["kmin"], wl["kmax"], wl["dims"],
                                                   wl["rtol"], wl["atol"])
    grad = name.endswith("_grad")
    if wl.get("objective") == "loglike":
        return _loglike_inputs(name, wl, rank, world, seed)
    if wl["cosmo"] == "sample":
        params, rejected = sample_cosmologies(ncosmo * world, seed=seed)
    else:
        fixed = fiducial_mnu_param() if wl["cosmo"] == "fiducial" else lcdm_massless_param()
        params, rejected = [dict(fixed) for _ in range(ncosmo * world)], 0
    mine = [params[i] for i in shard(ncosmo, world, rank)]
    pert, bgs = None, None
    if grad:
        pert = [perturbed_params(p) for p in mine]
        flat = []
        for p, pp in zip(mine, pert):
            flat.append(p)
            for (_, _, a, b) in pp:
                flat += [a, b]
        ev = evolve_backgrounds(flat)
        nset1 = 1 + 2 * len(pert[0])
        bgs = [ev[i * nset1:(i + 1) * nset1] for i in range(len(mine))]
        ps = [b[0] for b in bgs]
    else:
        ps = [background.evolve_background(param=p) for p in mine]
    tabs = tables.pack_batch(ps, dims["nqmax"])
    tau = np.stack([tables.tau_of_a(p, wl["aexp"]) for p in ps])
    k = np.geomspace(kmin, kmax, num_k)
    kk = np.tile(k, ncosmo)
    com = np.repeat(np.arange(ncosmo, dtype=np.int32), num_k)
    return dict(ps=ps, tables=tabs, tau=tau, k=kk, cosmo=com, dims=dims, rtol=rtol, atol=atol, ncosmo=ncosmo,
                num_k=num_k, rejected=rejected, grad=grad, params=mine, pert=pert, bgs=bgs, kgrid=k, aexp=wl["aexp"],
                cosmo_kind=wl["cosmo"], step_ts=bool(wl.get("step_ts", False)))


def _loglike_inputs(name, wl, rank, world, seed):
    from discoeb_gb300 import tables, tables_gpu
    from discoeb_gb300.gradient import perturbed_params
    from discoeb_gb300.sharding import shard
    from discoeb_gb300.workloads import sample_cosmologies

    ncosmo, num_k, dims = wl["ncosmo"], wl["num_k"], wl["dims"]
    params, rejected = sample_cosmologies(ncosmo * world, seed=seed)
    mine = [params[i] for i in shard(ncosmo, world, rank)]
    pert = [perturbed_params(p) for p in mine]
    # cosmology 0's 13 table sets on the host (for the CPU figures); the GPU problem produces its own
    sets0 = [mine[0]] + [q for (_, _, a, b) in pert[0] for q in (a, b)]
    tabs0, _ = tables_gpu.evolve_background_tables_host(sets0, dims["nqmax"],
                                                        leader=tables_gpu.follow_nominal(1, len(sets0) - 1))
    k = np.geomspace(wl["kmin"], wl["kmax"], num_k)
    return dict(params=mine, pert=pert, bgs="native", dims=dims, rtol=wl["rtol"], atol=wl["atol"], ncosmo=ncosmo,
                num_k=num_k, rejected=rejected, grad=True, objective="loglike", kgrid=k, aexp=wl["aexp"],
                cosmo_kind=wl["cosmo"], step_ts=bool(wl.get("step_ts", False)), tables13=tabs0,
                tau13=tables.tau_of_a_blob(tabs0, wl["aexp"]),
                eps0=np.array([e for (_, e, _, _) in pert[0]]), max_steps=wl["max_steps"], ck_cap=wl["ck_cap"],
                tables=tabs0[:1], tau=tables.tau_of_a_blob(tabs0[:1], wl["aexp"]))


def loglike_weights(kmodes, nout, volume=VOLUME_MPC3):
    """N_k / 2 per (k, a): the inverse variance of ln P for a diagonal Gaussian
    covariance with N_k = V k^2 dk / (2 pi^2) modes per log-spaced k-bin."""
    k = np.asarray(kmodes, dtype=np.float64)
    edges = np.sqrt(k[1:] * k[:-1])
    dk = np.empty_like(k)
    dk[1:-1] = edges[1:] - edges[:-1]
    dk[0] = edges[0] - k[0] ** 2 / edges[0]
    dk[-1] = k[-1] ** 2 / edges[-1] - edges[-1]
    nk = volume * k ** 2 * dk / (2.0 * np.pi ** 2)
    return np.repeat((nk / 2.0)[:, None], nout, axis=1)


def cpu_measure(inp, budget_s=20.0, threads=0, dense_steps=None):
    """CPU figures on one sample of the workload: every 64th mode of
    cosmology 0's k-grid (at least 8 modes).

    * structured: the kernel's own code built for the host (tests/native),
      threads over modes, each mode run to completion -- the nominal solve
      with checkpoints and, for gradient workloads, one adjoint sweep;
      cosmology solves/s = sampled fraction of a cosmology / wall time;
    * dense (the oracle, the reference algorithm): every sampled mode run for
      at most ``dense_steps`` attempted steps (chosen to fill ~budget_s / 2),
      OpenMP over modes; its attempted steps per second, divided by the
      work of one cosmology solve -- (num_k / sampled modes) x sum over the
      sample of (attempted + 6 accepted) steps, the nominal solve plus one
      forward solve's work per ODE parameter for the reference's
      forward-mode gradient (its jacfwd of one parameter takes 1.98x its
      forward solve: nb_minimal_example.ipynb cells 11, 15), or attempted
      steps alone for forward workloads."""
    import oracle
    from concurrent.futures import ThreadPoolExecutor

    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from native import harness as H

    threads = threads or os.cpu_count() or 1
    num_k, dims = inp["num_k"], inp["dims"]
    stride = max(1, min(64, num_k // 8))
    sel = np.arange(0, num_k, stride)
    ks = np.asarray(inp["kgrid"])[sel]
    dtup = tuple(dims[n] for n in ("lmaxg", "lmaxgp", "lmaxr", "lmaxnu", "nqmax"))
    grad = bool(inp.get("grad"))
    max_steps = inp.get("max_steps", 8192)
    tab0 = inp["tables"][0]
    tau0 = np.asarray(inp["tau"])[0]
    if grad and "tables13" in inp:
        tabs13, tau13, eps0 = inp["tables13"], inp["tau13"], inp["eps0"]
    else:
        tabs13 = None
    nout = tau0.shape[0]

    def one(k):
        if tabs13 is not None:
            gy = np.zeros((nout, 20))
            gy[:, 4] = 1.0
            _, _, info, st = H.adjoint(tabs13, eps0, float(k), tau13, dtup, gy, rtol=inp["rtol"], atol=inp["atol"],
                                       max_steps=max_steps, ck_cap=inp.get("ck_cap", 32),
                                       step_to_outputs=inp["step_ts"], full_info=True)
            return info[1] + info[3], info[1], info[0]
        _, ss, _, _ = H.solve_rr(tab0[None], 1, np.array([k]), tau0[None], record=True, rtol=inp["rtol"],
                                 atol=inp["atol"], max_steps=max_steps, step_to_outputs=inp["step_ts"], **dims)
        return int(ss[0, 1] + ss[0, 2]), int(ss[0, 1]), int(ss[0, 0])

    H.lib()
    t0 = time.perf_counter()
    with ThreadPoolExecutor(threads) as ex:
        res = list(ex.map(one, ks))
    t_struct = time.perf_counter() - t0
    att = np.array([r[0] for r in res])
    acc = np.array([r[1] for r in res])
    frac = sel.size / num_k
    work = (att + (6 * acc if grad else 0)).sum() / frac
    # dense: a bounded number of steps per sampled mode, grown until it fills half the budget
    cap = dense_steps or 8
    while True:
        t0 = time.perf_counter()
        _, so = oracle.solve(tab0, ks, tau0, rtol=inp["rtol"], atol=inp["atol"], max_steps=int(cap), nthreads=threads,
                             step_to_outputs=inp["step_ts"], **dims)
        t_dense = time.perf_counter() - t0
        if dense_steps or t_dense >= budget_s / 8 or cap >= max_steps:
            break
        cap = min(max_steps, int(cap * max(2.0, budget_s / 2 / max(t_dense, 1e-3))))
    done = int(so[:, 1].sum() + so[:, 2].sum())
    rate = done / t_dense
    gtxt = " + 8-parameter gradient" if grad else ""
    return {
        "dense": {"value": rate / work, "unit": "cosmology solves/s", "cores": threads, "kind": "port",
                  "sample": f"{sel.size} modes (every {stride}th of cosmology 0's {num_k}-point k-grid), at most "
                            f"{int(cap)} attempted steps each: {done} steps in {t_dense:.2f} s = {rate:.1f} steps/s; "
                            f"one cosmology solve{gtxt} = {work:.4g} steps (attempted"
                            + (" + 6 x accepted, forward-mode gradient model" if grad else "")
                            + "; counted on the sample by the structured solve, same controller, scaled by "
                            f"{1 / frac:g})", "seconds": t_dense, "cap": int(cap)},
        "structured": {"value": frac / t_struct, "unit": "cosmology solves/s", "cores": threads,
                       "kind": "kernel code built for the host",
                       "sample": f"the same {sel.size} modes run to completion" + (" (nominal solve with checkpoints "
                                 "and one adjoint sweep each)" if tabs13 is not None else "")
                                 + f" in {t_struct:.2f} s; value = {frac:g} of a cosmology / wall time",
                       "attempted_steps": int(att.sum())},
        "sample_modes": int(sel.size), "stride": int(stride), "work_steps_per_cosmology": float(work)}


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while running."""

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.samples = []
        self._p = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                        "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self._p = None
        return self

    def _read(self):
        for line in self._p.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self._p is not None:
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def cpu_baseline(inp, seconds=20.0, threads=0):
    """Oracle (CPU port, FP64, OpenMP over modes) on a bounded sample of the
    workload; returns cosmology solves/s scaled from the sampled modes."""
    import oracle

    threads = threads or os.cpu_count() or 1
    num_k = inp["num_k"]
    # sample: every s-th k of cosmology 0, growing until the time budget is used
    stride = 64
    done_modes, t_used = 0, 0.0
    while True:
        sel = np.arange(0, num_k, stride)
        t = time.perf_counter()
        oracle.solve(inp["tables"][0], inp["k"][sel], inp["tau"][0], rtol=inp["rtol"], atol=inp["atol"],
                     nthreads=threads, **inp["dims"])
        dt = time.perf_counter() - t
        done_modes += sel.size
        t_used += dt
        if t_used >= seconds or stride == 1:
            break
        stride = max(1, stride // 2)
    per_mode = t_used / done_modes
    solves = 13 if inp.get("grad") else 1   # nominal + 6 parameters x +-eps by central differences
    return {"value": 1.0 / (per_mode * num_k * solves), "unit": "cosmology solves/s", "cores": threads, "kind": "port",
            "sample": f"{done_modes} modes of cosmology 0 (k strided over the {num_k}-point grid), {t_used:.1f} s"
                      + (", x13 solves per cosmology for the 6 ODE gradients (+-eps) and the nominal P(k)" if solves > 1 else "")}


def _launch_arg(text):
    where, _, per_sm = text.partition("/")
    return (where, int(per_sm or 0))


def l2_flush_buffer():
    """256 MB device buffer written before every timed step (L2 is 129 MB), so
    no step starts with the previous step's tables or outputs in L2."""
    import torch

    buf = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    buf.fill_(0)   # first touch outside the timed region
    torch.cuda.synchronize()
    return buf


def algorithmic_flops_per_step(dims, nq):
    """FP64 flops of one attempted step of the structured Rodas5 solve: 8 RHS evaluations (one
    forward-mode), stage sums, the O(n) factorisation and 8 structured solves."""
    from discoeb_gb300.perturbations import nvar

    n = nvar(dims["lmaxg"], dims["lmaxgp"], dims["lmaxr"], dims["lmaxnu"], dims["nqmax"])
    rhs = 12 * n + 60 * nq + 220          # one RHS evaluation
    rhs_dual = 2 * rhs                    # f and d f / d a
    stage_sums = 2 * n * (1 + 2 + 3 + 4 + 5 + 1 + 1)   # u_i
    stage_rhs = 2 * n * (0 + 1 + 2 + 3 + 4 + 5 + 6 + 7) + 4 * n   # C_ij k_j and d_i dT
    factor = 10 * n + 600 + 2 * 13 * n    # chain pivots, 8x8 LU, Z_h, Z_e
    solves = 8 * 13 * n                   # per-stage structured solve
    ctrl = 2 * n + 80
    return rhs_dual + 7 * rhs + stage_sums + stage_rhs + factor + solves + ctrl


def run_ours(args):
    import torch

    world, rank, local = _dist()
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    import discoeb_gb300 as deb
    from discoeb_gb300 import _native, perturbations as pt

    inp = make_inputs(args.workload, rank, world)
    dims = inp["dims"]
    if inp.get("objective") == "loglike":
        return run_loglike(args, inp, world, rank, local)
    if inp["grad"]:
        return run_gradient(args, inp, world, rank, local)
    prob = deb.DeviceProblem(inp["tables"], inp["k"], inp["tau"], inp["cosmo"], exec_mode=args.exec_mode, **dims)
    cfg = pt._cfg(inp["rtol"], inp["atol"], 0.25, 0.80, 0.0, 20.0, 0.3, args.max_steps)
    stream = torch.cuda.current_stream()

    if args.launch:
        prob.plan = pt.get_plan(prob.dims, prob.nmode, _launch_arg(args.launch))
    tune_ms = prob.tune(cfg) if args.tune and not args.launch else {}
    launch = prob.plan.launch_info()
    for _ in range(args.warmup):
        prob.launch(cfg, stream)
        prob.power(4, stream)
    # the whole solve (queue reset, persistent launch, get_power) as one CUDA graph
    prob.capture(cfg, 4)
    torch.cuda.synchronize()
    st = prob.status.cpu().numpy()
    steps = prob.steps.cpu().numpy()
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    flush = l2_flush_buffer()
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        e_start.record(stream)
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            ev0[i].record(stream)
            prob.replay()
            ev1[i].record(stream)
        e_end.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    dev_s = e_start.elapsed_time(e_end) / 1e3
    if world > 1:
        torch.distributed.barrier()
    kern_ms = [a.elapsed_time(b) for a, b in zip(ev0, ev1)]
    from discoeb_gb300.sharding import max_over_ranks

    t_step = max_over_ranks(dev_s / args.steps, device="cuda")
    total_cosmo = inp["ncosmo"] * world
    value = total_cosmo / t_step

    # end to end through the public call with host buffers
    e2e_steps = max(1, min(args.steps, 3))
    host_tabs, host_k, host_tau, host_com = (np.ascontiguousarray(inp["tables"]), np.ascontiguousarray(inp["k"]),
                                             np.ascontiguousarray(inp["tau"]), np.ascontiguousarray(inp["cosmo"]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        y = deb.solve(host_tabs, host_k, host_tau, host_com, rtol=inp["rtol"], atol=inp["atol"], max_steps=args.max_steps,
                      throw=False, exec_mode=args.exec_mode, **dims)
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    h2d = host_tabs.nbytes + host_k.nbytes + host_tau.nbytes + host_com.nbytes
    d2h = int(y.nbytes) + prob.status.numel() * 4

    peak = _native.measure_fp64_peak(stream.cuda_stream)
    nsteps_attempted = int(steps.sum())
    flops = algorithmic_flops_per_step(dims, dims["nqmax"]) * nsteps_attempted
    kern_s = statistics.median(kern_ms) * 1e-3
    achieved = flops / kern_s
    out = {
        "metric": "P(k) forward solves/s on 1 GB300, batched FP64 structured Rodas5 (gradient not included)",
        "value": value, "unit": "cosmology solves/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded cosmology sample, host RECFAST tables)",
        "config": {"workload": args.workload, "ncosmo_per_gpu": inp["ncosmo"], "num_k": inp["num_k"],
                   "modes_per_step": int(inp["k"].shape[0]), "nvar": prob.n, "rtol": inp["rtol"],
                   "linear_solver": "structured", "exec_mode": ["auto", "lane", "warp"][prob.plan.dims.exec_mode]
                   if args.exec_mode != "auto" else "auto",
                   "cuda_graph": "queue reset + persistent launch + get_power captured once, replayed per step",
                   "launch_shape": launch, "autotune_ms": {f"{a}/{b}": round(v, 2) for (a, b), v in tune_ms.items()},
                   "l2": "flushed before every timed step (256 MB write); per-mode state in shared memory "
                         "(stage vectors in L2 with the global launch shape)",
                   "aexp_out": inp["aexp"], "cosmology": inp["cosmo_kind"], "step_to_outputs": inp["step_ts"],
                   "redrawn_cosmologies": inp["rejected"]},
        "e2e": {"value": total_cosmo / t_e2e if world == 1 else None, "unit": "cosmology solves/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "note": "FP64-pipe bound; peak = FP64 FMA microkernel measured in this run"},
        "gpu_launches": 2 * args.steps,
        "clocks": clk.summary(),
        "kernel_ms_median": statistics.median(kern_ms),
        "attempted_steps_per_launch": nsteps_attempted,
        "mode_status_nonzero": int((st != 0).sum()),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(inp, seconds=args.cpu_seconds)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


# DRAM read + write bytes per accepted step of adjoint_kernel, from an ncu capture of
# profile_1cosmo_1216k_n1098_8a_rtol1e-6_loglike at 4 warps per SM (23.8 GB for 30 893 accepted steps)
ADJ_DRAM_BYTES_PER_STEP = 23.80e9 / 30893


def algorithmic_flops_adjoint_step(dims, nq):
    """FP64 flops of one accepted step of the adjoint sweep: the recomputed
    forward step, and the eight stages backwards -- a transposed structured
    solve, two bilinear-form passes and one transposed Jacobian product each,
    the stage-vector updates (sum_s s k-bar axpys, u and u-bar passes) -- plus
    the step's W-term (one more form and a transposed product with
    a-derivative coefficients) and the two transposed solves of Y_h, Y_e.
    The scalar coefficient evaluations on single lanes are not counted."""
    from discoeb_gb300.perturbations import nvar

    n = nvar(dims["lmaxg"], dims["lmaxgp"], dims["lmaxr"], dims["lmaxnu"], dims["nqmax"])
    solve_t = 13 * n
    form = 8 * n + 40 * nq
    jt = 8 * n + 10 * nq
    per_stage = solve_t + 2 * form + jt + 4 * n
    vectors = 2 * n * 3 * (1 + 2 + 3 + 4 + 5 + 6 + 7)
    wterm = form + 2 * jt + 2 * solve_t
    return algorithmic_flops_per_step(dims, nq) + 8 * per_stage + vectors + wterm


def plain_fp64(inp, args, seconds=10.0):
    """The plain single-cosmology FP64 form on the GPU: the reference's method
    (dense W = I/(gamma h) - J formed and LU-factored every step,
    DEB_SOLVE_DENSE), one warp per mode, on the CPU figures' sample of
    cosmology 0's modes, each run for a bounded number of attempted steps;
    cosmology solves/s = its attempted steps per second / the work of one
    cosmology solve (the forward-mode gradient model of cpu_measure)."""
    import torch

    import discoeb_gb300 as deb
    from discoeb_gb300 import perturbations as pt

    num_k = inp["num_k"]
    stride = max(1, min(64, num_k // 8))
    sel = np.arange(0, num_k, stride)
    ks = np.asarray(inp["kgrid"])[sel]
    tab0, tau0 = inp["tables"][0], np.asarray(inp["tau"])[0]
    cap = 4
    while True:
        prob = deb.DeviceProblem(tab0[None], ks, tau0[None], None, linear_solver="dense", exec_mode="warp",
                                 **inp["dims"])
        cfg = pt._cfg(inp["rtol"], inp["atol"], 0.25, 0.80, 0.0, 20.0, 0.3, cap)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        prob.launch(cfg)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) * 1e-3
        done = int(prob.steps.sum().item())
        if t >= seconds / 4 or cap >= inp.get("max_steps", args.max_steps):
            break
        cap = int(cap * max(2.0, seconds / 2 / max(t, 1e-3)))
    return {"steps": done, "seconds": t, "cap": cap, "modes": int(sel.size), "rate": done / t}


def loglike_config(args, inp):
    """The workload as both arms name it."""
    from discoeb_gb300.perturbations import nvar
    from discoeb_gb300.gradient import THETA

    d = inp["dims"]
    return {"workload": args.workload, "ncosmo_per_gpu": inp["ncosmo"], "num_k": inp["num_k"],
            "kmin": float(inp["kgrid"][0]), "kmax": float(inp["kgrid"][-1]), "nout": len(inp["aexp"]),
            "aexp_out": [inp["aexp"][0], inp["aexp"][-1]], "modes_per_step": inp["ncosmo"] * inp["num_k"],
            "steps_on_outputs": inp["step_ts"],
            "nvar": nvar(d["lmaxg"], d["lmaxgp"], d["lmaxr"], d["lmaxnu"], d["nqmax"]), "rtol": inp["rtol"],
            "theta": list(THETA),
            "gradient": "d ln L / d theta of a Gaussian likelihood of P(k, a) (diagonal covariance 2 / N_k, "
                        f"V = {VOLUME_MPC3:g} Mpc^3): one discrete-adjoint sweep per mode on the recorded steps "
                        "(jacfwd semantics); A_s, n_s analytic",
            "l2": "GPU arm: flushed before every timed step (256 MB write)", "cosmology": inp["cosmo_kind"],
            "redrawn_cosmologies": inp["rejected"]}


def run_loglike(args, inp, world, rank, local):
    """P(k, a) and the 8-parameter gradient of a Gaussian log-likelihood per
    cosmology: recorded solve with checkpoints + one adjoint sweep per mode."""
    import torch

    import discoeb_gb300 as deb
    from discoeb_gb300 import _native, perturbations as pt
    from discoeb_gb300.gradient import LoglikeProblem

    dims = inp["dims"]
    nout = len(inp["aexp"])
    nc = inp["ncosmo"]
    w = loglike_weights(inp["kgrid"], nout)
    lp = LoglikeProblem(inp["params"], "native", inp["pert"], inp["kgrid"], inp["aexp"],
                        np.zeros((nc, inp["num_k"], nout)), w, rtol=inp["rtol"], atol=inp["atol"],
                        max_steps=inp["max_steps"], ck_cap=inp["ck_cap"], step_to_outputs=inp["step_ts"], **dims)
    gp = lp.gp
    stream = torch.cuda.current_stream()
    if args.launch:
        gp.plan = pt.get_plan(gp.dims, gp.nmode, _launch_arg(args.launch))
    tune_ms = {}
    if args.tune and not args.launch:
        from discoeb_gb300 import autotune

        best, tune_ms = autotune.tune(gp.dims, gp.nmode, gp._record, (("global", 0), ("all_global", 0)))
        gp.plan = pt.get_plan(gp.dims, gp.nmode, best)
    launch = gp.plan.launch_info()
    # synthetic data: the first solve's ln P with 5% seeded scatter
    P0 = gp.forward(stream)
    torch.cuda.synchronize()
    gp.fit_checkpoints()
    rng = np.random.default_rng(4321)
    lnPd = np.log(P0.cpu().numpy()).reshape(nc, inp["num_k"], nout) + 0.05 * rng.standard_normal((nc, inp["num_k"], nout))
    lp.set_data(lnPd)
    # eager warm-up steps, timed per launch: forward (record + get_power), likelihood + adjoint; the
    # first also loads the kernels' modules and uploads their constants, so its split is not used
    split = []
    for _ in range(max(2, args.warmup)):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        ev[0].record(stream)
        P = gp.forward(stream)
        ev[1].record(stream)
        lp.backward(P, stream)
        ev[2].record(stream)
        split.append(ev)
    torch.cuda.synchronize()
    lp.check()
    fwd_ms = [e[0].elapsed_time(e[1]) for e in split[1:]]
    step_ms = [e[1].elapsed_time(e[2]) for e in split[1:]]
    lp.capture()
    lp.replay(stream)
    torch.cuda.synchronize()
    lp.check()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    flush = l2_flush_buffer()
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        e_start.record(stream)
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            ev0[i].record(stream)
            lp.replay(stream)
            ev1[i].record(stream)
        e_end.record(stream)
        torch.cuda.synchronize()
    dev_s = e_start.elapsed_time(e_end) / 1e3
    graph_ms = [a.elapsed_time(b) for a, b in zip(ev0, ev1)]
    lp.check()
    if world > 1:
        torch.distributed.barrier()
    from discoeb_gb300.sharding import max_over_ranks

    t_step = max_over_ranks(dev_s / args.steps, device="cuda")
    total_cosmo = nc * world
    value = total_cosmo / t_step

    # end to end through the public call from the parameters: the first two calls of a shape build the problem
    # and capture its graph (untimed); a timed call produces the tables of all 13 sets per cosmology on the host
    # cores, copies them and the data vector in, replays the graph and copies P, ln L and the gradient out
    def e2e_call():
        return deb.loglike_grad(params=inp["params"], lnP_data=lnPd, weights=w, aexp_out=inp["aexp"],
                                kmin=float(inp["kgrid"][0]), kmax=float(inp["kgrid"][-1]), num_k=inp["num_k"],
                                rtol=inp["rtol"], atol=inp["atol"], max_steps=inp["max_steps"], ck_cap=inp["ck_cap"],
                                step_to_outputs=inp["step_ts"], tables="native", **dims)

    e2e_steps = max(1, min(args.steps, 2))
    e2e_call()
    e2e_call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        Pe, lnL, g, _ = e2e_call()
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / e2e_steps
    from discoeb_gb300 import gradient as _grad

    lpe = list(_grad._ll_problems.values())[-1]
    h2d = lpe.gp.input_bytes() + lnPd.nbytes
    d2h = int(Pe.nbytes + lnL.nbytes + g.nbytes)

    peak = _native.measure_fp64_peak(stream.cuda_stream)
    att = int(gp.d_steps.sum().item())
    acc = int(gp.d_nrec.sum().item())
    strides = gp.d_ckstride.cpu().numpy()
    nrec = gp.d_nrec.cpu().numpy()
    recomputed = int((nrec - (nrec + strides - 1) // strides).sum())
    f_fwd = algorithmic_flops_per_step(dims, dims["nqmax"])
    f_adj = algorithmic_flops_adjoint_step(dims, dims["nqmax"])
    adj_flops = f_adj * acc + f_fwd * recomputed
    t_adj = statistics.median(step_ms) * 1e-3
    t_fwd = statistics.median(fwd_ms) * 1e-3
    achieved = adj_flops / t_adj
    # the plain single-cosmology FP64 form (dense LU per step, the reference's method) on the same GPU
    plain = None
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu = cpu_measure(inp, budget_s=args.cpu_seconds)
        pf = plain_fp64(inp, args)
        plain = {"value": pf["rate"] / cpu["work_steps_per_cosmology"], "unit": "cosmology solves/s",
                 "sample": f"{pf['modes']} modes of cosmology 0 (the CPU figures' sample), dense W and LU per step "
                           f"(DEB_SOLVE_DENSE), one warp per mode, at most {pf['cap']} attempted steps each: "
                           f"{pf['steps']} steps in {pf['seconds']:.2f} s on the GPU, scaled by the work of one "
                           f"cosmology solve as the dense CPU figure"}
        plain["batched_over_plain"] = value / plain["value"]
    out = {
        "metric": METRIC,
        "value": value, "unit": "cosmology solves/s (P(k, a) + 8-parameter gradient)", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded cosmology sample; tables of theta and theta +- 1e-4 theta from the library's "
                "RECFAST producer; data vector = each cosmology's own ln P with 5% seeded scatter)",
        "config": loglike_config(args, inp),
        "detail": {"checkpoints": f"per-mode slots fitted to the step counts ({gp.d_ckpt.numel() * 8 / 1e9:.1f} GB), "
                                  f"strides {int(strides.min())}-{int(strides.max())}",
                   "cuda_graph": "record + get_power + likelihood + adjoint captured once, replayed per step",
                   "launch_shape": launch, "adjoint_launch": gp.adj_plan.launch_info(),
                   "autotune_ms": {f"{a}/{b}": round(v, 2) for (a, b), v in tune_ms.items()}},
        "e2e": {"value": total_cosmo / t_e2e if world == 1 else None,
                "unit": "cosmology solves/s (P(k, a) + 8-parameter gradient)",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "inputs": "parameter dicts (tables of all 13 sets per cosmology produced on the host cores inside "
                          "the timed call) and the data vector; P(k, a), ln L and the gradient copied back"},
        "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": ADJ_DRAM_BYTES_PER_STEP * acc, "kernel": "adjoint_kernel",
                     "note": "FP64 pipe ~half busy, latency-bound (2 warps per scheduler at 255 registers, global-memory "
                             "waits); peak = FP64 FMA microkernel measured in this run (MEASURED_PEAKS.json has no FP64 "
                             "figure); achieved = algorithmic FLOPs of the adjoint sweep (per accepted step + "
                             "recomputed segment steps) / the adjoint launch's time; traffic = DRAM bytes per accepted "
                             "step of an ncu capture of the counter-capture workload x accepted steps"},
        "gpu_launches": 3 * args.steps,
        "clocks": clk.summary(),
        "forward_ms_median": statistics.median(fwd_ms), "adjoint_ms_median": statistics.median(step_ms),
        "graph_ms_median": statistics.median(graph_ms),
        "attempted_steps_per_step": att, "accepted_steps_per_step": acc, "recomputed_steps_per_step": recomputed,
    }
    if cpu is not None:
        out["cpu_baseline"] = {k: cpu["dense"][k] for k in ("value", "unit", "cores", "kind", "sample")}
        out["cpu_structured"] = {k: cpu["structured"][k] for k in ("value", "unit", "cores", "kind", "sample")}
        out["plain_fp64"] = plain
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


def run_gradient(args, inp, world, rank, local):
    """P(k) + 8-parameter gradient per cosmology: record + replay launches."""
    import torch

    import discoeb_gb300 as deb
    from discoeb_gb300 import _native, perturbations as pt
    from discoeb_gb300.gradient import GradientProblem

    dims = inp["dims"]
    gp = GradientProblem(inp["params"], inp["bgs"], inp["pert"], inp["kgrid"], inp["aexp"], rtol=inp["rtol"],
                         atol=inp["atol"], max_steps=args.max_steps, step_to_outputs=inp["step_ts"], **dims)
    stream = torch.cuda.current_stream()
    if args.launch:
        gp.plan = pt.get_plan(gp.dims, gp.nset * gp.nmode, _launch_arg(args.launch))
    tune_ms = gp.tune() if args.tune and not args.launch else {}
    launch = gp.plan.launch_info()
    # eager warm-up steps, timed per launch for the record / replay split
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(max(1, args.warmup))]
    for i in range(len(evs)):
        gp.run(stream, evs[i])
    torch.cuda.synchronize()
    gp.check()
    rec_ms = [e[0].elapsed_time(e[1]) for e in evs]
    rep_ms = [e[1].elapsed_time(e[2]) for e in evs]
    # the whole step (record, replay, get_power, difference quotients) as one CUDA graph
    gp.capture()
    gp.replay(stream)
    torch.cuda.synchronize()
    gp.check()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    flush = l2_flush_buffer()
    e_start, e_end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ev1 = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        e_start.record(stream)
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            ev0[i].record(stream)
            gp.replay(stream)
            ev1[i].record(stream)
        e_end.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    dev_s = e_start.elapsed_time(e_end) / 1e3
    graph_ms = [a.elapsed_time(b) for a, b in zip(ev0, ev1)]
    gp.check()
    if world > 1:
        torch.distributed.barrier()
    from discoeb_gb300.sharding import max_over_ranks

    t_step = max_over_ranks(dev_s / args.steps, device="cuda")
    total_cosmo = inp["ncosmo"] * world
    value = total_cosmo / t_step

    # end to end through the public call from host buffers (tables for theta and theta +- eps): the first
    # two calls of a shape build the problem and capture its graph (untimed), later calls pack and copy
    # their inputs through pinned memory, replay the graph and copy P and the gradient back
    e2e_steps = max(1, min(args.steps, 2))

    def e2e_call():
        return deb.evolve_perturbations_grad(params=inp["params"], aexp_out=inp["aexp"], kmin=inp["kgrid"][0],
                                             kmax=inp["kgrid"][-1], num_k=inp["num_k"], rtol=inp["rtol"],
                                             atol=inp["atol"], max_steps=args.max_steps, backgrounds=inp["bgs"],
                                             step_to_outputs=inp["step_ts"], **dims)

    e2e_call()
    e2e_call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        P, D, _ = e2e_call()
    torch.cuda.synchronize()
    t_e2e = (time.perf_counter() - t0) / e2e_steps

    # the same from the parameters alone: the tables of all 13 sets per cosmology produced by the library's
    # producer on the host cores inside the timed call
    def e2e_params_call():
        return deb.evolve_perturbations_grad(params=inp["params"], aexp_out=inp["aexp"], kmin=inp["kgrid"][0],
                                             kmax=inp["kgrid"][-1], num_k=inp["num_k"], rtol=inp["rtol"],
                                             atol=inp["atol"], max_steps=args.max_steps, tables="native",
                                             step_to_outputs=inp["step_ts"], **dims)

    e2e_params_call()
    e2e_params_call()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        e2e_params_call()
    torch.cuda.synchronize()
    t_e2e_params = (time.perf_counter() - t0) / e2e_steps
    from discoeb_gb300 import gradient as _grad, tables_gpu

    gpp = [g for g in _grad._problems.values() if g.table_source == "native"][0]
    # table production alone, all 13 sets per cosmology: host cores (C++ threads) and GPU (one launch)
    all_sets = list(inp["params"]) + [q for pp in inp["pert"] for (_, _, a, b) in pp for q in (a, b)]
    lead = tables_gpu.follow_nominal(len(inp["params"]), len(all_sets) // len(inp["params"]) - 1)
    t0 = time.perf_counter()
    tables_gpu.evolve_background_tables_host(all_sets, dims["nqmax"], leader=lead)
    native_tables_ms = (time.perf_counter() - t0) * 1e3
    tables_gpu.evolve_background_tables(all_sets, dims["nqmax"], aexp_out=inp["aexp"], leader=lead)
    te0, te1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    te0.record(stream)
    tables_gpu.evolve_background_tables(all_sets, dims["nqmax"], aexp_out=inp["aexp"], leader=lead)
    te1.record(stream)
    torch.cuda.synchronize()
    gpu_tables_ms = te0.elapsed_time(te1)
    h2d = gp.input_bytes()
    d2h = int(P.nbytes + D.nbytes) + 4 * (gp.nmode * (1 + gp.nset))

    peak = _native.measure_fp64_peak(stream.cuda_stream)
    att = int(gp.d_steps.sum().item())
    acc = int(gp.d_nrec.sum().item())
    adjoint = gp.method == "adjoint"
    if adjoint:
        # one adjoint sweep per (output, mode) on the recorded steps
        rep = 0
        flops = (algorithmic_flops_per_step(dims, dims["nqmax"]) * att
                 + algorithmic_flops_adjoint_step(dims, dims["nqmax"]) * acc * gp.nseed)
        how = "discrete adjoint of the recorded steps (deb_adjoint, one sweep per output and mode; jacfwd semantics)"
    else:
        rep = acc * gp.nset
        flops = algorithmic_flops_per_step(dims, dims["nqmax"]) * (att + rep)
        how = "central differences over the replayed nominal step sequence (jacfwd semantics)"
    kern_s = statistics.median(graph_ms) * 1e-3     # the graph's two solver launches + sub-ms tail work
    achieved = flops / kern_s
    out = {
        "metric": "P(k)+dP/dtheta solves/s on 1 GB300, batched FP64 (8 parameters; structured Rodas5, "
                  + ("adjoint of" if adjoint else "tangents of") + " the recorded step sequence)",
        "value": value, "unit": "cosmology solves/s (P(k) + 8-parameter gradient)", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded cosmology sample, host RECFAST tables for theta and theta +- 1e-4 theta)",
        "config": {"workload": args.workload, "ncosmo_per_gpu": inp["ncosmo"], "num_k": inp["num_k"],
                   "modes_per_step": gp.nmode,
                   ("adjoint_items_per_step" if adjoint else "replay_items_per_step"):
                       gp.nmode * (gp.nseed if adjoint else gp.nset),
                   "nvar": pt.nvar(dims["lmaxg"], dims["lmaxgp"], dims["lmaxr"], dims["lmaxnu"], dims["nqmax"]),
                   "rtol": inp["rtol"], "theta": list(gp.theta),
                   "gradient": how,
                   "cuda_graph": "record + " + ("adjoint" if adjoint else "replay + quotients")
                                 + " + get_power captured once, replayed per step",
                   "launch_shape": launch, "autotune_ms": {f"{a}/{b}": round(v, 2) for (a, b), v in tune_ms.items()},
                   "l2": "flushed before every timed step (256 MB write); tables %.1f MB read per step" % ((gp.d_tab0.numel() + gp.d_tabs.numel()) * 8 / 1e6),
                   "aexp_out": inp["aexp"], "cosmology": inp["cosmo_kind"], "step_to_outputs": inp["step_ts"],
                   "redrawn_cosmologies": inp["rejected"]},
        "e2e": {"value": total_cosmo / t_e2e if world == 1 else None, "unit": "cosmology solves/s (P(k) + 8-parameter gradient)",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "inputs": "host tables of the 13 parameter sets per cosmology (evolve_background output), packed per call"},
        "e2e_from_params": {"value": total_cosmo / t_e2e_params if world == 1 else None,
                            "unit": "cosmology solves/s (P(k) + 8-parameter gradient)",
                            "h2d_bytes_per_step": int(gpp.input_bytes()), "d2h_bytes_per_step": int(d2h),
                            "inputs": "parameter dicts only; background + RECFAST tables of all 13 sets per cosmology "
                                      "produced inside the timed call by the library's producer on the host cores",
                            "table_production_ms": {"host_cores": native_tables_ms, "gpu": gpu_tables_ms,
                                                    "sets": len(all_sets)}},
        "roofline": {"bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "note": "FP64-pipe bound (state in shared memory / L2, DRAM idle); peak = FP64 FMA microkernel measured in this run; "
                             + ("achieved = algorithmic FLOPs of the record (attempted steps) and of the adjoint sweeps "
                                "(accepted steps x outputs) / the graph's time" if adjoint else
                                "achieved = algorithmic FLOPs of the structured Rodas5 step x (attempted + replayed steps)")},
        "gpu_launches": 4 * args.steps,
        "clocks": clk.summary(),
        "forward_value": total_cosmo / (statistics.median(rec_ms) * 1e-3),
        "graph_ms_median": statistics.median(graph_ms),
        "record_ms_eager_median": statistics.median(rec_ms),
        ("adjoint_ms_eager_median" if adjoint else "replay_ms_eager_median"): statistics.median(rep_ms),
        "attempted_steps_per_launch": att, "replayed_steps_per_launch": rep, "accepted_steps_per_launch": acc,
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(inp, seconds=args.cpu_seconds)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        torch.distributed.destroy_process_group()


# width of each parameter's sampled range (the batched spec), the scale of the reference derivative's step
PRIOR_WIDTH = {"Omegam": 0.1, "Omegab": 0.015, "h": 0.15, "mnu": 0.24, "w_DE_0": 0.4, "w_DE_a": 0.6}


def _accuracy_large(args, inp):
    """The accuracy record of a large workload (nvar 1098, 64 outputs) on
    cosmology 0 at accuracy_modes log-spaced k over its range: P(k) at the
    workload's tolerance against the same solver at rtol = atol = 1e-9 (the
    dense oracle takes minutes per step at this size; the structured solve
    equals it to rounding, tests/test_gpu_parity.py at this hierarchy), and
    the adjoint's d ln P / d theta at every output against central
    differences over 1e-3 of each parameter's range of rtol 1e-9 solves on
    tables that follow the nominal RECFAST steps.  Errors relative to the
    largest |value| of each output's P and of each parameter's derivative."""
    import torch

    import discoeb_gb300 as deb
    from discoeb_gb300 import tables as tb, tables_gpu
    from discoeb_gb300.gradient import THETA, _get, _with

    dims, aexp = inp["dims"], np.asarray(inp["aexp"])
    p0 = inp["params"][0]
    k = np.geomspace(inp["kgrid"][0], inp["kgrid"][-1], args.accuracy_modes)
    P, D, _ = deb.evolve_perturbations_grad(params=p0, aexp_out=aexp, kmin=float(k[0]), kmax=float(k[-1]),
                                            num_k=k.size, rtol=inp["rtol"], atol=inp["atol"], max_steps=args.max_steps,
                                            method="adjoint", step_to_outputs=inp["step_ts"], **dims)
    names = [n for n in PRIOR_WIDTH]
    sets = [p0]
    for name in names:
        v, e = float(_get(p0, name)), 1e-3 * PRIOR_WIDTH[name]
        sets += [_with(p0, name, v + e), _with(p0, name, v - e)]
    tabs, st = tables_gpu.evolve_background_tables_host(sets, dims["nqmax"],
                                                        leader=tables_gpu.follow_nominal(1, len(sets) - 1))
    taus = tb.tau_of_a_blob(tabs, aexp)
    ns = len(sets)
    kk, com = np.tile(k, ns), np.repeat(np.arange(ns, dtype=np.int32), k.size)
    t0 = time.perf_counter()
    y = deb.solve(tabs, kk, taus, com, rtol=1e-9, atol=1e-9, max_steps=2000000, step_to_outputs=inp["step_ts"],
                  **dims)
    tight_s = time.perf_counter() - t0
    lp = np.log(y[..., 4] ** 2).reshape(ns, k.size, aexp.size)
    param0 = tables_gpu.param_from_blob(p0, tabs[0])
    Pt = np.stack([deb.get_power(k=k, y=y[:k.size, o, :], idx=4, param=param0) for o in range(aexp.size)], axis=1)
    out = {"workload": args.workload, "modes": int(k.size), "k": [float(x) for x in k], "n_outputs": int(aexp.size),
           "steps_on_outputs": inp["step_ts"],
           "rtol": inp["rtol"], "reference": "same solver at rtol = atol = 1e-9 (tight solve %.0f s)" % tight_s,
           "pk_max_rel_err": float((np.abs(P - Pt) / np.abs(Pt)).max())}
    errs = {}
    for j, name in enumerate(names):
        gt = (lp[1 + 2 * j] - lp[2 + 2 * j]) / (2e-3 * PRIOR_WIDTH[name])
        col = THETA.index(name)
        errs[name] = float(np.abs(D[:, :, col] - gt).max() / np.abs(gt).max())
    out["grad_max_rel_err"] = max(errs.values())
    out["grad_rel_err_by_param"] = errs
    out["grad_method"] = "adjoint (deb_adjoint), one seed per output"
    out["table_status_ok"] = bool((st == 0).all())
    torch.cuda.synchronize()
    print(json.dumps(out))


def run_accuracy(args):
    """Max relative error of the GPU result at the workload's tolerance
    against tight oracle solves on log-spaced k over the workload's range:
    P(k) against rtol 1e-8; for gradient workloads also d ln P / d theta
    against central differences over 1e-3 of each parameter's range of
    rtol 1e-9 oracle solves (error relative to each parameter's largest
    |d ln P / d theta|).  Prints one JSON line."""
    import torch

    import oracle
    import discoeb_gb300 as deb
    from discoeb_gb300 import tables as tb

    inp = make_inputs(args.workload, 0, 1)
    if inp.get("objective") == "loglike":
        return _accuracy_large(args, inp)
    dims = inp["dims"]
    k = np.geomspace(inp["kgrid"][0], inp["kgrid"][-1], args.accuracy_modes)
    out = {"workload": args.workload, "modes": int(k.size), "k": [float(x) for x in k],
           "aexp_out": inp["aexp"], "rtol": inp["rtol"]}
    p0 = inp["ps"][0]
    tab0, tau0 = tb.pack_cosmology(p0, dims["nqmax"]), tb.tau_of_a(p0, inp["aexp"])
    yt, st = oracle.solve(tab0, k, tau0, rtol=1e-8, atol=1e-8 * min(1.0, inp["atol"] / inp["rtol"]),
                          max_steps=2000000, step_to_outputs=inp["step_ts"], **dims)
    if inp["grad"]:
        from discoeb_gb300.gradient import THETA, _get, _with, evolve_backgrounds

        P, D, _ = deb.evolve_perturbations_grad(params=inp["params"][0], aexp_out=inp["aexp"], kmin=float(k[0]),
                                                kmax=float(k[-1]), num_k=k.size, rtol=inp["rtol"], atol=inp["atol"],
                                                max_steps=args.max_steps, backgrounds=[inp["bgs"][0]],
                                                step_to_outputs=inp["step_ts"], **dims)
        # reference derivative: central differences over 1e-3 of each parameter's range
        # (eps = 1e-4 theta is as small as 5e-6 for some draws, where differences of
        # adaptive solves are dominated by step-control noise) of rtol 1e-9 solves
        pert = inp["pert"][0]
        p = inp["params"][0]
        tp = []
        for (name, _, _, _) in pert:
            v, e = float(_get(p, name)), 1e-3 * PRIOR_WIDTH[name]
            tp += [_with(p, name, v + e), _with(p, name, v - e)]
        tb_ = evolve_backgrounds(tp)
        errs = {}
        for j, (name, _, _, _) in enumerate(pert):
            sols = []
            for q in tb_[2 * j:2 * j + 2]:
                yq, sq = oracle.solve(tb.pack_cosmology(q, dims["nqmax"]), k, tb.tau_of_a(q, inp["aexp"]), rtol=1e-9,
                                      atol=1e-9, max_steps=4000000, step_to_outputs=inp["step_ts"], **dims)
                if (sq[:, 0] != 0).any():
                    raise RuntimeError(f"reference solve failed for {name}")
                sols.append(yq)
            gt = (np.log(sols[0][..., 4] ** 2) - np.log(sols[1][..., 4] ** 2)) / (2e-3 * PRIOR_WIDTH[name])
            col = THETA.index(name)
            errs[name] = float(np.abs(D[:, :, col] - gt).max() / np.abs(gt).max())
        out["grad_max_rel_err"] = max(errs.values())
        out["grad_rel_err_by_param"] = errs
        out["step_to_outputs"] = inp["step_ts"]
    else:
        y = deb.solve(tab0[None], k, tau0[None], rtol=inp["rtol"], atol=inp["atol"], max_steps=args.max_steps,
                      step_to_outputs=inp["step_ts"], **dims)
        P = np.stack([deb.get_power(k=k, y=y[:, o, :], idx=4, param=p0) for o in range(y.shape[1])], axis=1)
    Pt = np.stack([deb.get_power(k=k, y=yt[:, o, :], idx=4, param=p0) for o in range(yt.shape[1])], axis=1)
    out["pk_max_rel_err"] = float((np.abs(P - Pt) / np.abs(Pt)).max())
    out["oracle_status_ok"] = bool((st[:, 0] == 0).all())
    torch.cuda.synchronize()
    print(json.dumps(out))


def run_reference(args):
    """The reference algorithm on the host cores (oracle/: Rodas5, PID, dense
    forward-mode Jacobian and dense LU in FP64, OpenMP over modes) on the
    workload's sample: every step times the same bounded run (each sampled
    mode for at most the same number of attempted steps) and scales its
    steps per second by the work of one cosmology solve, counted once on the
    sample (cpu_measure).  The reference's own JAX code is not installable
    here.  Prints the same metric, unit and config as the GPU arm."""
    import oracle

    world, rank, local = _dist()
    if rank != 0:
        return
    inp = make_inputs(args.workload, 0, 1)
    threads = os.cpu_count() or 1
    cm = cpu_measure(inp, budget_s=args.cpu_seconds, threads=threads)
    # each timed step: the same sample for fewer attempted steps per mode, about ref_step_seconds of work
    # (steps/s does not depend on how many of a mode's early steps are run: the dense LU costs the same
    # every step), so that warm-up + timed steps end within minutes
    cap = max(4, int(cm["dense"]["cap"] * min(1.0, args.ref_step_seconds / max(cm["dense"]["seconds"], 1e-3))))
    num_k = inp["num_k"]
    ks = np.asarray(inp["kgrid"])[np.arange(0, num_k, cm["stride"])]
    tab0, tau0 = inp["tables"][0], np.asarray(inp["tau"])[0]
    times, rates = [], []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        _, so = oracle.solve(tab0, ks, tau0, rtol=inp["rtol"], atol=inp["atol"], max_steps=int(cap), nthreads=threads,
                             step_to_outputs=inp["step_ts"], **inp["dims"])
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
            rates.append(int(so[:, 1].sum() + so[:, 2].sum()) / dt)
    rate = statistics.median(rates)
    v = rate / cm["work_steps_per_cosmology"]
    grad = inp.get("objective") == "loglike" or inp["grad"]
    unit = ("cosmology solves/s (P(k, a) + 8-parameter gradient)" if inp.get("objective") == "loglike" else
            "cosmology solves/s (P(k) + 8-parameter gradient)" if inp["grad"] else "cosmology solves/s")
    sample = (f"each step: {cm['sample_modes']} modes (every {cm['stride']}th of cosmology 0's {num_k}-point k-grid), "
              f"at most {cap} attempted steps each, {statistics.median(times):.2f} s, "
              f"{rate:.1f} steps/s; value = steps/s / {cm['work_steps_per_cosmology']:.4g} steps per cosmology solve"
              + (" (attempted + 6 x accepted: nominal solve + forward-mode gradient)" if grad else ""))
    out = {"impl": "reference", "metric": METRIC if inp.get("objective") == "loglike" else
           ("P(k)+dP/dtheta solves/s on 1 GB300, batched FP64 (8 parameters; structured Rodas5, tangents of the "
            "recorded step sequence)" if inp["grad"] else
            "P(k) forward solves/s on 1 GB300, batched FP64 structured Rodas5 (gradient not included)"),
           "value": v, "unit": unit, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": statistics.median(times) * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64",
           "data": "synthetic (seeded cosmology sample, the same tables as the GPU arm's cosmology 0)",
           "config": (loglike_config(args, inp) if inp.get("objective") == "loglike" else
                      {"workload": args.workload, "ncosmo_per_gpu": inp["ncosmo"], "num_k": inp["num_k"]}),
           "cpu_baseline": {"value": v, "unit": unit, "cores": threads, "kind": "port", "sample": sample,
                            "extrapolated": "steps/s measured on the sample, scaled by the counted work of one "
                                            "cosmology solve"},
           "cpu_structured": cm["structured"],
           "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "the reference's JAX path is not installable offline; the oracle (a CPU restatement of its "
                   "algorithm) is timed instead, on a bounded sample per step, scaled to cosmology solves"}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--max-steps", type=int, default=8192)
    ap.add_argument("--cpu-seconds", type=float, default=20.0)
    ap.add_argument("--ref-step-seconds", type=float, default=4.0,
                    help="reference arm: CPU seconds of each timed step's bounded sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--exec-mode", default="auto", choices=["auto", "lane", "warp"])
    ap.add_argument("--no-tune", dest="tune", action="store_false", help="skip the launch-shape autotuner")
    ap.add_argument("--launch", default=None,
                    help="fixed launch shape STAGE/MODES_PER_SM (e.g. global/8, shared/5) instead of the autotuner")
    ap.add_argument("--accuracy", action="store_true", help="print the error against tight oracle solves instead")
    ap.add_argument("--accuracy-modes", type=int, default=8)
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.accuracy:
        run_accuracy(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
