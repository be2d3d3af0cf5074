"""Launch-shape autotuner for the warp-per-mode kernel.

The kernel's speed depends on where a mode's eight Rodas5 stage vectors live
and on how many modes share an SM (``deb_launch_cfg`` in
``include/discoeb_gb300.h``): in shared memory a mode at nvar 323 takes 44 KB
and five fit per SM; with the stage vectors in an L2-resident global array it
takes 24 KB and up to eight fit (the register file's limit), at the price of
an L2 round trip per stage access.  Which wins depends on the hierarchy sizes
and on how much FP64 issue latency more resident warps hide, so it is
measured, not guessed: :func:`tune` times one launch per candidate shape on
the caller's own workload (CUDA events on the launching stream, after one
untimed launch) and keeps the fastest.  Choices are remembered per (device
name, hierarchy sizes, output count, solver) for the process and, when
``DISCOEB_GB300_TUNE_CACHE`` names a JSON file, across processes.
"""
from __future__ import annotations

import json
import os

from . import _native

# (stage vectors, modes-per-SM cap); 0 = as many as fit.  "all_global" keeps
# the whole mode state in L2-resident global memory: at nvar 1098 the shared
# part alone (72 KB) limits the other shapes to three modes per SM.
CANDIDATES = (("shared", 0), ("shared", 4), ("global", 0), ("global", 6), ("all_global", 0))

_chosen: dict = {}
_loaded = False


def _key(dims: _native.DebDims) -> str:
    import torch

    name = torch.cuda.get_device_name(torch.cuda.current_device())
    return "|".join(str(v) for v in (name, dims.lmaxg, dims.lmaxgp, dims.lmaxr, dims.lmaxnu, dims.nqmax, dims.nout,
                                     dims.return_full, dims.linear_solver))


def _cache_path():
    return os.environ.get("DISCOEB_GB300_TUNE_CACHE")


def _load():
    global _loaded
    if _loaded:
        return
    _loaded = True
    path = _cache_path()
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                for k, v in json.load(f).items():
                    _chosen.setdefault(k, (str(v[0]), int(v[1])))
        except (OSError, ValueError, TypeError, IndexError):
            pass


def _store():
    path = _cache_path()
    if not path:
        return
    try:
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        with open(path, "w") as f:
            json.dump({k: list(v) for k, v in _chosen.items()}, f, indent=1)
    except OSError:
        pass


def chosen(dims: _native.DebDims):
    """The tuned launch shape for these sizes, or None if not tuned yet."""
    if dims.exec_mode == _native.EXEC_MODES["lane"]:
        return None
    _load()
    return _chosen.get(_key(dims))


def remember(dims: _native.DebDims, launch) -> None:
    _load()
    _chosen[_key(dims)] = (str(launch[0]), int(launch[1]))
    _store()


def tune(dims: _native.DebDims, max_modes: int, launch_fn, candidates=CANDIDATES, stream=None):
    """Time ``launch_fn(plan, stream)`` (one kernel launch on ``plan``) for
    every candidate shape on a plan of ``max_modes`` modes; remember and
    return ``(best_shape, {shape: ms})``.  Synchronises the device."""
    import torch

    s = stream if stream is not None else torch.cuda.current_stream()
    times = {}
    for cand in candidates:
        try:
            plan = _native.Plan(dims, max_modes, cand)
        except RuntimeError:
            continue   # shape impossible for these sizes (e.g. too large for shared memory)
        info = plan.launch_info()
        shape = (info["stage_vectors"], info["modes_per_sm"])
        if shape in times:
            continue
        launch_fn(plan, s)   # untimed: first-touch of the plan's workspace
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        launch_fn(plan, s)
        e1.record(s)
        torch.cuda.synchronize()
        times[shape] = e0.elapsed_time(e1)
        del plan
    if not times:
        raise RuntimeError("autotune: no candidate launch shape could be planned")
    best = min(times, key=times.get)
    remember(dims, best)
    return best, times
