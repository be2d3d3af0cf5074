"""ctypes binding of the C ABI in ``include/discoeb_gb300.h``.

The CUDA library is the only compute path: if it is missing or no CUDA
device is present, every call raises.  There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libdiscoeb_gb300.so")

DEB_SOLVE_STRUCTURED = 0
DEB_SOLVE_DENSE = 1
EXEC_MODES = {"auto": 0, "lane": 1, "warp": 2}
MODE_STATUS = {0: "OK", 1: "MAX_STEPS", 2: "DT_UNDERFLOW", 3: "NONFINITE", 4: "BAD_INPUT"}


class DebDims(ctypes.Structure):
    _fields_ = [("lmaxg", ctypes.c_int), ("lmaxgp", ctypes.c_int), ("lmaxr", ctypes.c_int), ("lmaxnu", ctypes.c_int),
                ("nqmax", ctypes.c_int), ("nout", ctypes.c_int), ("return_full", ctypes.c_int),
                ("linear_solver", ctypes.c_int), ("exec_mode", ctypes.c_int)]


class DebLaunchCfg(ctypes.Structure):
    _fields_ = [("stage_vectors", ctypes.c_int), ("modes_per_sm", ctypes.c_int)]


STAGE_VECTORS = {"auto": 0, "shared": 1, "global": 2, "all_global": 3}


class DebSolverCfg(ctypes.Structure):
    _fields_ = [("rtol", ctypes.c_double), ("atol", ctypes.c_double), ("pcoeff", ctypes.c_double),
                ("icoeff", ctypes.c_double), ("dcoeff", ctypes.c_double), ("factormax", ctypes.c_double),
                ("factormin", ctypes.c_double), ("safety", ctypes.c_double), ("error_order", ctypes.c_double),
                ("max_steps", ctypes.c_int), ("hist_on_reject", ctypes.c_int), ("step_to_outputs", ctypes.c_int)]


_lib = None
EXPORTS = ("deb_nvar", "deb_plan_create", "deb_plan_create_ex", "deb_plan_launch_info", "deb_plan_workspace_bytes",
           "deb_plan_set_order", "deb_forward", "deb_forward_static", "deb_tables_blob_len", "deb_evolve_background",
           "deb_evolve_background_host", "deb_evolve_background_frozen", "deb_evolve_background_frozen_host",
           "deb_tau_of_a", "deb_plan_create_grouped", "deb_forward_grouped",
           "deb_forward_record", "deb_forward_record_ckpt", "deb_plan_create_adjoint", "deb_adjoint", "deb_replay",
           "deb_get_power", "deb_power_multipoles", "deb_density_velocity",
           "deb_power_kaiser", "deb_savgol_log", "deb_fftlog_phase",
           "deb_plan_destroy", "deb_measure_fp64_peak", "deb_error_string", "deb_version")


def load(path: str | None = None):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"CUDA library not built: {p} is missing (run __graft_entry__.build() "
                           f"or python disco-eb_gb300/build.py)")
    L = ctypes.CDLL(p)
    vp = ctypes.c_void_p
    L.deb_nvar.argtypes = [ctypes.POINTER(DebDims)]
    L.deb_plan_create.argtypes = [ctypes.POINTER(DebDims), ctypes.c_int, ctypes.POINTER(vp)]
    L.deb_plan_create_ex.argtypes = [ctypes.POINTER(DebDims), ctypes.c_int, ctypes.POINTER(DebLaunchCfg),
                                     ctypes.POINTER(vp)]
    L.deb_plan_launch_info.argtypes = [vp, ctypes.POINTER(DebLaunchCfg), ctypes.POINTER(ctypes.c_int)]
    L.deb_plan_workspace_bytes.argtypes = [vp, ctypes.POINTER(ctypes.c_size_t)]
    L.deb_plan_set_order.argtypes = [vp, vp, ctypes.c_int]
    L.deb_forward.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, vp,
                              ctypes.POINTER(DebSolverCfg), vp, vp, vp, vp]
    L.deb_forward_static.argtypes = [ctypes.POINTER(DebDims), vp, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, vp,
                                     ctypes.POINTER(DebSolverCfg), vp, vp, vp, vp]
    L.deb_forward_record.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, vp,
                                     ctypes.POINTER(DebSolverCfg), vp, vp, vp, vp, ctypes.c_int, vp, vp]
    L.deb_forward_record_ckpt.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, vp,
                                          ctypes.POINTER(DebSolverCfg), vp, vp, vp, vp, ctypes.c_int, vp, vp,
                                          ctypes.c_int, vp, vp, vp, vp]
    L.deb_plan_create_adjoint.argtypes = [ctypes.POINTER(DebDims), ctypes.c_int, ctypes.c_int, ctypes.POINTER(vp)]
    L.deb_adjoint.argtypes = [vp, vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, vp, ctypes.c_int, vp, vp,
                              vp, ctypes.c_int, vp, vp, ctypes.c_int, vp, vp, vp, ctypes.c_int, vp, vp, vp]
    L.deb_replay.argtypes = [vp, vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, vp,
                             ctypes.POINTER(DebSolverCfg), vp, ctypes.c_int, vp, vp, vp, vp]
    L.deb_get_power.argtypes = [vp, ctypes.c_int, ctypes.c_int, vp, vp, ctypes.c_int, ctypes.c_int, vp, ctypes.c_int,
                                ctypes.c_int, vp, vp]
    ci, cd = ctypes.c_int, ctypes.c_double
    L.deb_power_multipoles.argtypes = [vp, ci, ci, vp, vp, ci, ci, vp, ci, cd, vp, vp, vp, vp]
    L.deb_density_velocity.argtypes = [vp, ci, ci, vp, vp, ci, vp, ci, vp, vp, vp]
    L.deb_power_kaiser.argtypes = [vp, vp, ci, vp, ci, cd, vp, vp]
    L.deb_savgol_log.argtypes = [vp, ci, ci, vp, ci, vp, vp]
    L.deb_fftlog_phase.argtypes = [ci, cd, ci, vp, vp]
    L.deb_plan_create_grouped.argtypes = [ctypes.POINTER(DebDims), ci, ci, ctypes.POINTER(vp)]
    L.deb_forward_grouped.argtypes = [vp, vp, ci, ci, vp, vp, ci, vp, ctypes.POINTER(DebSolverCfg), vp, vp, vp, vp]
    L.deb_tables_blob_len.argtypes = [ci, ci, ci]
    L.deb_evolve_background.argtypes = [vp, vp, ci, vp, vp, vp, ci, vp, vp]
    L.deb_tau_of_a.argtypes = [vp, ci, ci, vp, ci, vp, vp]
    L.deb_evolve_background_host.argtypes = [vp, vp, ci, vp, vp, vp, ci, vp, ci]
    L.deb_evolve_background_frozen.argtypes = [vp, vp, ci, vp, vp, vp, vp, ci, vp, ci, vp, vp]
    L.deb_evolve_background_frozen_host.argtypes = [vp, vp, ci, vp, vp, vp, vp, ci, vp, ci, vp, ci]
    L.deb_plan_destroy.argtypes = [vp]
    L.deb_plan_destroy.restype = None
    L.deb_measure_fp64_peak.argtypes = [ctypes.POINTER(ctypes.c_double), vp]
    L.deb_error_string.argtypes = [ctypes.c_int]
    L.deb_error_string.restype = ctypes.c_char_p
    _lib = L
    return L


def check(rc: int, what: str):
    if rc != 0:
        msg = load().deb_error_string(rc).decode()
        raise RuntimeError(f"{what} failed: {msg} ({rc})")


class Plan:
    """Owns one deb_plan (device workspace sized for max_modes)."""

    def __init__(self, dims: DebDims, max_modes: int, launch: tuple[str, int] | None = None, batch_size: int = 0,
                 adjoint_seg_cap: int = 0):
        """``launch`` = (stage vectors "auto" | "shared" | "global", modes per SM cap or 0);
        ``batch_size`` > 0 makes a grouped plan (deb_plan_create_grouped);
        ``adjoint_seg_cap`` > 0 an adjoint plan (deb_plan_create_adjoint)
        for ``max_modes`` items and checkpoint strides up to that value."""
        self.dims = dims
        self.max_modes = max_modes
        self.batch_size = batch_size
        self.ptr = ctypes.c_void_p()
        if adjoint_seg_cap > 0:
            check(load().deb_plan_create_adjoint(ctypes.byref(dims), int(max_modes), int(adjoint_seg_cap),
                                                 ctypes.byref(self.ptr)), "deb_plan_create_adjoint")
        elif batch_size > 0:
            check(load().deb_plan_create_grouped(ctypes.byref(dims), int(max_modes), int(batch_size),
                                                 ctypes.byref(self.ptr)), "deb_plan_create_grouped")
        elif launch is None:
            check(load().deb_plan_create(ctypes.byref(dims), int(max_modes), ctypes.byref(self.ptr)), "deb_plan_create")
        else:
            lc = DebLaunchCfg(STAGE_VECTORS[launch[0]], int(launch[1]))
            check(load().deb_plan_create_ex(ctypes.byref(dims), int(max_modes), ctypes.byref(lc), ctypes.byref(self.ptr)),
                  "deb_plan_create_ex")

    def launch_info(self) -> dict:
        """Resolved launch shape: stage vector placement, modes per SM, modes in flight."""
        lc, nf = DebLaunchCfg(), ctypes.c_int()
        check(load().deb_plan_launch_info(self.ptr, ctypes.byref(lc), ctypes.byref(nf)), "deb_plan_launch_info")
        names = {v: k for k, v in STAGE_VECTORS.items()}
        return {"stage_vectors": names[lc.stage_vectors], "modes_per_sm": int(lc.modes_per_sm),
                "modes_in_flight": int(nf.value)}

    def workspace_bytes(self) -> int:
        b = ctypes.c_size_t()
        check(load().deb_plan_workspace_bytes(self.ptr, ctypes.byref(b)), "deb_plan_workspace_bytes")
        return int(b.value)

    def __del__(self):
        try:
            if self.ptr:
                load().deb_plan_destroy(self.ptr)
        except Exception:
            pass


def measure_fp64_peak(stream: int = 0) -> float:
    v = ctypes.c_double()
    check(load().deb_measure_fp64_peak(ctypes.byref(v), ctypes.c_void_p(stream)), "deb_measure_fp64_peak")
    return float(v.value)
