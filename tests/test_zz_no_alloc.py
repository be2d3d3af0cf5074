"""The allocation-free entry point deb_forward_static against deb_forward.

Callers that cannot allocate device memory -- code running inside a host
framework that owns every device buffer, so neither it nor this library may
call cudaMalloc -- use deb_forward_static instead of a plan.  Its scratch is a
fixed array compiled into the library.  This test calls it through the C ABI
twice in a row (the second call reuses the array the first one left behind)
and compares each result with the planned entry point deb_forward, at the
tolerance of the other GPU parity tests.  It is collected last so that a run
stopping at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LCDM = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=8, nqmax=3)


def _c(t):
    return ctypes.c_void_p(t.data_ptr())


def test_static_entry_point_matches_planned_entry_point():
    import torch

    import discoeb_gb300.background as bg
    import discoeb_gb300.tables as tb
    from discoeb_gb300 import _native
    from discoeb_gb300 import perturbations as pt
    from discoeb_gb300.workloads import lcdm_massless_param

    torch.cuda.set_device(0)
    p = bg.evolve_background(param=lcdm_massless_param())
    k = np.geomspace(1e-4, 1.0, 24)
    a_out = [0.5, 1.0]
    blob = tb.pack_cosmology(p, 3)
    tau = tb.tau_of_a(p, a_out)
    ref = pt.solve(blob[None], k, tau[None], rtol=1e-3, atol=1e-6, exec_mode="warp", **LCDM)

    L = _native.load()
    dev = torch.device("cuda", 0)
    d_tab = torch.as_tensor(blob[None]).to(dev)
    d_k = torch.as_tensor(k).to(dev)
    d_tau = torch.as_tensor(tau[None]).to(dev)
    d_y = torch.empty((k.size, len(a_out), 20), dtype=torch.float64, device=dev)
    d_st = torch.empty(k.size, dtype=torch.int32, device=dev)
    d_steps = torch.empty((k.size, 2), dtype=torch.int32, device=dev)
    dims = pt._dims(nout=len(a_out), return_full=False, linear_solver="structured", **LCDM)
    cfg = pt._cfg(1e-3, 1e-6, 0.25, 0.80, 0.0, 20.0, 0.3, 2048)
    stream = torch.cuda.current_stream()
    for _ in range(2):
        d_y.fill_(0.0)
        d_st.fill_(-7)
        rc = L.deb_forward_static(ctypes.byref(dims), _c(d_tab), 1, blob.shape[0], _c(d_k), None, k.size, _c(d_tau),
                                  ctypes.byref(cfg), _c(d_y), _c(d_st), _c(d_steps), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.deb_error_string(rc)
        torch.cuda.synchronize()
        assert (d_st.cpu().numpy() == 0).all()
        y = d_y.cpu().numpy()
        np.testing.assert_allclose(y[:, :, 4] ** 2, ref[:, :, 4] ** 2, rtol=1e-6)
        for f in (6, 8, 10):
            np.testing.assert_allclose(y[:, :, f], ref[:, :, f], rtol=1e-6, atol=1e-9 * np.abs(ref[:, :, f]).max())


def _static_vs_planned(param, lm, k, a_out, rtol, return_full=False, step_to_outputs=False, max_steps=4096):
    """deb_forward_static twice in a row against the planned deb_forward."""
    import torch

    import discoeb_gb300.background as bg
    import discoeb_gb300.tables as tb
    from discoeb_gb300 import _native
    from discoeb_gb300 import perturbations as pt

    torch.cuda.set_device(0)
    p = bg.evolve_background(param=param)
    blob = tb.pack_cosmology(p, lm["nqmax"])
    tau = tb.tau_of_a(p, a_out)
    cfg = pt._cfg(rtol, rtol, 0.25, 0.80, 0.0, 20.0, 0.3, max_steps, step_to_outputs=step_to_outputs)
    # the planned launch in the static entry's shape (every per-mode vector in
    # global memory): the same instructions, so the same accept / reject
    # decisions at any tolerance
    prob = pt.DeviceProblem(blob[None], k, tau[None], exec_mode="warp", return_full=return_full, **lm)
    prob.plan = pt.get_plan(prob.dims, prob.nmode, ("all_global", 8))
    prob.launch(cfg)
    ref = prob.y.cpu().numpy()
    assert (prob.status.cpu().numpy() == 0).all()
    L = _native.load()
    dev = torch.device("cuda", 0)
    d_tab = torch.as_tensor(blob[None]).to(dev)
    d_k = torch.as_tensor(k).to(dev)
    d_tau = torch.as_tensor(tau[None]).to(dev)
    osz = pt.nvar(**lm) if return_full else 20
    d_y = torch.empty((k.size, len(a_out), osz), dtype=torch.float64, device=dev)
    d_st = torch.empty(k.size, dtype=torch.int32, device=dev)
    d_steps = torch.empty((k.size, 2), dtype=torch.int32, device=dev)
    dims = pt._dims(nout=len(a_out), return_full=return_full, linear_solver="structured", **lm)
    stream = torch.cuda.current_stream()
    for _ in range(2):
        d_y.fill_(0.0)
        d_st.fill_(-7)
        rc = L.deb_forward_static(ctypes.byref(dims), _c(d_tab), 1, blob.shape[0], _c(d_k), None, k.size, _c(d_tau),
                                  ctypes.byref(cfg), _c(d_y), _c(d_st), _c(d_steps), ctypes.c_void_p(stream.cuda_stream))
        assert rc == 0, L.deb_error_string(rc)
        torch.cuda.synchronize()
        assert (d_st.cpu().numpy() == 0).all()
        y = d_y.cpu().numpy()
        scale = np.abs(ref).max(axis=(0, 1), keepdims=True)
        bad = np.abs(y - ref) > 1e-6 * np.abs(ref) + 1e-9 * scale
        assert not bad.any(), (int(bad.sum()), np.argwhere(bad)[:5].tolist())


def test_static_entry_point_with_more_modes_than_array_slots():
    """nvar 323: one mode's state is 44 KB, so the 16 MiB array holds 380
    modes in flight; 420 modes make the warps take further modes from the
    work queue inside the same array."""
    from discoeb_gb300.workloads import fiducial_mnu_param

    lm = dict(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=17, nqmax=15)
    _static_vs_planned(fiducial_mnu_param(), lm, np.geomspace(1e-4, 1.0, 420), [1.0], 1e-3)


def test_static_entry_point_full_state_with_steps_on_outputs():
    """return_full (the whole state at every output) and steps landing on
    the output times, against the planned entry point."""
    from discoeb_gb300.workloads import lcdm_massless_param

    _static_vs_planned(lcdm_massless_param(), LCDM, np.geomspace(1e-4, 1.0, 16), [0.25, 0.5, 1.0], 1e-4,
                       return_full=True, step_to_outputs=True)


def test_static_entry_point_rejects_state_beyond_the_array():
    """A mode whose state exceeds DEB_STATIC_SCRATCH_BYTES is refused before any launch."""
    from discoeb_gb300 import _native
    from discoeb_gb300 import perturbations as pt

    L = _native.load()
    # nvar = 202 053: 16 vectors of it alone are 25.9 MB > 16 MiB
    dims = pt._dims(lmaxg=12, lmaxgp=12, lmaxr=17, lmaxnu=100, nqmax=2000, nout=1, return_full=False,
                    linear_solver="structured")
    cfg = pt._cfg(1e-3, 1e-6, 0.25, 0.80, 0.0, 20.0, 0.3, 2048)
    rc = L.deb_forward_static(ctypes.byref(dims), None, 1, 1000, None, None, 1, None, ctypes.byref(cfg), None, None,
                              None, None)
    assert rc == -6 and b"static scratch" in L.deb_error_string(rc)
