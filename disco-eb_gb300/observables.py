"""Observables on top of the perturbations, on the GPU.

Same keyword-only signatures and return values as the reference
(``src/discoeb/perturbations.py``):

* :func:`get_power_smoothed` -- ``:1126-1159`` (Savitzky-Golay smoothing of ln P);
* :func:`power_Kaiser` -- ``:1162-1199`` (anisotropic P(k, mu));
* :func:`power_multipoles` -- ``:1202-1224`` (P0, P2, P4);
* :func:`get_xi_from_P` -- ``:1065-1098`` (FFTLog correlation function).

The elementwise work and the FFTLog phase factors run in the CUDA library
(``deb_observables.cu``); the two FFTs of FFTLog use cuFFT through
``torch.fft``.  The Savitzky-Golay window is solved on the host (a (p+1) x w
least-squares problem, ``util.py:407-444``).  Inputs may be numpy arrays or
CUDA tensors; outputs follow the input container type.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from . import tables as _tables
from .perturbations import _torch, get_power


def _dev():
    torch = _torch()
    return torch.device("cuda", torch.cuda.current_device())


def _t(a):
    torch = _torch()
    return (a if torch.is_tensor(a) else torch.as_tensor(np.asarray(a, dtype=np.float64))).to(_dev(), torch.float64).contiguous()


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(_torch().cuda.current_stream().cuda_stream)


def _scalar_blob(param):
    """The A_s, n_s, k_p header of a table blob (all that get_power reads)."""
    hdr = np.zeros((1, _tables.HDR_LEN + 3 * 2 * 7 + 2), dtype=np.float64)
    hdr[0, 16] = float(param["A_s"])
    hdr[0, 17] = float(param["n_s"])
    hdr[0, 18] = float(param.get("k_p", 0.05))
    return hdr


def savgol_coeffs(window_length: int, polyorder: int) -> np.ndarray:
    """Savitzky-Golay smoothing window: the minimum-norm solution c of
    A c = e_0 with A[p, j] = x_j^p, x = (w-1)/2 .. -(w-1)/2 (``util.py:427-442``)."""
    halflen, rem = divmod(window_length, 2)
    pos = halflen - 0.5 if rem == 0 else halflen
    x = np.arange(-pos, window_length - pos, dtype=np.float64)[::-1]
    A = x[None, :] ** np.arange(polyorder + 1)[:, None]
    Y = np.zeros(polyorder + 1)
    Y[0] = 1.0
    return np.linalg.lstsq(A, Y, rcond=None)[0]


def smoothing_window(k, dlogk: float) -> int:
    """Odd window length covering dlogk in ln k (``perturbations.py:1148-1149``)."""
    kk = np.asarray(k.cpu() if hasattr(k, "cpu") else k, dtype=np.float64)
    w = int(round(dlogk / (np.log(kk[1]) - np.log(kk[0]))))
    return w + (w + 1) % 2


def _savgol_log(P, window: int):
    """exp(SG(ln P)) along the last axis with the reference's boundary copies."""
    torch = _torch()
    Pt = _t(P)
    n = int(Pt.shape[-1])
    rows = Pt.reshape(-1, n).contiguous()
    c = _t(savgol_coeffs(window, 3))
    out = torch.empty_like(rows)
    _native.check(_native.load().deb_savgol_log(_ptr(rows), int(rows.shape[0]), n, _ptr(c), int(window), _ptr(out),
                                                _stream()), "deb_savgol_log")
    return out.reshape(Pt.shape)


def get_power_smoothed(*, k, y, dlogk: float, idx: int, param: dict):
    """Savitzky-Golay smoothed P(k) (``perturbations.py:1126-1159``); ``y`` is
    [num_k, 20] (one output time) or [num_k, nout, 20] (smoothed along k per output)."""
    torch = _torch()
    w = smoothing_window(k, dlogk)
    P = get_power(k=k, y=y, idx=idx, param=param)
    Pt = _t(P)
    if Pt.dim() == 1:
        out = _savgol_log(Pt, w)
    else:
        out = _savgol_log(Pt.transpose(0, 1).contiguous(), w).transpose(0, 1).contiguous()
    return out if torch.is_tensor(y) else out.cpu().numpy()


def _fields(kmodes, y, param):
    """delta = A y[:, 4] and theta = A y[:, 5] for one output time."""
    torch = _torch()
    yt = _t(y)
    kt = _t(kmodes)
    if yt.dim() != 2:
        raise ValueError("y must be [num_k, nfields] (one output time)")
    blob = _t(_scalar_blob(param))
    nmode = int(kt.shape[0])
    d = torch.empty(nmode, dtype=torch.float64, device=_dev())
    th = torch.empty_like(d)
    _native.check(_native.load().deb_density_velocity(_ptr(blob), 1, int(blob.shape[1]), _ptr(kt), None, nmode, _ptr(yt),
                                                      int(yt.shape[1]), _ptr(d), _ptr(th), _stream()),
                  "deb_density_velocity")
    return d, th


def power_Kaiser(*, y, kmodes, bias: float, mu_sampling: bool = True, smooth_dlogk: float = None, nmu: int,
                 param: dict):
    """Anisotropic P(k, mu) = (b delta - mu^2 theta)^2 (``perturbations.py:1162-1199``).
    Returns (Pkmu [num_k, nmu], mu [nmu])."""
    torch = _torch()
    mu = np.linspace(-1.0, 1.0, nmu) if mu_sampling else np.cos(np.linspace(0.0, np.pi, nmu))
    if smooth_dlogk is None:
        d, th = _fields(kmodes, y, param)
    else:
        d = torch.sqrt(_t(get_power_smoothed(y=y, k=kmodes, dlogk=smooth_dlogk, idx=4, param=param)))
        th = -torch.sqrt(_t(get_power_smoothed(y=y, k=kmodes, dlogk=smooth_dlogk, idx=5, param=param)))
    mut = _t(mu)
    nmode = int(d.shape[0])
    out = torch.empty((nmode, nmu), dtype=torch.float64, device=_dev())
    _native.check(_native.load().deb_power_kaiser(_ptr(d.contiguous()), _ptr(th.contiguous()), nmode, _ptr(mut), int(nmu),
                                                  float(bias), _ptr(out), _stream()), "deb_power_kaiser")
    return (out, mut) if torch.is_tensor(y) else (out.cpu().numpy(), mu)


def power_multipoles(*, y, kmodes, b: float, param):
    """Redshift-space multipoles (P0, P2, P4) of the Kaiser spectrum
    (``perturbations.py:1202-1224``); ``y`` is [num_k, 20] or [num_k, nout, 20]."""
    torch = _torch()
    yt = _t(y)
    kt = _t(kmodes)
    nmode = int(kt.shape[0])
    shape = tuple(yt.shape[:-1])
    nout = int(np.prod(shape[1:])) if len(shape) > 1 else 1
    blob = _t(_scalar_blob(param))
    outs = [torch.empty((nmode, nout), dtype=torch.float64, device=_dev()) for _ in range(3)]
    _native.check(_native.load().deb_power_multipoles(_ptr(blob), 1, int(blob.shape[1]), _ptr(kt), None, nmode, nout,
                                                      _ptr(yt), int(yt.shape[-1]), float(b), _ptr(outs[0]), _ptr(outs[1]),
                                                      _ptr(outs[2]), _stream()), "deb_power_multipoles")
    res = tuple(o.reshape(shape) for o in outs)
    return res if torch.is_tensor(y) else tuple(r.cpu().numpy() for r in res)


def get_xi_from_P(*, k, Pk, N: int = None, ell: int = 0):
    """Correlation function multipole by FFTLog (``perturbations.py:1065-1098``):
    xi_ell(r) at r = 2 pi / k, returned in increasing r as (xi, r).  ``k`` must
    be log-spaced; like the reference, ``N`` is taken from ``len(k)``."""
    torch = _torch()
    kt, Pt = _t(k), _t(Pk)
    N = int(kt.shape[0])
    if N % 2:
        raise ValueError("FFTLog needs an even number of k (the inverse real FFT returns 2 (N // 2) points)")
    L = float(torch.log(kt[N - 1] / kt[0]))
    fP = torch.fft.rfft(Pt * kt ** 1.5)
    nf = int(fP.shape[0])
    ph = torch.empty(2 * nf, dtype=torch.float64, device=_dev())
    _native.check(_native.load().deb_fftlog_phase(nf, L, int(ell), _ptr(ph), _stream()), "deb_fftlog_phase")
    fP = fP * torch.view_as_complex(ph.reshape(nf, 2))
    r = 2.0 * np.pi / kt
    # 1j**ell is real for even ell, imaginary (no real part) for odd ell
    sign = 0.0 if ell % 2 else (-1.0) ** (ell // 2)
    xi = sign * torch.fft.irfft(fP, n=N) / (2.0 * np.pi * r) ** 1.5
    xi, r = torch.flip(xi, [0]), torch.flip(r, [0])
    return (xi, r) if torch.is_tensor(Pk) else (xi.cpu().numpy(), r.cpu().numpy())
