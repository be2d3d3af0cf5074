"""Pack a cosmology ``param`` dict into the flat FP64 blob the GPU receives.

Layout (one blob per cosmology, all cosmologies of a batch the same length;
the C side of the layout is ``include/discoeb_gb300.h``):

* ``HDR_LEN`` = 32 header doubles: the scalars the reference reads from
  ``param`` (``perturbations.py:113-371``, ``background.py:100-122``), the
  momentum-bin count, the seven spline sizes, the blob length and a magic
  number;
* seven natural cubic splines, each stored as ``x[n], y[n], S[n]``
  (``spline_interpolation.py:112-113`` fields ``_x_``, ``_y_``, ``_S_full_``)
  in the order of :data:`SPLINE_KEYS`;
* the ``nq`` momentum nodes q and kernel weights w of
  ``get_neutrino_momentum_bins`` (``background.py:13-44``);
* a derived section (offset in header slot 29): for each spline its
  per-interval polynomial coefficients and its knots rounded to FP32.

Splines are read duck-typed through ``_x_``, ``_y_``, ``_S_full_`` so a
``param`` produced by the reference's own ``evolve_background`` packs the
same way as one produced by :func:`background.evolve_background`.
"""
from __future__ import annotations

import numpy as np

from .background import get_neutrino_momentum_bins

HDR_LEN = 32
MAGIC = 20231103.0
SCALAR_KEYS = ("Omegam", "Omegab", "OmegaDE", "Omegak", "grhom", "grhog", "grhor", "Neff", "Nmnu",
               "amnu", "w_DE_0", "w_DE_a", "cs2_DE", "YHe", "H0", "taumin", "A_s", "n_s", "k_p")
H_NQ = 19
H_NSPL0 = 20
H_BLOBLEN = 27
H_MAGIC = 28
SPLINE_KEYS = ("xe_of_loga_spline", "cs2a_of_loga_spline", "logrhonu_of_loga_spline",
               "logpnu_of_loga_spline", "a_of_tau_spline", "tau_of_a_spline", "xe_of_tau_spline")
SP_TAU_OF_A = 5


def _arr(x):
    if hasattr(x, "__array__"):
        return np.asarray(x, dtype=np.float64)
    return np.asarray(x, dtype=np.float64)


H_DERIVED = 29   # offset of the derived section (polynomial coefficients, FP32 knots)


def blob_length(spline_sizes, nq: int) -> int:
    return HDR_LEN + 3 * int(sum(spline_sizes)) + 2 * nq + derived_length(spline_sizes)


def derived_length(spline_sizes) -> int:
    """Per spline: 4 (n-1) polynomial coefficients + n FP32 knots packed in ceil(n/2) doubles."""
    return int(sum(4 * (n - 1) + (n + 1) // 2 for n in spline_sizes))


def spline_derived(x, y, S):
    """Per-interval coefficients of p(u) = c0 + u (c1 + u (c2 + u c3)), u = x - x_i.

    The same natural cubic as the A/B form of spline_interpolation.py:150-152
    (c0 = y_i, c1 = (y_{i+1}-y_i)/h - h (S_{i+1} + 2 S_i)/6, c2 = S_i/2,
    c3 = (S_{i+1}-S_i)/(6h), spline_interpolation.py:94-101), so evaluation
    needs no division; plus the knots rounded to FP32 for a fast search.
    """
    h = x[1:] - x[:-1]
    c = np.empty((x.shape[0] - 1, 4))
    c[:, 0] = y[:-1]
    c[:, 1] = (y[1:] - y[:-1]) / h - h * (S[1:] + 2.0 * S[:-1]) / 6.0
    c[:, 2] = S[:-1] / 2.0
    c[:, 3] = (S[1:] - S[:-1]) / (6.0 * h)
    xf = x.astype(np.float32)
    if xf.shape[0] % 2:
        xf = np.concatenate([xf, np.array([np.inf], dtype=np.float32)])
    return c.ravel(), xf.view(np.float64)


def pack_cosmology(param: dict, nqmax: int) -> np.ndarray:
    """One cosmology's FP64 table blob."""
    scal = []
    for key in SCALAR_KEYS:
        if key == "k_p":
            scal.append(float(param.get("k_p", 0.05)))
        elif key == "Omegak":
            scal.append(float(param.get("Omegak", 0.0)))
        else:
            if key not in param:
                raise KeyError(f"param is missing '{key}' (run evolve_background first)")
            scal.append(float(np.asarray(param[key])))
    splines = []
    for key in SPLINE_KEYS:
        sp = param[key]
        x, y, S = _arr(sp._x_), _arr(sp._y_), _arr(sp._S_full_)
        if not (x.shape == y.shape == S.shape) or x.ndim != 1 or x.shape[0] < 2:
            raise ValueError(f"spline '{key}' has inconsistent arrays")
        splines.append((x, y, S))
    q, w = get_neutrino_momentum_bins(nqmax)
    sizes = [s[0].shape[0] for s in splines]
    L = blob_length(sizes, nqmax)
    b = np.zeros(L, dtype=np.float64)
    b[: len(scal)] = scal
    b[H_NQ] = nqmax
    b[H_NSPL0:H_NSPL0 + 7] = sizes
    b[H_BLOBLEN] = L
    b[H_MAGIC] = MAGIC
    p = HDR_LEN
    for (x, y, S) in splines:
        n = x.shape[0]
        b[p:p + n] = x
        b[p + n:p + 2 * n] = y
        b[p + 2 * n:p + 3 * n] = S
        p += 3 * n
    b[p:p + nqmax] = q
    b[p + nqmax:p + 2 * nqmax] = w
    p += 2 * nqmax
    b[H_DERIVED] = p
    for (x, y, S) in splines:
        cf, xf = spline_derived(x, y, S)
        b[p:p + cf.shape[0]] = cf
        p += cf.shape[0]
        b[p:p + xf.shape[0]] = xf
        p += xf.shape[0]
    assert p == L
    return b


def pack_batch(params, nqmax: int) -> np.ndarray:
    """[ncosmo, blob_len] table array; all cosmologies must share spline sizes."""
    blobs = [pack_cosmology(p, nqmax) for p in params]
    L = blobs[0].shape[0]
    for bb in blobs:
        if bb.shape[0] != L or not np.array_equal(bb[H_NSPL0:H_NSPL0 + 7], blobs[0][H_NSPL0:H_NSPL0 + 7]):
            raise ValueError("all cosmologies of one batch need identical table sizes")
    return np.ascontiguousarray(np.stack(blobs))


def tau_of_a(param: dict, aexp) -> np.ndarray:
    """Conformal times of the output scale factors (``perturbations.py:975``)."""
    from .spline import SplineInterpolation

    sp = param["tau_of_a_spline"]
    s = SplineInterpolation.__new__(SplineInterpolation)
    s._x_, s._y_, s._S_full_ = _arr(sp._x_), _arr(sp._y_), _arr(sp._S_full_)
    return s.evaluate(np.atleast_1d(np.asarray(aexp, dtype=np.float64)))


def tau_of_a_blob(blobs: np.ndarray, aexp) -> np.ndarray:
    """tau(a) at the scale factors ``aexp`` from the tau_of_a spline stored in
    each blob of ``blobs`` [nset, blob_len] (the A/B form of
    spline_interpolation.py:130-153); returns [nset, len(aexp)]."""
    from .spline import SplineInterpolation

    blobs = np.atleast_2d(blobs)
    aexp = np.atleast_1d(np.asarray(aexp, dtype=np.float64))
    out = np.empty((blobs.shape[0], aexp.shape[0]))
    for i, b in enumerate(blobs):
        sizes = b[H_NSPL0:H_NSPL0 + 7].astype(int)
        p = HDR_LEN + 3 * int(sizes[:SP_TAU_OF_A].sum())
        n = int(sizes[SP_TAU_OF_A])
        s = SplineInterpolation.__new__(SplineInterpolation)
        s._x_, s._y_, s._S_full_ = b[p:p + n], b[p + n:p + 2 * n], b[p + 2 * n:p + 3 * n]
        out[i] = s.evaluate(aexp)
    return out
