"""Twiss parameters of a tracked beam from its moments.

The reference's track() calls get_envelope after every step
(ocelot/cpbd/track.py:466-486, ocelot/cpbd/beam/analysis.py:27-226).  On the
device the moments are taken by ``sc_moments`` (one pass over the rows of
rparticles, two with bounds) into a table with one slot per step; this module
turns a slot into a ``Twiss`` with get_envelope's derived quantities:
emittances sqrt(<xx><px px> - <x px>^2), normalised by gamma beta of the beam
energy, beta = <xx>/emit, alpha = -<x px>/emit, and the two eigen-emittances of
the 4D (x, y, px, py) second-moment matrix Sigma -- the moduli of the
eigenvalues of Sigma.S, S the symplectic form, which are +-i e1 and +-i e2;
eigemit_1 is the larger, eigemit_2 the smaller.
"""
from __future__ import annotations

import numpy as np

from . import _native as N
from .globals import m_e_GeV

MOMENTS = N.SC_MOMENTS  # count, tau mean/std (bounds), 6 means, 12 central moments
_MEANS = ("x", "y", "px", "py", "tau", "p")
_SECOND = ("xx", "xpx", "pxpx", "yy", "ypy", "pypy", "tautau", "xy", "pxpy", "xpy", "ypx", "pp")
_S4 = np.array([[0, 0, 1, 0], [0, 0, 0, 1], [-1, 0, 0, 0], [0, -1, 0, 0]], dtype=np.float64)


class Twiss:
    """The attributes get_envelope fills in the reference's Twiss
    (ocelot/cpbd/beam/core.py:16-75); dispersion and phase advance stay 0."""

    def __init__(self):
        self.E = 0.0
        self.q = 0.0
        self.s = 0.0
        self.emit_x = self.emit_y = self.emit_xn = self.emit_yn = 0.0
        self.eigemit_1 = self.eigemit_2 = 0.0
        self.beta_x = self.beta_y = self.alpha_x = self.alpha_y = 0.0
        self.Dx = self.Dy = self.Dxp = self.Dyp = 0.0
        self.mux = self.muy = 0.0
        self.xp = self.yp = 0.0
        for k in _MEANS + _SECOND:
            setattr(self, k, 0.0)
        self.id = ""

    @property
    def gamma_x(self):
        return (1 + self.alpha_x ** 2) / self.beta_x if self.beta_x != 0 else 0

    @property
    def gamma_y(self):
        return (1 + self.alpha_y ** 2) / self.beta_y if self.beta_y != 0 else 0

    def __repr__(self):
        return (f"Twiss(s={self.s}, E={self.E}, emit_x={self.emit_x}, emit_y={self.emit_y}, beta_x={self.beta_x}, "
                f"beta_y={self.beta_y}, alpha_x={self.alpha_x}, alpha_y={self.alpha_y})")


def eigen_emittances(tws) -> tuple[float, float]:
    sigma = np.array([[tws.xx, tws.xy, tws.xpx, tws.xpy],
                      [tws.xy, tws.yy, tws.ypx, tws.ypy],
                      [tws.xpx, tws.ypx, tws.pxpx, tws.pxpy],
                      [tws.xpy, tws.ypy, tws.pxpy, tws.pypy]])
    if not np.all(np.isfinite(sigma)):
        return float("nan"), float("nan")
    w = np.sort(np.abs(np.linalg.eigvals(sigma @ _S4).imag))
    # w = [e2, e2, e1, e1]
    return float(0.5 * (w[2] + w[3])), float(0.5 * (w[0] + w[1]))


def twiss_from_moments(m, energy: float, charge: float, s: float = 0.0) -> Twiss:
    """A Twiss from one slot of the sc_moments table (get_envelope's steps
    after the moments, analysis.py:83-226)."""
    m = np.asarray(m, dtype=np.float64)
    tws = Twiss()
    tws.E = energy
    tws.q = charge
    tws.s = s
    tws.p = float(m[8])
    if not m[0] >= 3:
        return tws     # fewer than 3 particles: E, q and p only, as the reference
    for k, v in zip(_MEANS, m[3:9]):
        setattr(tws, k, float(v))
    for k, v in zip(_SECOND, m[9:21]):
        setattr(tws, k, float(v))
    tws.emit_x = float(np.sqrt(tws.xx * tws.pxpx - tws.xpx ** 2))
    tws.emit_y = float(np.sqrt(tws.yy * tws.pypy - tws.ypy ** 2))
    relgamma = energy / m_e_GeV
    relbeta = np.sqrt(1 - relgamma ** -2) if relgamma != 0 else 1.
    tws.emit_xn = float(tws.emit_x * relgamma * relbeta)
    tws.emit_yn = float(tws.emit_y * relgamma * relbeta)
    tws.eigemit_1, tws.eigemit_2 = eigen_emittances(tws)
    with np.errstate(divide="ignore", invalid="ignore"):
        tws.beta_x = float(np.float64(tws.xx) / tws.emit_x)
        tws.beta_y = float(np.float64(tws.yy) / tws.emit_y)
        tws.alpha_x = float(-np.float64(tws.xpx) / tws.emit_x)
        tws.alpha_y = float(-np.float64(tws.ypy) / tws.emit_y)
    return tws


def moments_numpy(rp: np.ndarray, bounds=None) -> np.ndarray:
    """One slot of the moments table computed on the host with get_envelope's
    two numpy passes (means, then central moments): a check of the device
    table, which takes shifted sums in one pass."""
    rp = np.asarray(rp, dtype=np.float64)
    out = np.zeros(MOMENTS)
    tau = rp[4]
    sel = np.ones(rp.shape[1], dtype=bool)
    if bounds is not None:
        out[1] = np.mean(tau)
        out[2] = np.std(tau)
        sel = (out[1] + out[2] * bounds[0] <= tau) & (tau <= out[1] + out[2] * bounds[1])
    x, px, y, py, t, p = (rp[r][sel] for r in range(6))
    f = 1. - p - 0.5 * p * p + 0.5 * px * px + 0.5 * py * py
    px, py = px * f, py * f
    out[0] = x.size
    cols = (x, y, px, py, t, p)
    means = [np.mean(c) for c in cols]
    out[3:9] = means
    d = [c - mu for c, mu in zip(cols, means)]
    dx, dy, dpx, dpy, dt, dp = d
    out[9:21] = [np.mean(a * b) for a, b in ((dx, dx), (dx, dpx), (dpx, dpx), (dy, dy), (dy, dpy), (dpy, dpy),
                                              (dt, dt), (dx, dy), (dpx, dpy), (dx, dpy), (dy, dpx), (dp, dp))]
    return out


def get_envelope(p_array, tws_i=None, bounds=None, slice=None, auto_disp=False):
    """Twiss of a beam from its moments, taken on the GPU: the reference's
    get_envelope (ocelot/cpbd/beam/analysis.py:27-226) for a ParticleArray or
    DeviceParticleArray (host particles are copied to the device once).
    Dispersion correction (``tws_i``, ``auto_disp``) and the maximum-current
    reference slice (``slice``) are not supported."""
    import ctypes as C

    import torch

    from . import _native as N
    from .beam import DeviceParticleArray
    if tws_i is not None or auto_disp or slice is not None:
        raise NotImplementedError("get_envelope on the device: no dispersion correction and no reference slice")
    if isinstance(p_array, DeviceParticleArray):
        rp, q = p_array.rparticles, p_array.q_array
        dev = rp.device
    else:
        if not torch.cuda.is_available():
            raise N.NativeLibraryError("ocelot_gb300 needs a CUDA device; there is no CPU fallback")
        dev = torch.device("cuda", torch.cuda.current_device())
        rp = torch.from_numpy(np.ascontiguousarray(p_array.rparticles, dtype=np.float64)).to(dev)
        q = np.asarray(p_array.q_array, dtype=np.float64)
    n = int(rp.shape[1])
    if n < 1:
        raise ValueError("zero-size array")
    if rp.dtype != torch.float64 or rp.stride(1) != 1:
        raise ValueError("rparticles must be float64 with contiguous rows")
    lib = N.lib()
    out = torch.zeros((1, MOMENTS), dtype=torch.float64, device=dev)
    scratch = torch.zeros(int(lib.sc_moments_scratch_bytes()), dtype=torch.uint8, device=dev)
    lo, hi = (float(bounds[0]), float(bounds[1])) if bounds is not None else (0.0, 0.0)
    with torch.cuda.device(dev):
        s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
        N.check(lib.sc_moments(C.c_void_p(rp.data_ptr()), rp.stride(0), n, None, 1, 1 if bounds is not None else 0,
                               lo, hi, C.c_void_p(out.data_ptr()), C.c_void_p(scratch.data_ptr()), s))
        m = out[0].cpu().numpy()
    charge = float(np.sum(q.cpu().numpy() if isinstance(q, torch.Tensor) else q))
    return twiss_from_moments(m, float(p_array.E), charge, 0.0)
