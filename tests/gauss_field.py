"""Closed-form potential and field of a Gaussian bunch: the known answer of the
Poisson solve (test helper, numpy + scipy).

A charge Q distributed as a 3D Gaussian with rms sizes (sx, sy, sz), centred
at the origin, has in free space the potential

    phi(x) = Q / (4 pi eps0) / sqrt(pi) * Int_0^inf exp(-sum_i x_i^2 / (2 s_i^2 + t))
                                                   / sqrt(prod_i (2 s_i^2 + t)) dt

and the field E_i = -d phi / dx_i, the same integral with the extra factor
2 x_i / (2 s_i^2 + t).  (For s_x = s_y = s_z = s the integral is
sqrt(pi) erf(r / (sqrt(2) s)) / r, the point-charge potential of the enclosed
charge.)  The integral runs over log t with adaptive Gauss-Kronrod
quadrature; below t = 1e-8 min(2 s^2) the integrand is constant to that
precision and above t = 1e14 max(2 s^2) only the potential's t^(-3/2) tail is
left, added in closed form.
"""
from __future__ import annotations

import numpy as np
from scipy.integrate import quad_vec

# the reference's constants (ocelot/common/globals.py:13-24)
_SPEED_OF_LIGHT = 299792458.0
_EPS0 = 1 / (4 * 3.141592653589793 * 1e-7) / _SPEED_OF_LIGHT ** 2
COULOMB = 1.0 / (4 * np.pi * _EPS0)


def potential_and_field(pts, sigma, charge):
    """phi [M] (V) and E [M, 3] (V/m) of the Gaussian bunch at pts [M, 3] (m)."""
    pts = np.asarray(pts, dtype=np.float64)
    s2 = 2.0 * np.asarray(sigma, dtype=np.float64) ** 2
    x2 = pts ** 2
    m = pts.shape[0]

    def f(t):
        d = s2 + t
        e = np.exp(-(x2 / d).sum(axis=1)) / np.sqrt(d.prod())
        return np.concatenate([e, (2.0 * pts / d * e[:, None]).T.ravel()])

    lo, hi = np.log(1e-8 * s2.min()), np.log(1e14 * s2.max())
    val, _ = quad_vec(lambda s: f(np.exp(s)) * np.exp(s), lo, hi, epsabs=0, epsrel=1e-11, limit=2000)
    val = val + f(0.0) * np.exp(lo)
    val[:m] += 2.0 / np.sqrt(np.exp(hi))
    c = COULOMB * charge / np.sqrt(np.pi)
    return c * val[:m], c * val[m:].reshape(3, m).T


def node_grid(nmesh, sigma, charge, span=4.0):
    """A mesh of nmesh nodes spanning +-span sigma on each axis, centred on
    the bunch: (node positions [nx, ny, nz, 3], steps [3], the charge grid
    rho(node) * hx hy hz -- the midpoint rule of the cell charges)."""
    n = np.asarray(nmesh)
    sig = np.asarray(sigma, dtype=np.float64)
    h = 2 * span * sig / (n - 1)
    axes = [(np.arange(n[a]) - (n[a] - 1) / 2) * h[a] for a in range(3)]
    pos = np.stack(np.meshgrid(*axes, indexing="ij"), axis=-1)
    rho = charge / ((2 * np.pi) ** 1.5 * sig.prod()) * np.exp(-0.5 * ((pos / sig) ** 2).sum(axis=-1))
    return pos, h, rho * h.prod()


def grid_errors(phi, pos, h, sigma, charge, stride=3):
    """Relative RMS errors of a potential on the node grid and of its
    forward-difference fields (the reference's field grids, sc.py:195-200,
    which sit half a step along their axis from the nodes) against the closed
    form, on every stride-th node of each axis: (e_phi, [e_Ex, e_Ey, e_Ez])."""
    sl = (slice(None, None, stride),) * 3
    p = pos[sl].reshape(-1, 3)
    ph_ex, _ = potential_and_field(p, sigma, charge)
    e_phi = float(np.linalg.norm(phi[sl].ravel() - ph_ex) / np.linalg.norm(ph_ex))
    e_field = []
    for a in range(3):
        num = (phi - np.roll(phi, -1, axis=a)) / h[a]
        cut = [slice(None, None, stride)] * 3
        cut[a] = slice(0, phi.shape[a] - 1, stride)
        cut = tuple(cut)
        q = pos[cut].reshape(-1, 3).copy()
        q[:, a] += h[a] / 2
        _, E_ex = potential_and_field(q, sigma, charge)
        e_field.append(float(np.linalg.norm(num[cut].ravel() - E_ex[:, a]) / np.linalg.norm(E_ex[:, a])))
    return e_phi, e_field
