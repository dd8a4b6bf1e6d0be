"""Second-order transport between kicks (Ocelot's SecondTM) for drifts and
quadrupoles, applied to GPU-resident particles.

The reference's second-order map of an element slice
(ocelot/cpbd/transformations/second_order.py:31-38) is

    X <- R.X + sum_jk T[:, j, k] X_j X_k,   then   X <- X + B

with R the first-order matrix (uni_matrix), T the second-order tensor of
``t_nnn`` in its MAD convention (ocelot/cpbd/high_order.py:456-617, the
default ``__MAD__ = True``), element offsets folded into R and B
(tm_utils.map_transform_with_offsets, ocelot/cpbd/tm_utils.py:186-206) and a
tilt applied as rot(-tilt).R.rot(tilt) and the rotated, symmetrised tensor
(tm_params/second_order_params.py:20-22, tm_utils.py:156-172).

The host builds R, B and T of every slice in FP64 (a few hundred flops per
slice) and packs each map for the device: R and B dense, T as the list of
its (i, j<=k) coefficients with the (j, k) and (k, j) terms combined.
``sc_tmap2_apply`` then applies a sequence of such maps to every particle in
one pass over ``rparticles`` (coordinates kept in registers between maps).
Second-order maps do not compose exactly, so a step's slices are applied one
after the other, as the reference's Navigator does.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native as N
from .globals import m_e_GeV

MAP2_DOUBLES = N.SC_MAP2_DOUBLES  # R[36], B[6], then Tc[6][21]


def _cs(k2: float, L: float):
    """cos(sqrt(k2) L) and sin(sqrt(k2) L)/sqrt(k2) for any sign of k2 (the
    real parts the reference takes of its complex square roots)."""
    if k2 > 0:
        w = math.sqrt(k2)
        return math.cos(w * L), math.sin(w * L) / w
    if k2 < 0:
        w = math.sqrt(-k2)
        return math.cosh(w * L), math.sinh(w * L) / w
    return 1.0, L


def second_order_tensor(L: float, h: float, k1: float, k2: float, energy: float) -> np.ndarray:
    """T[6, 6, 6] of a slice of length L [m], curvature h [1/m], quadrupole
    strength k1 [1/m^2] and sextupole strength k2 [1/m^3] at energy [GeV] in
    Ocelot's coordinates (x, x', y, y', tau, delta): the MAD second-order
    coefficients of ocelot/cpbd/high_order.py:456-617, stored with the
    reference's convention that an off-diagonal (j < k) entry carries twice
    the coefficient and (k, j) is zero."""
    ig2 = 0.0
    if energy != 0:
        g = energy / m_e_GeV
        ig2 = 1.0 / (g * g)
    beta = math.sqrt(1.0 - ig2)
    b2, b3 = beta * beta, beta * beta * beta
    h2, h3 = h * h, h * h * h
    kx2, ky2 = k1 + h * h, -k1
    kx4 = kx2 * kx2
    cx, sx = _cs(kx2, L)
    cy, sy = _cs(ky2, L)
    sx2, sy2 = sx * sx, sy * sy
    L2 = L * L
    L3, L4, L5 = L2 * L, L2 * L2, L2 * L2 * L
    dx = (1.0 - cx) / kx2 if kx2 != 0 else L2 / 2.0
    dx2 = dx * dx
    d2y, s2y = 0.5 * sy * sy, sy * cy
    c2y = _cs(ky2, 2 * L)[0]
    fx = (L - sx) / kx2 if kx2 != 0 else L3 / 6.0
    f2y = (L - s2y) / ky2 if ky2 != 0 else L3 / 6.0
    J1 = fx
    J2 = (3.0 * L - 4.0 * sx + sx * cx) / (2 * kx4) if kx2 != 0 else L ** 5 / 20.0
    J3 = ((15 * L - 22.5 * sx + 9 * sx * cx - 1.5 * sx * cx * cx + kx2 * sx2 * sx) / (6 * kx4 * kx2)
          if kx2 != 0 else L ** 7 / 56.0)
    jd = kx2 - 4 * ky2
    Jc = (c2y - cx) / jd if jd != 0 else 0.5 * L2
    Js = (cy * sy - sx) / jd if jd != 0 else L3 / 6
    Jd = (d2y - dx) / jd if jd != 0 else L4 / 24
    Jf = (f2y - fx) / jd if jd != 0 else L5 / 120
    K1, K2 = k1, k2
    khk = K2 + 2 * h * K1

    c = {}
    # x
    c[0, 0, 0] = -1 / 6 * khk * (sx2 + dx) - 0.5 * h * kx2 * sx2
    c[0, 0, 1] = -1 / 6 * khk * sx * dx + 0.5 * h * sx * cx
    c[0, 1, 1] = -1 / 6 * khk * dx2 + 0.5 * h * dx * cx
    c[0, 0, 5] = -h / 12 / beta * khk * (3 * sx * J1 - dx2) + 0.5 * h2 / beta * sx2 + 0.25 / beta * K1 * L * sx
    c[0, 1, 5] = (-h / 12 / beta * khk * (sx * dx2 - 2 * cx * J2) + 0.25 * h2 / beta * (sx * dx + cx * J1)
                  - 0.25 / beta * (sx + L * cx))
    c[0, 5, 5] = (-h2 / 6 / b2 * khk * (dx2 * dx - 2 * sx * J2) + 0.5 * h3 / b2 * sx * J1 - 0.5 * h / b2 * L * sx
                  - 0.5 * h / b2 * ig2 * dx)
    c[0, 2, 2] = K1 * K2 * Jd + 0.5 * (K2 + h * K1) * dx
    c[0, 2, 3] = 0.5 * K2 * Js
    c[0, 3, 3] = K2 * Jd - 0.5 * h * dx
    # x'
    c[1, 0, 0] = -1 / 6 * khk * sx * (1 + 2 * cx)
    c[1, 0, 1] = -1 / 6 * khk * dx * (1 + 2 * cx)
    c[1, 1, 1] = -1 / 3 * khk * sx * dx - 0.5 * h * sx
    c[1, 0, 5] = -h / 12 / beta * khk * (3 * cx * J1 + sx * dx) - 0.25 / beta * K1 * (sx - L * cx)
    c[1, 1, 5] = -h / 12 / beta * khk * (3 * sx * J1 + dx2) + 0.25 / beta * K1 * L * sx
    c[1, 5, 5] = (-h2 / 6 / b2 * khk * (sx * dx2 - 2 * cx * J2) - 0.5 * h / b2 * K1 * (cx * J1 - sx * dx)
                  - 0.5 * h / b2 * ig2 * sx)
    c[1, 2, 2] = K1 * K2 * Js + 0.5 * (K2 + h * K1) * sx
    c[1, 2, 3] = 0.5 * K2 * Jc
    c[1, 3, 3] = K2 * Js - 0.5 * h * sx
    # y
    c[2, 0, 2] = 0.5 * K2 * (cy * Jc - 2 * K1 * sy * Js) + 0.5 * h * K1 * sx * sy
    c[2, 0, 3] = 0.5 * K2 * (sy * Jc - 2 * cy * Js) + 0.5 * h * sx * cy
    c[2, 1, 2] = 0.5 * K2 * (cy * Js - 2 * K1 * sy * Jd) + 0.5 * h * K1 * dx * sy
    c[2, 1, 3] = 0.5 * K2 * (sy * Js - 2 * cy * Jd) + 0.5 * h * dx * cy
    c[2, 2, 5] = 0.5 * h / beta * K2 * (cy * Jd - 2 * K1 * sy * Jf) + 0.5 * h2 / beta * K1 * J1 * sy - 0.25 / beta * K1 * L * sy
    c[2, 3, 5] = 0.5 * h / beta * K2 * (sy * Jd - 2 * cy * Jf) + 0.5 * h2 / beta * J1 * cy - 0.25 / beta * (sy + L * cy)
    # y'
    c[3, 0, 2] = 0.5 * K1 * K2 * (2 * cy * Js - sy * Jc) + 0.5 * (K2 + h * K1) * sx * cy
    c[3, 0, 3] = 0.5 * K2 * (2 * K1 * sy * Js - cy * Jc) + 0.5 * (K2 + h * K1) * sx * sy
    c[3, 1, 2] = 0.5 * K1 * K2 * (2 * cy * Jd - sy * Js) + 0.5 * (K2 + h * K1) * dx * cy
    c[3, 1, 3] = 0.5 * K2 * (2 * K1 * sy * Jd - cy * Js) + 0.5 * (K2 + h * K1) * dx * sy
    c[3, 2, 5] = (0.5 * h / beta * K1 * K2 * (2 * cy * Jf - sy * Jd) + 0.5 * h / beta * (K2 + h * K1) * J1 * cy
                  + 0.25 / beta * K1 * (sy - L * cy))
    c[3, 3, 5] = (0.5 * h / beta * K2 * (2 * K1 * sy * Jf - cy * Jd) + 0.5 * h / beta * (K2 + h * K1) * J1 * sy
                  - 0.25 / beta * K1 * L * sy)
    # tau (the reference's sign convention: minus the path-length coefficients)
    c[4, 0, 0] = -(h / 12 / beta * khk * (sx * dx + 3 * J1) - 0.25 / beta * K1 * (L - sx * cx))
    c[4, 0, 1] = -(h / 12 / beta * khk * dx2 + 0.25 / beta * K1 * sx2)
    c[4, 1, 1] = -(h / 6 / beta * khk * J2 - 0.5 / beta * sx - 0.25 / beta * K1 * (J1 - sx * dx))
    c[4, 0, 5] = -(h2 / 12 / b2 * khk * (3 * dx * J1 - 4 * J2) + 0.25 * h / b2 * K1 * J1 * (1 + cx)
                   + 0.5 * h / b2 * ig2 * sx)
    c[4, 1, 5] = -(h2 / 12 / b2 * khk * (dx * dx2 - 2 * sx * J2) + 0.25 * h / b2 * K1 * sx * J1
                   + 0.5 * h / b2 * ig2 * dx)
    c[4, 5, 5] = -(h3 / 6 / b3 * khk * (3 * J3 - 2 * dx * J2) + h2 / 6 / b3 * K1 * (sx * dx2 - J2 * (1 + 2 * cx))
                   + 1.5 / b3 * ig2 * (h2 * J1 - L))
    c[4, 2, 2] = -(-h / beta * K1 * K2 * Jf - 0.5 * h / beta * (K2 + h * K1) * J1 + 0.25 / beta * K1 * (L - cy * sy))
    c[4, 2, 3] = -(-0.5 * h / beta * K2 * Jd - 0.25 / beta * K1 * sy2)
    c[4, 3, 3] = -(-h / beta * K2 * Jf + 0.5 * h2 / beta * J1 - 0.25 / beta * (L + cy * sy))

    T = np.zeros((6, 6, 6))
    for (i, j, k), v in c.items():
        T[i, j, k] = v * 2 if j != k else v
    return T


def rot_matrix(angle: float) -> np.ndarray:
    """6x6 roll by ``angle`` (the reference's rot_mtx, ocelot/cpbd/r_matrix.py:11-19)."""
    cs, sn = math.cos(angle), math.sin(angle)
    m = np.eye(6)
    m[0, 0] = m[1, 1] = m[2, 2] = m[3, 3] = cs
    m[0, 2] = m[1, 3] = sn
    m[2, 0] = m[3, 1] = -sn
    return m


def symmetrize(T: np.ndarray) -> np.ndarray:
    """T[i, j, k] = T[i, k, j] = (T[i, j, k] + T[i, k, j]) / 2 for j != k (tm_utils.sym_matrix)."""
    S = T.copy()
    for j in range(6):
        for k in range(j + 1, 6):
            a = (S[:, j, k] + S[:, k, j]) / 2.0
            S[:, j, k] = a
            S[:, k, j] = a
    return S


def rotate_tensor(T: np.ndarray, tilt: float) -> np.ndarray:
    """Second-order tensor of a rolled element: rot(-tilt) applied to the
    output index and rot(tilt) to both input indices (the T part of
    tm_utils.transfer_map_rotation), then symmetrised."""
    ra, rb = rot_matrix(tilt), rot_matrix(-tilt)
    Tin = np.einsum("ilm,lj,mk->ijk", T, ra, ra)
    return symmetrize(np.einsum("il,ljk->ijk", rb, Tin))


def with_offsets(M: np.ndarray, R: np.ndarray, T: np.ndarray):
    """(B, R) of an element displaced by M = (-dx, 0, -dy, 0, 0, 0): R gains
    the T terms linear in M, B = R.M - M + M.T.M (tm_utils.map_transform_with_offsets)."""
    R_off = R + np.einsum("l,ijl->ij", M, T) + np.einsum("l,ilj->ij", M, T)
    B = R @ M - M + np.einsum("j,ijk,k->i", M, T, M)
    return B, R_off


def element_map2(e, length: float, energy: float):
    """(R, T, B) of a ``length`` slice of a drift/quadrupole/marker ``e``
    as the reference's SecondTM applies it (R and T rolled by the tilt, B as
    built from the offsets)."""
    from .track import _element_params, first_order_matrix
    _, k1, tilt, dx, dy = _element_params(e)
    R0 = first_order_matrix(length, k1, energy)
    T0 = second_order_tensor(length, 0.0, k1, 0.0, energy)
    M = np.array([-dx, 0.0, -dy, 0.0, 0.0, 0.0])
    B, R1 = with_offsets(M, R0, T0)
    if tilt != 0.0:
        return rot_matrix(-tilt) @ R1 @ rot_matrix(tilt), rotate_tensor(T0, tilt), B
    return R1, T0, B


def pack_map(R, T, B) -> np.ndarray:
    """One map in the device layout: R (row-major), B, then Tc[6][21], the
    coefficient of x_j x_k (j <= k, lexicographic pairs) in output i:
    T[i,j,k] + T[i,k,j] off the diagonal, T[i,j,j] on it."""
    out = np.zeros(MAP2_DOUBLES)
    out[:36] = np.asarray(R, dtype=np.float64).reshape(-1)
    out[36:42] = np.asarray(B, dtype=np.float64).reshape(-1)
    q = 0
    for j in range(6):
        for k in range(j, 6):
            out[42 + np.arange(6) * 21 + q] = T[:, j, k] + (T[:, k, j] if k != j else 0.0)
            q += 1
    return out


def tmap2_apply(maps, rparticles) -> None:
    """Apply the packed maps (array [m, MAP2_DOUBLES]) in order to the CUDA
    float64 [6, N] ``rparticles`` (rows contiguous), in place."""
    import torch
    maps = np.ascontiguousarray(np.asarray(maps, dtype=np.float64).reshape(-1, MAP2_DOUBLES))
    if not (isinstance(rparticles, torch.Tensor) and rparticles.is_cuda and rparticles.dtype == torch.float64):
        raise TypeError("rparticles must be a CUDA float64 tensor")
    if rparticles.dim() != 2 or rparticles.shape[0] != 6 or rparticles.stride(1) != 1:
        raise ValueError("rparticles must be [6, N] with contiguous rows")
    dev_maps = torch.from_numpy(maps).to(rparticles.device)
    lib = N.lib()
    stream = C.c_void_p(torch.cuda.current_stream(rparticles.device).cuda_stream)
    with torch.cuda.device(rparticles.device):
        N.check(lib.sc_tmap2_apply(C.c_void_p(dev_maps.data_ptr()), maps.shape[0], C.c_void_p(rparticles.data_ptr()),
                                   rparticles.stride(0), rparticles.shape[1], stream))
        torch.cuda.current_stream(rparticles.device).synchronize()
