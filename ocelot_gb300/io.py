"""Beam files: the formats a space-charge transport line is loaded from and
saved to, with the reference's function names and results.

* ``.npz``: the arrays of a ParticleArray (ocelot/cpbd/io.py:223-241).
* ``.ast`` / ``.001``: ASTRA particle lists, converted between ASTRA's
  Cartesian (x, y, z, px, py, pz) and Ocelot's MAD coordinates with the exact
  transforms of ocelot/adaptors/astra2ocelot.py:7-56 and 150-233; the first
  ASTRA line is the reference particle.
* ``.fmt1``: CSRtrack lists (ocelot/adaptors/csrtrack2ocelot.py:9-87).

Loading and saving are host work (text parsing and a few vector operations
per file); the loaded arrays go to the GPU with
``DeviceParticleArray.from_host``.  The arithmetic follows the reference's
operation order, so a file round trip gives the reference's numbers.  The
openPMD (.h5) branch of the reference needs h5py and is not provided.
"""
from __future__ import annotations

import os

import numpy as np

from .beam import ParticleArray
from .globals import m_e_eV, m_e_GeV


# ---------------------------------------------------------------------------
# npz
# ---------------------------------------------------------------------------
def save_particle_array2npz(filename, p_array):
    np.savez_compressed(filename, rparticles=p_array.rparticles, q_array=p_array.q_array, E=p_array.E, s=p_array.s)


def load_particle_array_from_npz(filename, print_params=False):
    p_array = ParticleArray()
    with np.load(filename) as data:
        for key in data.keys():
            setattr(p_array, key, data[key])
    if print_params:
        print(_summary(p_array))
    return p_array


# ---------------------------------------------------------------------------
# ASTRA
# ---------------------------------------------------------------------------
def exact_xp_2_xxstg_mad(xp, gamref):
    """ASTRA Cartesian [N, 6] (x, y, z, px, py, pz - pref; eV/c) -> MAD
    (x, x', y, y', tau, delta) [N, 6] at reference gamma ``gamref``."""
    n = xp.shape[0]
    out = np.zeros((n, 6))
    pref = m_e_eV * np.sqrt(gamref ** 2 - 1)
    u = np.c_[xp[:, 3], xp[:, 4], xp[:, 5] + pref]
    gamma = np.sqrt(1 + np.sum(u * u, 1) / m_e_eV ** 2)
    beta = np.sqrt(1 - gamma ** -2)
    betaref = np.sqrt(1 - gamref ** -2)
    p0 = np.linalg.norm(u, 2, 1).reshape((n, 1))
    u = u / p0
    cdt = -xp[:, 2] / (beta * u[:, 2])
    out[:, 0] = xp[:, 0] + beta * u[:, 0] * cdt
    out[:, 2] = xp[:, 1] + beta * u[:, 1] * cdt
    out[:, 4] = cdt
    out[:, 1] = xp[:, 3] / pref
    out[:, 3] = xp[:, 4] / pref
    out[:, 5] = (gamma / gamref - 1) / betaref
    return out


def exact_xxstg_2_xp_mad(xxstg, gamref):
    """MAD [6, N] -> ASTRA Cartesian [N, 6] (pz relative to pref)."""
    n = int(xxstg.size / 6)
    xp = np.zeros((n, 6))
    pref = m_e_eV * np.sqrt(gamref ** 2 - 1)
    betaref = np.sqrt(1 - gamref ** -2)
    gamma = (betaref * xxstg[5] + 1) * gamref
    beta = np.sqrt(1 - gamma ** -2)
    pz2pref = np.sqrt(((gamma * beta) / (gamref * betaref)) ** 2 - xxstg[1] ** 2 - xxstg[3] ** 2)
    u = np.c_[xxstg[1] / pz2pref, xxstg[3] / pz2pref, np.ones(n)]
    u = u / np.linalg.norm(u, 2, 1).reshape((n, 1))
    xp[:, 0] = xxstg[0] - u[:, 0] * beta * xxstg[4]
    xp[:, 1] = xxstg[2] - u[:, 1] * beta * xxstg[4]
    xp[:, 2] = -u[:, 2] * beta * xxstg[4]
    xp[:, 3] = u[:, 0] * gamma * beta * m_e_eV
    xp[:, 4] = u[:, 1] * gamma * beta * m_e_eV
    xp[:, 5] = u[:, 2] * gamma * beta * m_e_eV - pref
    return xp


def astraBeam2particleArray(filename, print_params=True):
    """ASTRA particle file -> ParticleArray.  Particles with a non-positive
    status flag (column 10: lost or not injected) are dropped; the first line
    is the reference particle (its z is the position s, its pz the
    reference momentum); if its charge is zero it is not a particle."""
    P0 = np.loadtxt(filename)
    P0 = P0[np.argwhere(P0[:, 9] > 0).reshape(-1), :]
    s_ref = P0[0, 2]
    Pref = P0[0, 5]
    if P0[0, 7] == 0:
        xp = P0[1:, :6]
        charge = abs(P0[1:, 7]) * 1e-9  # nC -> C
    else:
        charge = abs(P0[:, 7]) * 1e-9
        xp = P0[:, :6]
        xp[0, 2] = 0.
        xp[0, 5] = 0.
    gamref = np.sqrt((Pref / m_e_eV) ** 2 + 1)
    xxstg = exact_xp_2_xxstg_mad(xp, gamref)
    p_array = ParticleArray(len(charge))
    p_array.s = s_ref
    p_array.E = np.sqrt((Pref / m_e_eV) ** 2 + 1) * m_e_GeV
    for k in range(6):
        p_array.rparticles[k] = xxstg[:, k]
    p_array.q_array = charge
    if print_params:
        print(_summary(p_array))
    return p_array


def particleArray2astraBeam(p_array, filename="tytest.ast"):
    """ParticleArray -> ASTRA particle file: a reference particle at z = s
    with pz = pref first, then the particles (charge in nC, negative for
    electrons), time 0, species 1 (electron), status 5 (standard)."""
    gamref = p_array.E / m_e_GeV
    s0 = p_array.s
    xp = exact_xxstg_2_xp_mad(p_array.rparticles.view(), gamref)
    Pref = np.sqrt(p_array.E ** 2 / m_e_GeV ** 2 - 1) * m_e_eV
    xp = np.vstack((np.array([0, 0, s0, 0, 0, Pref]), xp))
    charge = -p_array.q_array.reshape(len(p_array.q_array), 1) * 1e+9  # C -> nC
    charge = np.vstack((0, charge))
    flag = np.ones((len(charge + 1), 1))
    table = np.append(xp, flag * 0, axis=1)
    table = np.append(table, charge, axis=1)
    table = np.append(table, flag, axis=1)
    table = np.append(table, flag * 5, axis=1)
    np.savetxt(filename, table, fmt='%20.12e %20.12e %20.12e %20.12e %20.12e %20.12e %20.12e %20.12e %d %d')


# ---------------------------------------------------------------------------
# CSRtrack
# ---------------------------------------------------------------------------
def csrtrackBeam2particleArray(filename, orient="H"):
    """CSRtrack .fmt1 -> ParticleArray.  Orientation "H": columns
    z x y pz px py; "V": z y x pz py px with x and px negated.  The first
    particle is the reference; the others are stored relative to it."""
    pd = np.loadtxt(filename)
    n = np.shape(pd)[0] - 1
    pd1 = np.zeros((n, 6))
    if orient == "H":
        cols = (1, 2, 0, 4, 5, 3)
        sign = (1, 1, 1, 1, 1, 1)
    else:
        cols = (2, 1, 0, 5, 4, 3)
        sign = (-1, 1, 1, -1, 1, 1)
    for k in range(6):
        pd1[:, k] = pd[1:, cols[k]] if sign[k] > 0 else -pd[1:, cols[k]]
    for k in range(6):
        pd1[1:n, k] = pd1[1:n, k] + pd1[0, k]
    p_ref = np.sqrt(pd1[0, 3] ** 2 + pd1[0, 4] ** 2 + pd1[0, 5] ** 2)
    px = pd1[:, 3] / p_ref
    py = pd1[:, 4] / p_ref
    Eref = np.sqrt(m_e_eV ** 2 + p_ref ** 2)
    pe = (np.sqrt(m_e_eV ** 2 + (pd1[:, 3] ** 2 + pd1[:, 4] ** 2 + pd1[:, 5] ** 2)) - Eref) / p_ref
    p_array = ParticleArray(n)
    p_array.rparticles[0] = pd1[:, 0]
    p_array.rparticles[2] = pd1[:, 1]
    p_array.rparticles[4] = -(pd1[:, 2] - pd1[0, 2])
    p_array.rparticles[1] = px[:]
    p_array.rparticles[3] = py[:]
    p_array.rparticles[5] = pe[:]
    p_array.q_array[:] = pd[1:, 6]
    p_array.s = pd1[0, 2]
    p_array.E = Eref * 1e-9
    return p_array


def particleArray2csrtrackBeam(p_array, filename="csr_beam.fmt1"):
    """ParticleArray -> CSRtrack .fmt1 (orientation "H")."""
    Eref = p_array.E * 1e9  # GeV -> eV
    p_ref = np.sqrt(Eref ** 2 - m_e_eV ** 2)
    E = p_array.rparticles[5] * p_ref + Eref
    p = np.sqrt(E ** 2 - m_e_eV ** 2)
    px = p_array.rparticles[1] * p_ref
    py = p_array.rparticles[3] * p_ref
    pz = np.sqrt(p ** 2 - px ** 2 - py ** 2)
    x = p_array.rparticles[0]
    y = p_array.rparticles[2]
    z = -p_array.rparticles[4] + p_array.s
    n = p_array.rparticles.shape[1]
    pd = np.zeros((n + 1, 7))
    pd[0] = [0, 0, 0, 0, 0, 0, 0]
    pd[1] = [z[0], x[0], y[0], pz[0], px[0], py[0], p_array.q_array[0]]
    for col, v in enumerate((z, x, y, pz, px, py)):
        pd[2:, col] = v[1:] - v[0]
    pd[2:, 6] = p_array.q_array[1:]
    np.savetxt(filename, pd, fmt='%.7e')


# ---------------------------------------------------------------------------
# by extension
# ---------------------------------------------------------------------------
def load_particle_array(filename, print_params=False):
    """.npz, .ast/.001 (ASTRA) or .fmt1 (CSRtrack) -> ParticleArray."""
    ext = os.path.splitext(filename)[1]
    if ext == ".npz":
        p_array = load_particle_array_from_npz(filename)
    elif ext in (".ast", ".001"):
        p_array = astraBeam2particleArray(filename, print_params=False)
    elif ext == ".fmt1":
        p_array = csrtrackBeam2particleArray(filename)
    else:
        raise ValueError(f"Unknown format of the beam file: {ext} but must be *.ast, *fmt1 or *.npz")
    if print_params:
        print(_summary(p_array))
    return p_array


def save_particle_array(filename, p_array):
    """ParticleArray -> .npz, .ast (ASTRA) or .fmt1 (CSRtrack)."""
    ext = os.path.splitext(filename)[1]
    if ext == ".npz":
        save_particle_array2npz(filename, p_array)
    elif ext == ".ast":
        particleArray2astraBeam(p_array, filename)
    elif ext == ".fmt1":
        particleArray2csrtrackBeam(p_array, filename)
    else:
        raise ValueError(f"Unknown format of the beam file: {ext} but must be *.ast, *.fmt1 or *.npz")


def _summary(p_array):
    q = np.asarray(p_array.q_array)
    return (f"ParticleArray: {p_array.rparticles.shape[1]} particles, charge {q.sum():.6g} C, "
            f"E = {float(p_array.E):.6g} GeV, s = {float(p_array.s):.6g} m")
