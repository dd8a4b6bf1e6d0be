"""CPU oracle for Ocelot's 3D space-charge kick -- TEST INFRASTRUCTURE ONLY.

This module restates, in numpy/scipy, the algorithm of Ocelot's
``SpaceCharge.apply`` (ocelot/cpbd/sc.py:208-251) together with the two
coordinate transforms it calls (ocelot/cpbd/coord_transform.py:16-96).
Every function cites the reference lines it follows and performs the same
floating-point operations in the same order, so that on the same machine its
results are bit-identical to the reference's numpy fallback path (numpy.fft,
no numexpr).

Only the test-suite, the smoke check and the CPU-baseline leg of the bench may
import this module, and only as the checker.  The product path
(``ocelot_gb300``) never calls it.

Parity is pinned in two ways (both committed under tests/golden/):
  * fixtures generated by importing the reference itself and running its
    ``SpaceCharge`` on seeded beams (tests/golden/make_golden.py);
  * the reference's own regression vectors of ``test_track_with_sp``
    (unit_tests/ebeam_test/space_charge/ref_results/test_track_with_sp.json),
    reproduced by running the reference's ``track()`` with this oracle swapped
    in for its kick (tests/golden/make_golden.py, recorded in tests/golden/track_pin.json).
"""
from __future__ import annotations

import numpy as np
import scipy.ndimage as ndimage

# Physical constants, computed with the same expressions as
# ocelot/common/globals.py:13-24 so that they are bit-identical.
pi = 3.141592653589793
speed_of_light = 299792458.0
q_e = 1.6021766208e-19
m_e_kg = 9.10938215e-31
m_e_eV = m_e_kg * speed_of_light ** 2 / q_e
m_e_GeV = m_e_eV / 1e+9
mu_0 = 4 * pi * 1e-7
epsilon_0 = 1 / mu_0 / speed_of_light ** 2


# --------------------------------------------------------------------------
# Coordinate transforms
# --------------------------------------------------------------------------
def mad_to_cartesian(rp: np.ndarray, gamref: float) -> np.ndarray:
    """MAD (x, x', y, y', tau, delta) -> lab (x, y, z, px, py, pz[eV/c]).

    Follows coord_transform.py:57-96 (``xxstg_2_xp_mad``, numpy branch).
    """
    n = rp.shape[1]
    xp = np.zeros(rp.shape)
    betaref = np.sqrt(1 - gamref ** -2)
    gamma = (betaref * rp[5] + 1) * gamref                       # :65
    beta = np.sqrt(1 - gamma ** -2)                               # :66
    pz2pref = np.sqrt(((gamma * beta) / (gamref * betaref)) ** 2
                      - rp[1] ** 2 - rp[3] ** 2)                  # :67
    u = np.c_[rp[1] / pz2pref, rp[3] / pz2pref, np.ones(n)]       # :69
    norm = np.linalg.norm(u, 2, 1).reshape((n, 1))                # :71
    u = u / norm
    u0, u1, u2 = u[:, 0], u[:, 1], u[:, 2]
    xp[0] = rp[0] - u0 * beta * rp[4]                             # :86-91
    xp[1] = rp[2] - u1 * beta * rp[4]
    xp[2] = -u2 * beta * rp[4]
    xp[3] = u0 * gamma * beta * m_e_eV
    xp[4] = u1 * gamma * beta * m_e_eV
    xp[5] = u2 * gamma * beta * m_e_eV
    return xp


def cartesian_to_mad(xp: np.ndarray, gamref: float, out: np.ndarray | None = None) -> np.ndarray:
    """Lab Cartesian -> MAD, re-projecting onto the reference plane.

    Follows coord_transform.py:16-54 (``xp_2_xxstg_mad``, numpy branch).
    All six rows are rewritten.
    """
    n = xp.shape[1]
    rp = np.zeros(xp.shape) if out is None else out
    pref = m_e_eV * np.sqrt(gamref ** 2 - 1)                      # :19
    betaref = np.sqrt(1 - gamref ** -2)
    u = np.c_[xp[3], xp[4], xp[5]]                                # :21
    gamma = np.sqrt(1 + np.sum(u * u, 1) / m_e_eV ** 2)           # :27
    beta = np.sqrt(1 - gamma ** -2)
    p0 = np.linalg.norm(u, 2, 1).reshape((n, 1))                  # :31
    u = u / p0
    u0, u1, u2 = u[:, 0], u[:, 1], u[:, 2]
    cdt = -xp[2] / (beta * u2)                                    # :46
    rp[0] = xp[0] + beta * u0 * cdt
    rp[2] = xp[1] + beta * u1 * cdt
    rp[5] = (gamma / gamref - 1) / betaref
    rp[4] = cdt
    rp[1] = xp[3] / pref
    rp[3] = xp[4] / pref
    return rp


# --------------------------------------------------------------------------
# Stages of the kick
# --------------------------------------------------------------------------
def velocity_frame(xp: np.ndarray):
    """Mean-momentum frame and rest-frame gamma (sc.py:224-239).

    Returns (T, Pav, gamma0, beta0) with T = [t1 t2 t3] as columns.
    """
    t3 = np.mean(xp[3:6], axis=1)
    Pav = np.linalg.norm(t3)
    t3 = t3 / Pav
    ey = np.array([0, 1, 0])
    t1 = np.cross(ey, t3)
    t1 = t1 / np.linalg.norm(t1)
    t2 = np.cross(t3, t1)
    T = np.c_[t1, t2, t3]
    gamma0 = np.sqrt((Pav / m_e_eV) ** 2 + 1)
    beta02 = 1 - gamma0 ** -2
    beta0 = np.sqrt(beta02)
    return T, Pav, gamma0, beta0


def mesh_geometry(xyz: np.ndarray, Q: np.ndarray, gamma0: float, nmesh,
                  mesh_scale: float | None = None, mesh_shift: float | None = None):
    """Rest-frame grid coordinates of the particles (sc.py:171-186).

    ``xyz`` is the [N, 3] rotated position array; it is modified in place
    exactly as the reference modifies it (z scaled by gamma0).
    ``mesh_scale``/``mesh_shift`` are the two uniform draws the reference
    takes when ``random_mesh`` is on (sc.py:174-175, 184-185).
    Returns (X [N,3] in cell units after the offset, steps[3]).
    """
    nxyz = np.array(nmesh)
    X = xyz
    X[:, 2] = X[:, 2] * gamma0
    XX = np.max(X, axis=0) - np.min(X, axis=0)
    if mesh_scale is not None:
        XX = XX * mesh_scale
    steps = XX / (nxyz - 3)
    X = X / steps
    X_min = np.min(X, axis=0)
    X_mid = np.dot(Q, X) / np.sum(Q)
    X_off = np.floor(X_min - X_mid) + X_mid
    if mesh_shift is not None:
        X_off = X_off + mesh_shift
    X = X - X_off
    return X, steps


def ngp_keys(X: np.ndarray, nmesh) -> np.ndarray:
    """Nearest-grid-point linear cell keys (sc.py:187-192)."""
    nx, ny, nz = (int(v) for v in nmesh)
    nzny = nz * ny
    Xi = np.int_(np.floor(X) + 1)
    return np.int_(Xi[:, 0] * nzny + Xi[:, 1] * nz + Xi[:, 2])


def deposit(keys: np.ndarray, Q: np.ndarray, nmesh) -> np.ndarray:
    """NGP charge deposition by sequential bincount (sc.py:193)."""
    nx, ny, nz = (int(v) for v in nmesh)
    return np.bincount(keys, Q, nz * ny * nx).reshape((nx, ny, nz))


def igf_kernel(ijk2, hxyz) -> np.ndarray:
    """Integrated Green's function on the (N)^3 lag octant (sc.py:109-133)."""
    i2, j2, k2 = (int(v) for v in ijk2)
    hx, hy, hz = hxyz
    x = hx * np.r_[0:i2 + 1] - hx / 2
    y = hy * np.r_[0:j2 + 1] - hy / 2
    z = hz * np.r_[0:k2 + 1] - hz / 2
    x, y, z = np.ix_(x, y, z)
    r = np.sqrt(x * x + y * y + z * z)
    IG = (-x * x * 0.5 * np.arctan(y * z / (x * r)) + y * z * np.log(x + r)
          - y * y * 0.5 * np.arctan(z * x / (y * r)) + z * x * np.log(y + r)
          - z * z * 0.5 * np.arctan(x * y / (z * r)) + x * y * np.log(z + r))
    return (IG[1:i2 + 1, 1:j2 + 1, 1:k2 + 1] - IG[0:i2, 1:j2 + 1, 1:k2 + 1]
            - IG[1:i2 + 1, 0:j2, 1:k2 + 1] + IG[0:i2, 0:j2, 1:k2 + 1]
            - IG[1:i2 + 1, 1:j2 + 1, 0:k2] + IG[0:i2, 1:j2 + 1, 0:k2]
            + IG[1:i2 + 1, 0:j2, 0:k2] - IG[0:i2, 0:j2, 0:k2])


def potential(q: np.ndarray, steps, fft_workers: int | None = None) -> np.ndarray:
    """Free-space potential by zero-padded FFT convolution (sc.py:135-168).

    With ``fft_workers=None`` the FFTs are numpy's (the reference's fallback
    path, sc.py:164).  With an integer, scipy.fft runs them on that many
    threads -- the analogue of the reference's threaded pyfftw branch
    (sc.py:150-162), used only for timing the CPU baseline.
    """
    hx, hy, hz = steps
    Nx, Ny, Nz = q.shape
    out = np.zeros((2 * Nx - 1, 2 * Ny - 1, 2 * Nz - 1))
    out[:Nx, :Ny, :Nz] = q
    K1 = igf_kernel(q.shape, steps)
    K2 = np.zeros((2 * Nx - 1, 2 * Ny - 1, 2 * Nz - 1))
    K2[0:Nx, 0:Ny, 0:Nz] = K1
    K2[0:Nx, 0:Ny, Nz:2 * Nz - 1] = K2[0:Nx, 0:Ny, Nz - 1:0:-1]
    K2[0:Nx, Ny:2 * Ny - 1, :] = K2[0:Nx, Ny - 1:0:-1, :]
    K2[Nx:2 * Nx - 1, :, :] = K2[Nx - 1:0:-1, :, :]
    if fft_workers is None:
        out = np.real(np.fft.ifftn(np.fft.fftn(out) * np.fft.fftn(K2)))
    else:
        import scipy.fft as sfft
        out = np.real(sfft.ifftn(sfft.fftn(out, workers=fft_workers)
                                 * sfft.fftn(K2, workers=fft_workers), workers=fft_workers))
    out[:Nx, :Ny, :Nz] = out[:Nx, :Ny, :Nz] / (4 * pi * epsilon_0 * hx * hy * hz)
    return out[:Nx, :Ny, :Nz]


def field_grids(p: np.ndarray, steps):
    """Forward-difference field grids, zero on the last plane (sc.py:195-200)."""
    nx, ny, nz = p.shape
    Ex = np.zeros(p.shape)
    Ey = np.zeros(p.shape)
    Ez = np.zeros(p.shape)
    Ex[:nx - 1, :, :] = (p[:nx - 1, :, :] - p[1:nx, :, :]) / steps[0]
    Ey[:, :ny - 1, :] = (p[:, :ny - 1, :] - p[:, 1:ny, :]) / steps[1]
    Ez[:, :, :nz - 1] = (p[:, :, :nz - 1] - p[:, :, 1:nz]) / steps[2]
    return Ex, Ey, Ez


def gather(Ex, Ey, Ez, X: np.ndarray, gamma0: float) -> np.ndarray:
    """Trilinear gather at staggered points (sc.py:201-204)."""
    n = X.shape[0]
    E = np.zeros((n, 3))
    E[:, 0] = ndimage.map_coordinates(Ex, np.c_[X[:, 0], X[:, 1] + 0.5, X[:, 2] + 0.5].T, order=1) * gamma0
    E[:, 1] = ndimage.map_coordinates(Ey, np.c_[X[:, 0] + 0.5, X[:, 1], X[:, 2] + 0.5].T, order=1) * gamma0
    E[:, 2] = ndimage.map_coordinates(Ez, np.c_[X[:, 0] + 0.5, X[:, 1] + 0.5, X[:, 2]].T, order=1)
    return E


def el_field(xyz: np.ndarray, Q: np.ndarray, gamma0: float, nmesh,
             mesh_scale=None, mesh_shift=None, fft_workers=None, record: dict | None = None):
    """Rest-frame field at the particles (sc.py:170-205)."""
    X, steps = mesh_geometry(xyz, Q, gamma0, nmesh, mesh_scale, mesh_shift)
    keys = ngp_keys(X, nmesh)
    q = deposit(keys, Q, nmesh)
    p = potential(q, steps, fft_workers)
    Ex, Ey, Ez = field_grids(p, steps)
    E = gather(Ex, Ey, Ez, X, gamma0)
    if record is not None:
        record.update(X=X, steps=steps, keys=keys, qgrid=q, phi=p, Exyz=E)
    return E


def sc_apply(rparticles: np.ndarray, q_array: np.ndarray, E_GeV: float, zstep: float, nmesh,
             mesh_scale=None, mesh_shift=None, fft_workers=None, record: dict | None = None) -> None:
    """One space-charge kick, in place on ``rparticles`` (sc.py:208-251)."""
    if zstep == 0:
        return
    gamref = E_GeV / m_e_GeV
    betref2 = 1 - gamref ** -2
    betref = np.sqrt(betref2)
    xp = mad_to_cartesian(rparticles, gamref)
    T, Pav, gamma0, beta0 = velocity_frame(xp)
    xyz = np.dot(xp[0:3].T, T)
    xp[3:6] = np.dot(xp[3:6].T, T).T
    Exyz = el_field(xyz, q_array, gamma0, nmesh, mesh_scale, mesh_shift, fft_workers, record)
    cdT = zstep / betref
    xp[3] = xp[3] + cdT * (1 - beta0 * beta0) * Exyz[:, 0]
    xp[4] = xp[4] + cdT * (1 - beta0 * beta0) * Exyz[:, 1]
    xp[5] = xp[5] + cdT * Exyz[:, 2]
    T = np.transpose(T)
    xp[3:6] = np.dot(xp[3:6].T, T).T
    if record is not None:
        record.update(T=np.transpose(T), gamma0=gamma0, beta0=beta0, Pav=Pav)
    cartesian_to_mad(xp, gamref, out=rparticles)


# --------------------------------------------------------------------------
# First-order transport between kicks (next row of the path)
# --------------------------------------------------------------------------
def tmap_apply(rparticles: np.ndarray, R: np.ndarray, B: np.ndarray) -> None:
    """X <- R.X + B in place (transformations/transfer_map.py:40-50)."""
    a = np.add(np.dot(R, rparticles), B)
    rparticles[:] = a[:]


def uni_matrix(z: float, k1: float, energy: float) -> np.ndarray:
    """6x6 first-order matrix of a drift (k1 = 0) or quadrupole of length z
    with no bend and no tilt: ocelot/cpbd/r_matrix.py:41-91 at hx = 0 and
    sum_tilts = 0, the call made by Element/Magnet.create_first_order_main_params
    (ocelot/cpbd/elements/element.py:83-96, magnet.py:106-117).  The same
    operations as the reference, complex square roots included."""
    hx = 0.0
    gamma = energy / m_e_GeV
    kx2 = k1 + hx * hx
    ky2 = -k1
    kx = np.sqrt(kx2 + 0.j)
    ky = np.sqrt(ky2 + 0.j)
    cx = np.cos(z * kx).real
    cy = np.cos(z * ky).real
    sy = (np.sin(ky * z) / ky).real if ky != 0 else z
    igamma2 = 1. / (gamma * gamma) if gamma != 0 else 0.
    beta = np.sqrt(1. - igamma2)
    if kx != 0:
        sx = (np.sin(kx * z) / kx).real
        dx = hx / kx2 * (1. - cx)
        r56 = hx * hx * (z - sx) / kx2 / beta ** 2
    else:
        sx = z
        dx = z * z * hx / 2.
        r56 = hx * hx * z ** 3 / 6. / beta ** 2
    r56 -= z / (beta * beta) * igamma2
    return np.array([[cx, sx, 0., 0., 0., dx / beta],
                     [-kx2 * sx, cx, 0., 0., 0., sx * hx / beta],
                     [0., 0., cy, sy, 0., 0.],
                     [0., 0., -ky2 * sy, cy, 0., 0.],
                     [hx * sx / beta, dx / beta, 0., 0., 1., r56],
                     [0., 0., 0., 0., 0., 1.]])


def _section_length(total_length: float, start_l: float, delta_l: float) -> float:
    if start_l < 1e-10 and np.isclose(delta_l, total_length):
        return total_length
    if start_l + delta_l > total_length or np.isclose(start_l + delta_l, total_length):
        return total_length - start_l
    return delta_l


def navigator_schedule(lengths, unit_step: float, step: int = 1):
    """The kicks of one space-charge process attached from the first to the
    last element, as Ocelot's Navigator steps them: a list of
    (slices, zstep, z0) where slices = [(element index, slice length)] are the
    element sections transported before the kick of length zstep taken at z0
    (track() passes phys_steps, ocelot/cpbd/track.py:474-476).  The slice
    length is the one OpticElement.get_section_tms builds its map for
    (ocelot/cpbd/elements/optic_element.py:376-403): the whole element when a
    slice from its start spans it, the rest of the element when a slice
    reaches its end, the requested length otherwise.

    Restates Navigator.get_next_step / get_next / check_overjump / get_map
    (ocelot/cpbd/navi.py:343-352, 354-371, 219-237, 406-434) for that single
    process, with the lattice length of MagneticLattice.totalLen
    (ocelot/cpbd/magnetic_lattice.py:226-227) and the stop position of
    add_physics_proc (navi.py:76-77).  The floating-point operations are the
    reference's, so z0 and dz are identical to its values.
    """
    lengths = [float(v) for v in lengths]
    nel = len(lengths)
    total = sum(lengths)
    l_stop = np.sum(np.array(lengths[:nel - 1]))
    z0, n_elem, sum_lengths = 0.0, 0, 0.0
    out = []
    while np.abs(z0 - total) > 1e-10:
        phys = np.array([step]) * unit_step
        dz = float(phys.min())
        phys_red = phys - dz
        if z0 + dz > l_stop:
            dz = l_stop - z0
        zstep = float((phys_red + dz)[0])
        if z0 + dz > total:
            dz = total - z0
        slices = []
        i = n_elem
        z1 = z0 + dz
        rem = dz
        L = sum_lengths + lengths[i]
        while z1 + 1e-10 > L:
            dl = L - z0
            slices.append((i, _section_length(lengths[i], z0 + lengths[i] - L, dl)))
            z0 = L
            rem -= dl
            if i >= nel - 1:
                break
            i += 1
            L += lengths[i]
        if abs(rem) > 1e-10:
            slices.append((i, _section_length(lengths[i], z0 + lengths[i] - L, rem)))
        z0 += rem
        sum_lengths = L - lengths[i]
        n_elem = i
        out.append((slices, zstep, float(z0)))
    return out


def track_first_order(rparticles: np.ndarray, q_array: np.ndarray, E_GeV: float, elements, unit_step: float,
                      nmesh, step: int = 1) -> list:
    """Track through drifts and quadrupoles ``elements`` = [(length, k1)] with
    first-order maps and a space-charge kick every ``step`` unit steps, as
    Ocelot's track() does (ocelot/cpbd/track.py:470-480: the maps of a step,
    then the kick).  Returns the (z0, dz) of each kick."""
    kicks = []
    for slices, dz, z0 in navigator_schedule([l for l, _ in elements], unit_step, step):
        for i, dl in slices:
            if dl != 0.0:
                tmap_apply(rparticles, uni_matrix(dl, elements[i][1], E_GeV), np.zeros((6, 1)))
        sc_apply(rparticles, q_array, E_GeV, dz, nmesh)
        kicks.append((z0, dz))
    return kicks


# --------------------------------------------------------------------------
# Seeded synthetic beams (shapes of the benchmark configurations)
# --------------------------------------------------------------------------
def gaussian_beam(n: int, seed: int, sigma_x=50e-6, sigma_px=1e-5, sigma_y=50e-6, sigma_py=1e-5,
                  sigma_tau=100e-6, sigma_p=1e-4, charge=250e-12):
    """Uncorrelated 6D Gaussian in MAD units with equal macro-charges."""
    rng = np.random.default_rng(seed)
    rp = np.empty((6, n))
    for row, s in enumerate((sigma_x, sigma_px, sigma_y, sigma_py, sigma_tau, sigma_p)):
        rp[row] = rng.standard_normal(n) * s
    q = np.full(n, charge / n)
    return rp, q


def flat_top_beam(n: int, seed: int, length=2e-3, edge=100e-6, chirp=-10.0, sigma_xy=200e-6, tilt=1e-3,
                  sigma_pxy=1e-5, sigma_p=1e-4, charge=500e-12):
    """Low-energy stress shape: tau uniform over `length` convolved with a
    Gaussian edge of `edge` (a flat top with Gaussian edges), delta chirped by
    `chirp`*tau, transverse Gaussian with an x-tau tilt of `tilt`."""
    rng = np.random.default_rng(seed)
    rp = np.empty((6, n))
    tau = rng.uniform(-length / 2, length / 2, n) + rng.standard_normal(n) * edge
    rp[4] = tau
    rp[5] = rng.standard_normal(n) * sigma_p + chirp * tau
    rp[0] = rng.standard_normal(n) * sigma_xy + tilt * tau
    rp[2] = rng.standard_normal(n) * sigma_xy
    rp[1] = rng.standard_normal(n) * sigma_pxy
    rp[3] = rng.standard_normal(n) * sigma_pxy
    q = np.full(n, charge / n)
    return rp, q
