"""Standing-wave RF cavities for device tracking: the element, the slice maps
and the energy gain, computed on the host once per tracking job.

A slice of a cavity is applied by the reference as CavityTM.map4cav
(ocelot/cpbd/transformations/cavity.py:29-128): the first-order map of the
slice (CavityAtom._R_main_matrix, ocelot/cpbd/elements/cavity_atom.py:93-179,
rotated by the tilt as FirstOrderParams.get_rotated_R,
tm_params/first_order_params.py:26-28), then a nonlinear update of the
longitudinal coordinates from their values before the slice.  The entrance
and exit coupler kicks are first-order maps (cavity_atom.py:63-91, 181-201),
and every main slice raises the reference energy by create_delta_e
(cavity_atom.py:215-220), which Transformation.apply adds to p_array.E
(transformations/transformation.py:123-130).

The scalars are evaluated here with the reference's expressions and numpy
functions, in its order of operations, so they are the reference's values;
the device applies them per particle (``sc_slices_apply``, record layout in
the C header: R, B, then E, beta0, E1 beta1, V beta0 / (E1 beta1), k, phi,
cos(phi), T566, T556, T555, the positive-energy flag, 1 / (E1 beta1), sin(phi)
and whether R has the pattern of cavity_R_z).
"""
from __future__ import annotations

import numpy as np

from . import _native as N
from .globals import m_e_GeV, speed_of_light

MAP2_DOUBLES = N.SC_MAP2_DOUBLES
SLICE_MAP = N.SC_SLICE_MAP
SLICE_CAVITY = N.SC_SLICE_CAVITY
SLICE_MAP_PLANAR = N.SC_SLICE_MAP_PLANAR
SLICE_MAP_DRIFT = N.SC_SLICE_MAP_DRIFT
SLICE_MAP_LINEAR = N.SC_SLICE_MAP_LINEAR


def _pair(j, k):
    return j * 6 - j * (j - 1) // 2 + (k - j)


def _pattern(r_entries, t_entries):
    mask = np.zeros(MAP2_DOUBLES, dtype=bool)
    for r, k in r_entries:
        mask[r * 6 + k] = True
    mask[36:42] = True
    for r, (j, k) in t_entries:
        mask[42 + r * 21 + _pair(j, k)] = True
    return mask


# the fixed patterns of the device's straight-line map forms (the C header's SC_SLICE_MAP_PLANAR / _DRIFT)
_PLANAR = _pattern([(0, 0), (0, 1), (1, 0), (1, 1), (2, 2), (2, 3), (3, 2), (3, 3), (4, 4), (4, 5), (5, 5)],
                   [(0, (0, 5)), (0, (1, 5)), (1, (0, 5)), (1, (1, 5)), (2, (2, 5)), (2, (3, 5)), (3, (2, 5)),
                    (3, (3, 5)), (4, (0, 0)), (4, (0, 1)), (4, (1, 1)), (4, (2, 2)), (4, (2, 3)), (4, (3, 3)),
                    (4, (5, 5))])
_DRIFT = _pattern([(0, 0), (0, 1), (1, 1), (2, 2), (2, 3), (3, 3), (4, 4), (4, 5), (5, 5)],
                  [(0, (1, 5)), (2, (3, 5)), (4, (1, 1)), (4, (3, 3)), (4, (5, 5))])


# the R pattern of cavity_R_z (x and y blocks, longitudinal 2x2 block)
_CAV_R = np.zeros((6, 6), dtype=bool)
for _r, _k in ((0, 0), (0, 1), (1, 0), (1, 1), (2, 2), (2, 3), (3, 2), (3, 3), (4, 4), (4, 5), (5, 4), (5, 5)):
    _CAV_R[_r, _k] = True


def map_kind(record) -> int:
    """The device form for a map record: first-order in the quadrupole
    pattern, the drift or quadrupole pattern when every non-zero entry lies
    in it, the general form otherwise."""
    nz = np.asarray(record).reshape(-1) != 0.0
    if not np.any(nz[42:]) and not np.any(nz & ~_PLANAR):
        return SLICE_MAP_LINEAR
    if not np.any(nz & ~_DRIFT):
        return SLICE_MAP_DRIFT
    if not np.any(nz & ~_PLANAR):
        return SLICE_MAP_PLANAR
    return SLICE_MAP
(CAV_E, CAV_BETA0, CAV_DEN, CAV_A, CAV_K, CAV_PHI, CAV_COSPHI, CAV_T566, CAV_T556, CAV_T555, CAV_RF, CAV_RDEN,
 CAV_SINPHI, CAV_RPAT) = range(42, 56)


class Cavity:
    """Standing-wave RF cavity (the reference's Cavity/CavityAtom attributes):
    l [m], v [GV], phi [deg], freq [Hz], coupler kicks vx/vy (zero order) and
    vxx/vxy (first order) up- and downstream (complex allowed), tilt [rad]."""

    def __init__(self, l=0., v=0., phi=0., freq=0., vx_up=0, vy_up=0, vxx_up=0, vxy_up=0,
                 vx_down=0, vy_down=0, vxx_down=0, vxy_down=0, tilt=0.0, eid=None):
        self.l = float(l)
        self.v = v
        self.phi = phi
        self.freq = freq
        self.vx_up, self.vy_up, self.vxx_up, self.vxy_up = vx_up, vy_up, vxx_up, vxy_up
        self.vx_down, self.vy_down, self.vxx_down, self.vxy_down = vx_down, vy_down, vxx_down, vxy_down
        self.tilt = float(tilt)
        self.dx = 0.0
        self.dy = 0.0
        self.id = eid


def is_cavity(e) -> bool:
    return type(e).__name__ == "Cavity"


def _rot(angle) -> np.ndarray:
    # rot_mtx (ocelot/cpbd/r_matrix.py:11-19)
    cs, sn = np.cos(angle), np.sin(angle)
    return np.array([[cs, 0., sn, 0., 0., 0.],
                     [0., cs, 0., sn, 0., 0.],
                     [-sn, 0., cs, 0., 0., 0.],
                     [0., -sn, 0., cs, 0., 0.],
                     [0., 0., 0., 0., 1., 0.],
                     [0., 0., 0., 0., 0., 1.]])


def _rotated(R: np.ndarray, tilt) -> np.ndarray:
    return np.dot(np.dot(_rot(-tilt), R), _rot(tilt))


def cavity_R_z(z, V, E, freq, phi=0.):
    """First-order matrix of a cavity section of length z [m] and voltage V
    [GV] entered at energy E [GeV] (cavity_atom.py:95-172: the Rosenzweig-
    Serafini transverse matrix for a pi-mode standing wave and the
    longitudinal terms R55, R56, R65, R66)."""
    phi = phi * np.pi / 180.
    de = V * np.cos(phi)
    eta = 1
    Ei = E / m_e_GeV
    Ef = (E + de) / m_e_GeV
    Ep = (Ef - Ei) / z
    if Ei == 0:
        raise ValueError("cavity: the initial energy is 0")
    cos_phi = np.cos(phi)
    alpha = np.sqrt(eta / 8.) / cos_phi * np.log(Ef / Ei)
    sin_alpha = np.sin(alpha)
    cos_alpha = np.cos(alpha)
    r11 = (cos_alpha - np.sqrt(2. / eta) * cos_phi * sin_alpha)
    if abs(Ep) > 1e-10:
        r12 = np.sqrt(8. / eta) * Ei / Ep * cos_phi * sin_alpha
    else:
        r12 = z
    r21 = -Ep / Ef * (cos_phi / np.sqrt(2. * eta) + np.sqrt(eta / 8.) / cos_phi) * sin_alpha
    r22 = Ei / Ef * (cos_alpha + np.sqrt(2. / eta) * cos_phi * sin_alpha)
    r56 = 0.
    beta0 = 1
    beta1 = 1
    k = 2. * np.pi * freq / speed_of_light
    r55_cor = 0.
    if V != 0 and E != 0:
        gamma2 = Ei * Ei
        beta0 = np.sqrt(1. - 1 / gamma2)
        gamma2 = Ef * Ef
        beta1 = np.sqrt(1. - 1 / gamma2)
        r56 = - z / (Ef * Ef * Ei * beta1) * (Ef + Ei) / (beta1 + beta0)
        g0 = Ei
        g1 = Ef
        zero_energy_gain = abs(g1 - g0) < 1e-8 * abs(g0)
        if zero_energy_gain and abs(cos_phi) < 1e-3:
            r55_cor = -k * z * V / (2.0 * m_e_GeV * g0 ** 3 * beta0 ** 2)
        else:
            r55_cor = (k * z * beta0 * V / m_e_GeV * np.sin(phi)
                       * (g0 * g1 * (beta0 * beta1 - 1.0) + 1.0)
                       / (beta1 * g1 * (g0 - g1) ** 2))
    r66 = Ei / Ef * beta0 / beta1
    r65 = k * np.sin(phi) * V / (Ef * beta1 * m_e_GeV)
    return np.array([[r11, r12, 0., 0., 0., 0.],
                     [r21, r22, 0., 0., 0., 0.],
                     [0., 0., r11, r12, 0., 0.],
                     [0., 0., r21, r22, 0., 0.],
                     [0., 0., 0., 0., 1. + r55_cor, r56],
                     [0., 0., 0., 0., r65, r66]]).real


def main_matrix(e, length, energy) -> np.ndarray:
    """R of a section of ``length`` (CavityAtom._R_main_matrix: a drift
    matrix, tilted, when v = 0; the voltage scaled by length / l otherwise)."""
    if e.v == 0.:
        from .track import first_order_matrix
        R = first_order_matrix(length, 0.0, energy)
        if e.tilt != 0:
            R = _rotated(R, e.tilt)
        return R
    return cavity_R_z(length, V=e.v * length / e.l, E=energy, freq=e.freq, phi=e.phi)


def edge_map(e, energy, upstream: bool):
    """(R, B) of the entrance (upstream) or exit coupler kick at ``energy``
    (cavity_atom.py:63-91 ck_matrix, 181-186 kick_b), R rotated by the tilt."""
    vxx, vxy = (e.vxx_up, e.vxy_up) if upstream else (e.vxx_down, e.vxy_down)
    vx, vy = (e.vx_up, e.vy_up) if upstream else (e.vx_down, e.vy_down)
    phi = e.phi * np.pi / 180.
    m21 = (vxx * e.v * np.exp(1j * phi)).real / energy
    m43 = - m21
    m23 = (vxy * e.v * np.exp(1j * phi)).real / energy
    R = np.array([[1, 0., 0., 0., 0., 0.],
                  [m21, 1, m23, 0., 0., 0.],
                  [0., 0., 1, 0., 0., 0.],
                  [m23, 0., m43, 1, 0., 0.],
                  [0., 0., 0., 0., 1., 0.],
                  [0., 0., 0., 0., 0., 1]])
    dxp = (vx * e.v * np.exp(1j * phi)).real / energy
    dyp = (vy * e.v * np.exp(1j * phi)).real / energy
    B = np.array([0., dxp, 0., dyp, 0., 0.])
    return _rotated(R, e.tilt), B


def delta_e(e, delta_length):
    """Reference-energy gain of a main slice (create_delta_e; None = the
    whole cavity built as one map)."""
    if delta_length is not None:
        phase_term = np.cos(e.phi * np.pi / 180.)
        return phase_term * e.v * delta_length / e.l if e.l != 0 else phase_term * e.v
    return e.v * np.cos(e.phi * np.pi / 180.)


def slice_record(e, delta_length, energy) -> np.ndarray:
    """Device record of a main slice entered at ``energy`` [GeV]; delta_length
    None is the whole cavity built as one map (map4cav's V and z then are
    v and l)."""
    length = e.l
    R0 = main_matrix(e, delta_length if delta_length is not None else e.l, energy)
    R = _rotated(R0, e.tilt)
    # Element._default_B (elements/element.py:80-81), from the unrotated R
    B = np.dot((np.eye(6) - R0), np.array([[e.dx], [0.], [e.dy], [0.], [0.], [0.]])).reshape(-1)
    if delta_length is not None:
        V = e.v * delta_length / length if length != 0 else e.v
        z = delta_length
    else:
        V = e.v
        z = length
    E = energy
    beta0, igamma2, g0 = 1.0, 0.0, 1e10
    if E != 0.0:
        g0 = E / m_e_GeV
        igamma2 = 1.0 / (g0 * g0)
        beta0 = np.sqrt(1.0 - igamma2)
    phi = e.phi * np.pi / 180.0
    E1 = E + V * np.cos(phi)
    T566 = 1.5 * z * igamma2 / (beta0 ** 3)
    T556 = 0.0
    T555 = 0.0
    out = np.zeros(MAP2_DOUBLES)
    out[:36] = R.reshape(-1)
    out[36:42] = B
    out[CAV_RPAT] = 0.0 if np.any((R != 0.0) & ~_CAV_R) else 1.0
    out[CAV_T566] = T566
    if E1 <= 0.0:
        out[CAV_RF] = 0.0
        return out
    k = 2.0 * np.pi * e.freq / speed_of_light
    g1 = E1 / m_e_GeV
    beta1 = np.sqrt(1.0 - 1.0 / (g1 * g1))
    dgamma = V / m_e_GeV
    dg = g1 - g0
    if abs(dg) < 1e-8 * abs(g0):
        if abs(np.cos(phi)) < 1e-3:
            T556 = 1.5 * z * k * dgamma / (beta0 ** 3 * g0 ** 3)
            T555 = 0.5 * z * k * k * dgamma * dgamma / (beta0 ** 3 * g0 ** 4)
    else:
        T566 = (z * (beta0 ** 3 * g0 ** 3 - beta1 ** 3 * g1 ** 3)
                / (2.0 * beta0 * beta1 ** 3 * g0 * (g0 - g1) * g1 ** 3))
        T556 = (beta0 * k * z * dgamma * g0 * (beta1 ** 3 * g1 ** 3 + beta0 * (g0 - g1 ** 3)) * np.sin(phi) /
                (beta1 ** 3 * g1 ** 3 * (g0 - g1) ** 2))
        T555 = (beta0 ** 2 * k ** 2 * z * dgamma / 2.0
                * (dgamma * (2.0 * g0 * g1 ** 3 * (beta0 * beta1 ** 3 - 1.0)
                             + g0 ** 2 + 3.0 * g1 ** 2 - 2.0) / (beta1 ** 3 * g1 ** 3 * (g0 - g1) ** 3) * np.sin(phi) ** 2
                   - (g1 * g0 * (beta1 * beta0 - 1.0) + 1.0)
                   / (beta1 * g1 * (g0 - g1) ** 2)
                   * np.cos(phi)))
    out[CAV_E] = E
    out[CAV_BETA0] = beta0
    out[CAV_DEN] = E1 * beta1
    out[CAV_A] = V * beta0 / (E1 * beta1)
    out[CAV_K] = k
    out[CAV_PHI] = phi
    out[CAV_COSPHI] = np.cos(phi)
    out[CAV_SINPHI] = np.sin(phi)
    out[CAV_RDEN] = 1.0 / (E1 * beta1)
    out[CAV_T566] = T566
    out[CAV_T556] = T556
    out[CAV_T555] = T555
    out[CAV_RF] = 1.0
    return out


def section_tms(e, start_l: float, delta_l: float, has_edge: bool):
    """The maps OpticElement.get_section_tms builds for a section of ``e``
    starting at ``start_l`` [m] of length ``delta_l`` (optic_element.py:376-415):
    [(kind, delta_length)], kind "entrance" | "main" | "exit", delta_length
    None for the whole element built as one map."""
    total = e.l
    out = []
    if start_l < 1e-10:
        if has_edge:
            out.append(("entrance", None))
        if np.isclose(delta_l, total):
            out.append(("main", None))
            if has_edge:
                out.append(("exit", None))
            return out
    if start_l + delta_l > total or np.isclose(start_l + delta_l, total):
        out.append(("main", total - start_l))
        if has_edge:
            out.append(("exit", None))
    else:
        out.append(("main", delta_l))
    return out


def section_records(e, start_l: float, delta_l: float, energy):
    """Device records of a cavity section (section_tms) entered at ``energy``:
    (records [m, MAP2_DOUBLES], kinds [m], energy after it).  A coupler kick
    that is the identity is left out: the reference's R.x + B with R = I and
    B = 0 returns x exactly."""
    from .second_order import pack_map
    recs, kinds = [], []
    E = energy
    for kind, d in section_tms(e, start_l, delta_l, True):
        if kind == "main":
            recs.append(slice_record(e, d, E))
            kinds.append(SLICE_CAVITY)
            E = E + delta_e(e, d)
        else:
            R, B = edge_map(e, E, kind == "entrance")
            if not (np.array_equal(R, np.eye(6)) and not np.any(B)):
                recs.append(pack_map(R, np.zeros((6, 6, 6)), B))
                kinds.append(map_kind(recs[-1]))
    return np.array(recs).reshape(-1, MAP2_DOUBLES), kinds, E


def apply_records_numpy(records: np.ndarray, kinds, X: np.ndarray) -> np.ndarray:
    """The device's per-particle evaluation of a table of records, in numpy
    (host-side check of the records; R.x as a sum over the inputs in index
    order like the kernel's FMA chain, up to the FMA roundings)."""
    X = np.array(X, dtype=np.float64, copy=True)
    for rec, kind in zip(np.asarray(records).reshape(-1, MAP2_DOUBLES), kinds):
        R = rec[:36].reshape(6, 6)
        B = rec[36:42]
        x4, x5 = X[4].copy(), X[5].copy()
        Y = R @ X + B[:, None]
        if kind == SLICE_CAVITY:
            if rec[CAV_RF] != 0.0:
                beta0 = rec[CAV_BETA0]
                Y[5] = (x5 * rec[CAV_E] * beta0 / rec[CAV_DEN]
                        + rec[CAV_A] * (np.cos(-x4 * beta0 * rec[CAV_K] + rec[CAV_PHI]) - rec[CAV_COSPHI]))
                Y[4] += rec[CAV_T566] * x5 * x5 + rec[CAV_T556] * x4 * x5 + rec[CAV_T555] * x4 * x4
            else:
                Y[4] += rec[CAV_T566] * x5 * x5
        else:
            Tc = rec[42:].reshape(6, 21)
            q = 0
            for j in range(6):
                for k in range(j, 6):
                    Y += Tc[:, q][:, None] * (X[j] * X[k])[None, :]
                    q += 1
        X = Y
    return X
