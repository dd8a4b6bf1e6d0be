"""Generate the committed golden fixtures for the space-charge kick.

Run in a container that holds the Ocelot reference checkout (it is not needed
anywhere else):

    python tests/golden/make_golden.py --reference <ocelot checkout> [--skip-track]

(or set OCELOT_REFERENCE to the checkout instead of passing --reference)

What it writes (all under tests/golden/):

* ``ref_<case>.npz`` -- seeded beams kicked by the reference's own
  ``SpaceCharge.apply`` (ocelot/cpbd/sc.py:208-251).  The reference's
  intermediates are captured by wrapping its public methods ``el_field``,
  ``potential`` and ``sym_kernel`` on the instance: the charge grid, the
  potential, the IGF octant, the mesh steps and the field at the particles.
* ``ref_track_kicks.npz`` -- input/output pairs of selected kicks of the
  reference's regression scenario ``test_track_with_sp``
  (unit_tests/ebeam_test/space_charge/space_charge_test.py:54-67, beam and
  lattice of space_charge_conf.py), captured while the reference tracks.
* ``ref_uni_matrix.npz`` -- first-order drift/quadrupole matrices of the
  reference's ``uni_matrix`` (ocelot/cpbd/r_matrix.py:41-91).
* ``ref_fodo_track.npz`` -- the reference's ``track()`` of a beam with
  ``SpaceCharge`` through FODO cells with first-order maps, with the kick
  positions and lengths its Navigator chose.
* ``ref_second_order.npz``, ``ref_fodo_track2.npz`` -- second-order
  tensors and maps (SecondTM) of drifts and quadrupoles and the reference's
  ``track()`` through FODO cells with SecondTM and SpaceCharge.
* ``ref_io.npz``, ``ref_beam.ast``, ``ref_beam.fmt1`` -- a seeded beam saved
  and loaded by the reference's ASTRA and CSRtrack adaptors.
* ``ref_navigator.npz`` -- the reference Navigator's steps (lengths,
  positions, processes applied and their step lengths) for lines with
  overlapping process ranges, gaps and three processes (passive processes).
* ``ref_cavity.npz`` -- sections of RF cavities (CavityTM, coupler kicks,
  tilt) applied by the reference to a seeded beam, with the energy before and
  after (elements/cavity_atom.py, transformations/cavity.py).
* ``ref_track_line.npz`` -- the reference's ``track()`` of the
  ``test_track_with_sp`` scenario (16 cavities, SecondTM, two SpaceCharge
  processes): its start beam, every kick's position, length, energy and
  process step, and the beam at the end.
* ``track_pin.json`` -- the pin of the oracle against the reference's golden
  vectors: the same scenario tracked by the reference's ``track()`` with the
  kick replaced by ``oracle.sc_oracle.sc_apply``, compared particle by
  particle with ref_results/test_track_with_sp.json at the reference test's
  own tolerance (1e-12 absolute).

The reference's import of ``pandas`` (not installed here, unused by the kick)
is satisfied by an empty stub module written to a temporary directory.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import sc_oracle  # noqa: E402


def import_reference(ref_root: str):
    stub = tempfile.mkdtemp(prefix="pandas_stub_")
    os.makedirs(os.path.join(stub, "pandas"))
    with open(os.path.join(stub, "pandas", "__init__.py"), "w") as f:
        f.write("class DataFrame:\n    pass\n\n\nclass Series:\n    pass\n")
    sys.path.insert(0, stub)
    sys.path.insert(0, ref_root)
    import logging
    logging.disable(logging.INFO)
    import ocelot  # noqa: F401
    return ocelot


# name: (n, nmesh, E_GeV, charge, dz, kicks, seed, random_mesh, beam overrides)
CASES = {
    "gauss_15": (3000, [15, 15, 15], 0.130, 250e-12, 0.1, 1, 101, False, {}),
    "aniso_low_energy": (5000, [13, 20, 33], 0.0065, 500e-12, 0.05, 1, 202, False,
                         dict(sigma_x=200e-6, sigma_y=200e-6, sigma_tau=700e-6)),
    "random_mesh": (2000, [15, 15, 15], 0.130, 250e-12, 0.1, 2, 303, True, {}),
    "multi_kick_31": (4000, [31, 31, 31], 0.130, 250e-12, 0.1, 3, 404, False, {}),
    "even_16": (2500, [16, 16, 16], 0.130, 1e-9, 0.1, 1, 505, False, {}),
}


def run_cases(ref_root: str):
    import_reference(ref_root)
    from ocelot.cpbd.sc import SpaceCharge
    from ocelot.cpbd.beam import ParticleArray

    for name, (n, nmesh, E, charge, dz, kicks, seed, rmesh, over) in CASES.items():
        rp, q = sc_oracle.gaussian_beam(n, seed, charge=charge, **over)
        pa = ParticleArray(n)
        pa.rparticles[:] = rp
        pa.q_array = q.copy()
        pa.E = E
        sc = SpaceCharge(step=1, nmesh_xyz=list(nmesh), random_mesh=rmesh)
        sc.prepare(None)  # seeds the global numpy RNG with 10 (sc.py:104-107)
        rec: dict = {}
        el_field = sc.el_field
        pot = sc.potential
        symk = sc.sym_kernel

        def el_field_rec(X, Q, gamma, nxyz):
            rec.setdefault("xyz_rot", []).append(np.array(X, copy=True))
            rec.setdefault("gamma0", []).append(gamma)
            out = el_field(X, Q, gamma, nxyz)
            rec.setdefault("Exyz", []).append(out.copy())
            return out

        def pot_rec(qg, steps):
            rec.setdefault("qgrid", []).append(qg.copy())
            rec.setdefault("steps", []).append(np.array(steps, copy=True))
            out = pot(qg, steps)
            rec.setdefault("phi", []).append(out.copy())
            return out

        def symk_rec(ijk2, hxyz):
            out = symk(ijk2, hxyz)
            rec.setdefault("igf", []).append(out.copy())
            return out

        sc.el_field, sc.potential, sc.sym_kernel = el_field_rec, pot_rec, symk_rec
        outs = []
        draws = []
        for _ in range(kicks):
            if rmesh:
                st = np.random.get_state()
                draws.append((np.random.uniform(low=1, high=1.1), np.random.uniform(low=-0.5, high=0.5)))
                np.random.set_state(st)
            sc.apply(pa, dz)
            outs.append(pa.rparticles.copy())
        data = dict(rp_in=rp, q=q, E=E, dz=dz, nmesh=np.array(nmesh), kicks=kicks,
                    random_mesh=rmesh, rp_out=np.stack(outs),
                    mesh_draws=np.array(draws) if draws else np.zeros((0, 2)))
        for k, v in rec.items():
            data[k] = np.stack([np.asarray(a) for a in v])
        path = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(path, **data)
        print(f"wrote {path} ({os.path.getsize(path) / 1e6:.2f} MB)")


def build_track_scenario(ref_root: str):
    """Lattice and beam of the reference's SC regression test.

    Restates the fixtures of unit_tests/ebeam_test/space_charge/space_charge_conf.py
    (lattice ``cell`` with SecondTM, beam ``p_array`` seeded with 11 and matched
    by BeamTransform) so the scenario can be rebuilt outside pytest.
    """
    sys.path.insert(0, os.path.join(ref_root, "unit_tests", "ebeam_test", "space_charge"))
    import space_charge_conf as conf
    from ocelot import (MagneticLattice, Marker, SecondTM, ParticleArray, Twiss, BeamTransform)

    cell = (Marker(), conf.D_14, conf.C_A1_1_1_I1, conf.D_15, conf.C_A1_1_2_I1, conf.D_15,
            conf.C_A1_1_3_I1, conf.D_15, conf.C_A1_1_4_I1, conf.D_15, conf.C_A1_1_5_I1, conf.D_15,
            conf.C_A1_1_6_I1, conf.D_15, conf.C_A1_1_7_I1, conf.D_15, conf.C_A1_1_8_I1, conf.D_22,
            conf.Q_37_I1, conf.D_23, conf.Q_38_I1)
    lattice = MagneticLattice(cell, method={'global': SecondTM})

    np.random.seed(11)
    n = 10000
    x = np.random.randn(n) * 0.000231507245956
    px = np.random.randn(n) * 0.000204206874319
    y = np.random.randn(n) * 0.000231583942392
    py = np.random.randn(n) * 0.000204272734636
    cov_t_p = [[6.89508231e-07, -2.98688604e-07], [-2.98688604e-07, 1.87434257e-07]]
    long_dist = np.random.multivariate_normal((0, 0), cov_t_p, n)
    p_array = ParticleArray(n=n)
    p_array.E = 0.0065
    p_array.rparticles[0] = x
    p_array.rparticles[1] = px
    p_array.rparticles[2] = y
    p_array.rparticles[3] = py
    p_array.rparticles[4] = long_dist[:, 0]
    p_array.rparticles[5] = long_dist[:, 1]
    p_array.q_array = np.ones(n) * 5e-10 / n
    tws = Twiss()
    tws.beta_x = 1.59966676201
    tws.beta_y = 1.60018325757
    tws.alpha_x = -0.995487979563
    tws.alpha_y = -0.996116091572
    tws.mux = 0.0
    tws.muy = 0.0
    BeamTransform(tws=tws).apply(p_array, dz=0.0)
    return lattice, p_array, conf


def track_scenario(ref_root: str, proc_factory, with_tws=False, **kw):
    from ocelot import Navigator, track
    lattice, p_array, conf = build_track_scenario(ref_root)
    sc1 = proc_factory(1)
    sc5 = proc_factory(5)
    navi = Navigator(lattice)
    navi.add_physics_proc(sc1, lattice.sequence[0], conf.C_A1_1_2_I1)
    navi.add_physics_proc(sc5, conf.C_A1_1_2_I1, lattice.sequence[-1])
    navi.unit_step = 0.02
    tws, p = track(lattice, p_array, navi, print_progress=False, **kw)
    return (tws, p) if with_tws else p


def run_track(ref_root: str, keep=(0, 120)):
    import_reference(ref_root)
    from ocelot.cpbd.sc import SpaceCharge
    from ocelot.cpbd.physics_proc import PhysProc

    golden = json.load(open(os.path.join(
        ref_root, "unit_tests/ebeam_test/space_charge/ref_results/test_track_with_sp.json")))["p_array"]
    gold = np.array([[d[k] for k in ("x", "px", "y", "py", "tau", "p")] for d in golden]).T

    kicks = []
    counter = [0]
    base_apply = SpaceCharge.apply

    def recording_apply(self, p_array, zstep):
        i = counter[0]
        counter[0] += 1
        rin = p_array.rparticles.copy()
        base_apply(self, p_array, zstep)
        if i in keep:
            kicks.append(dict(index=i, E=p_array.E, dz=zstep, rp_in=rin, rp_out=p_array.rparticles.copy(),
                              q=p_array.q_array.copy()))

    def make_ref(step):
        sc = SpaceCharge(step=step)
        sc.nmesh_xyz = [63, 63, 63]
        return sc

    SpaceCharge.apply = recording_apply
    t0 = time.time()
    p_ref = track_scenario(ref_root, make_ref)
    t_ref = time.time() - t0
    SpaceCharge.apply = base_apply
    n_kicks = counter[0]

    class OracleSC(PhysProc):
        def __init__(self, step):
            PhysProc.__init__(self, step)
            self.nmesh_xyz = [63, 63, 63]

        def prepare(self, lat):
            self.check_step()
            np.random.seed(10)

        def apply(self, p_array, zstep):
            sc_oracle.sc_apply(p_array.rparticles, p_array.q_array, p_array.E, zstep, self.nmesh_xyz)

    t0 = time.time()
    p_orc = track_scenario(ref_root, OracleSC)
    t_orc = time.time() - t0

    names = ("x", "px", "y", "py", "tau", "p")
    summary = {
        "scenario": "unit_tests/ebeam_test/space_charge/space_charge_test.py::test_track_with_sp",
        "golden": "unit_tests/ebeam_test/space_charge/ref_results/test_track_with_sp.json",
        "tolerance_abs": 1e-12,
        "n_particles": int(gold.shape[1]),
        "n_kicks": n_kicks,
        "reference_vs_golden_max_abs": {k: float(np.abs(p_ref.rparticles[i] - gold[i]).max()) for i, k in enumerate(names)},
        "oracle_vs_golden_max_abs": {k: float(np.abs(p_orc.rparticles[i] - gold[i]).max()) for i, k in enumerate(names)},
        "oracle_vs_reference_max_abs": {k: float(np.abs(p_orc.rparticles[i] - p_ref.rparticles[i]).max()) for i, k in enumerate(names)},
        "oracle_bit_identical_to_reference": bool(np.array_equal(p_orc.rparticles, p_ref.rparticles)),
        "seconds_reference": round(t_ref, 1),
        "seconds_oracle": round(t_orc, 1),
    }
    summary["oracle_pinned"] = all(v <= 1e-12 for v in summary["oracle_vs_golden_max_abs"].values())
    with open(os.path.join(HERE, "track_pin.json"), "w") as f:
        json.dump(summary, f, indent=1)
    print(json.dumps(summary, indent=1))
    data = {}
    for j, kk in enumerate(kicks):
        for k, v in kk.items():
            data[f"k{j}_{k}"] = v
    data["n_kept"] = len(kicks)
    path = os.path.join(HERE, "ref_track_kicks.npz")
    np.savez_compressed(path, **data)
    print(f"wrote {path} ({os.path.getsize(path) / 1e6:.2f} MB)")


def run_matrices(ref_root: str):
    """First-order matrices of drifts and quadrupoles from the reference's
    uni_matrix (ocelot/cpbd/r_matrix.py:41-91), for the transport between kicks."""
    import_reference(ref_root)
    from ocelot.cpbd.r_matrix import uni_matrix
    params = [(0.25, 0.0, 0.130), (1.0, 0.0, 0.130), (0.2, 1.2, 0.130), (0.2, -1.2, 0.130), (0.05, 1.2, 0.130),
              (0.15, -1.2, 0.0065), (0.3, -1.537886, 0.0065), (0.3, 1.435078, 2.0), (0.0, 1.2, 0.13)]
    R = np.stack([uni_matrix(z, k1, 0.0, 0.0, E) for z, k1, E in params])
    # a tilted, offset quadrupole section through the element's own first-order
    # parameters (elements/magnet.py:106-117, tm_params/first_order_params.py:26-28)
    from ocelot import Quadrupole
    quad = Quadrupole(l=0.2, k1=-1.2, tilt=0.3)
    quad.dx, quad.dy = 1e-3, -2e-3
    fp = quad.element.create_first_order_main_params(0.130, 0.15)
    path = os.path.join(HERE, "ref_uni_matrix.npz")
    np.savez_compressed(path, params=np.array(params), R=R, tilted_params=np.array([0.15, -1.2, 0.130, 0.3, 1e-3, -2e-3]),
                        tilted_R=fp.get_rotated_R(), tilted_B=np.asarray(fp.B).reshape(6))
    print(f"wrote {path}")


def run_fodo(ref_root: str, cells=2, n=4000, mesh=(15, 15, 15)):
    """The reference tracking a beam with SpaceCharge through FODO cells
    (quadrupoles of 0.2 m at k1 = +-1.2 m^-2, drifts of 1 m) with first-order
    maps, a kick every 0.25 m (Navigator unit_step 0.25, process step 1),
    through its own Navigator/track() (ocelot/cpbd/navi.py, track.py:431).
    The kick lengths and positions it used are recorded with the result."""
    import_reference(ref_root)
    from ocelot import Drift, Marker, Quadrupole, MagneticLattice, TransferMap, Navigator, track
    from ocelot.cpbd.sc import SpaceCharge
    from ocelot.cpbd.beam import ParticleArray
    seq = []
    for _ in range(cells):
        seq += [Quadrupole(l=0.2, k1=1.2), Drift(l=1.0), Quadrupole(l=0.2, k1=-1.2), Drift(l=1.0)]
    seq.append(Marker())
    lat = MagneticLattice(seq, method={"global": TransferMap})
    rp, q = sc_oracle.gaussian_beam(n, 606, sigma_x=200e-6, sigma_y=200e-6, sigma_px=2e-5, sigma_py=2e-5,
                                    charge=500e-12)
    pa = ParticleArray(n)
    pa.rparticles[:] = rp
    pa.q_array = q.copy()
    pa.E = 0.130
    sc = SpaceCharge(step=1, nmesh_xyz=list(mesh))
    kicks = []
    base_apply = SpaceCharge.apply

    def rec_apply(self, p_array, zstep):
        kicks.append((self.z0, zstep))
        base_apply(self, p_array, zstep)

    SpaceCharge.apply = rec_apply
    navi = Navigator(lat)
    navi.add_physics_proc(sc, lat.sequence[0], lat.sequence[-1])
    navi.unit_step = 0.25
    _, p = track(lat, pa, navi, print_progress=False, calc_tws=False)
    SpaceCharge.apply = base_apply
    path = os.path.join(HERE, "ref_fodo_track.npz")
    np.savez_compressed(path, rp_in=rp, q=q, E=0.130, cells=cells, nmesh=np.array(mesh),
                        kicks=np.array(kicks), rp_out=p.rparticles.copy())
    print(f"wrote {path} ({len(kicks)} kicks)")


def run_second_order(ref_root: str, cells=2, n=4000, mesh=(15, 15, 15)):
    """Second-order transport (SecondTM) of drifts and quadrupoles:
    the reference's t_nnn tensors (ocelot/cpbd/high_order.py:456-617), the
    offset and tilt handling of a quadrupole's SecondOrderParams, the maps
    applied by SecondTM.map_function to a small beam, and the reference's
    track() with SpaceCharge through FODO cells with method SecondTM."""
    import_reference(ref_root)
    from ocelot import Drift, Marker, Quadrupole, MagneticLattice, SecondTM, Navigator, track
    from ocelot.cpbd.high_order import t_nnn
    from ocelot.cpbd.sc import SpaceCharge
    from ocelot.cpbd.beam import ParticleArray
    params = [(0.25, 0.0, 0.130), (1.0, 0.0, 0.130), (0.2, 1.2, 0.130), (0.2, -1.2, 0.130), (0.05, 1.2, 0.130),
              (0.15, -1.2, 0.0065), (0.3, -1.537886, 0.0065), (0.3, 1.435078, 2.0)]
    T = np.stack([t_nnn(L, 0.0, k1, 0.0, E) for L, k1, E in params])
    quad = Quadrupole(l=0.2, k1=-1.2, tilt=0.3)
    quad.dx, quad.dy = 1e-3, -2e-3
    sp = quad.element.create_second_order_main_params(0.130, 0.15)
    # maps applied to a small beam by the reference's own SecondTM
    rng = np.random.default_rng(77)
    X0 = np.stack([rng.normal(0, s, 64) for s in (1e-3, 1e-4, 1e-3, 1e-4, 1e-4, 1e-3)])
    outs = []
    for e, dl in ((Drift(l=0.7), 0.7), (Quadrupole(l=0.2, k1=1.2), 0.2), (quad, 0.15)):
        tm = SecondTM.from_element(e.element if hasattr(e, "element") else e, delta_l=dl)
        outs.append(tm.map_function(X0.copy(), energy=0.130))
    path = os.path.join(HERE, "ref_second_order.npz")
    np.savez_compressed(path, params=np.array(params), T=T, quad=np.array([0.15, -1.2, 0.130, 0.3, 1e-3, -2e-3]),
                        quad_R=np.asarray(sp.R), quad_B=np.asarray(sp.B).reshape(6), quad_Rrot=sp.get_rotated_R(),
                        quad_Trot=sp.get_rotated_T(), X0=X0, X_drift=outs[0], X_quad=outs[1], X_tilted=outs[2])
    print(f"wrote {path}")
    seq = []
    for _ in range(cells):
        seq += [Quadrupole(l=0.2, k1=1.2), Drift(l=1.0), Quadrupole(l=0.2, k1=-1.2), Drift(l=1.0)]
    seq.append(Marker())
    lat = MagneticLattice(seq, method={"global": SecondTM})
    rp, q = sc_oracle.gaussian_beam(n, 607, sigma_x=200e-6, sigma_y=200e-6, sigma_px=2e-5, sigma_py=2e-5,
                                    charge=500e-12)
    pa = ParticleArray(n)
    pa.rparticles[:] = rp
    pa.q_array = q.copy()
    pa.E = 0.130
    sc = SpaceCharge(step=1, nmesh_xyz=list(mesh))
    navi = Navigator(lat)
    navi.add_physics_proc(sc, lat.sequence[0], lat.sequence[-1])
    navi.unit_step = 0.25
    _, p = track(lat, pa, navi, print_progress=False, calc_tws=False)
    path = os.path.join(HERE, "ref_fodo_track2.npz")
    np.savez_compressed(path, rp_in=rp, q=q, E=0.130, cells=cells, nmesh=np.array(mesh), rp_out=p.rparticles.copy())
    print(f"wrote {path}")


def run_io(ref_root: str, n=64):
    """Beam files written and read by the reference's adaptors
    (ocelot/cpbd/io.py:223-295, ocelot/adaptors/astra2ocelot.py:150-233,
    ocelot/adaptors/csrtrack2ocelot.py:9-87), from a seeded beam."""
    import_reference(ref_root)
    from ocelot.cpbd.beam import ParticleArray
    from ocelot.cpbd.io import load_particle_array, save_particle_array
    rp, q = sc_oracle.gaussian_beam(n, 909, sigma_x=80e-6, sigma_y=60e-6, sigma_px=3e-5, sigma_py=2e-5,
                                    sigma_tau=50e-6, sigma_p=2e-4, charge=100e-12)
    pa = ParticleArray(n)
    pa.rparticles[:] = rp
    pa.q_array = q.copy()
    pa.E = 0.130
    pa.s = 12.5
    ast = os.path.join(HERE, "ref_beam.ast")
    fmt1 = os.path.join(HERE, "ref_beam.fmt1")
    save_particle_array(ast, pa)
    save_particle_array(fmt1, pa)
    a = load_particle_array(ast)
    c = load_particle_array(fmt1)
    path = os.path.join(HERE, "ref_io.npz")
    np.savez_compressed(path, rp=rp, q=q, E=0.130, s=12.5, ast_rp=a.rparticles, ast_q=a.q_array, ast_E=a.E,
                        ast_s=a.s, fmt1_rp=c.rparticles, fmt1_q=c.q_array, fmt1_E=c.E, fmt1_s=c.s)
    print(f"wrote {path}, {ast}, {fmt1}")


CAVITY_CASES = [
    # (l, v, phi, freq, couplers (vx_up, vy_up, vxx_up, vxy_up, vx_down, vy_down, vxx_down, vxy_down), tilt, E)
    (1.0377, 18.50662e-3 / np.cos(18.7268 * np.pi / 180.0), 18.7268, 1.3e9, (0,) * 8, 0.0, 0.0065),
    (0.346, -20.2E-3 / 8.0 / np.cos(np.pi), 180.0, 3.9e9, (0,) * 8, 0.0, 0.13),
    (1.0377, 1e-3, 90.0, 1.3e9, (0,) * 8, 0.0, 0.05),
    (0.8, 0.0, 10.0, 1.3e9, (0,) * 8, 0.0, 0.02),
    (1.0377, 0.02, -30.0, 1.3e9, (1e-3 + 2e-3j, -5e-4 + 1e-4j, 2e-3 - 1e-3j, 1e-3 + 3e-3j,
                                   -1e-3 + 5e-4j, 3e-4 - 2e-4j, -2e-3 + 1e-3j, 5e-4 - 1e-3j), 0.05, 0.01),
]
# (start in the element, length) of the sections taken through each cavity
CAVITY_SECTIONS = [(0.0, 0.02), (0.0, None), (0.3, 0.02), (None, 0.02), (0.5, 0.1)]


def run_cavity(ref_root: str, n=64):
    """Sections of RF cavities (CavityTM with its coupler kicks) applied by
    the reference to a seeded beam: the maps OpticElement.get_section_tms
    builds, each applied by Transformation.apply (which also raises p_array.E)."""
    import_reference(ref_root)
    from ocelot import Cavity, ParticleArray
    rng = np.random.default_rng(21)
    data = {"n_cases": len(CAVITY_CASES), "n_sections": len(CAVITY_SECTIONS)}
    for c, (l, v, phi, freq, cp, tilt, E) in enumerate(CAVITY_CASES):
        cav = Cavity(l=l, v=v, phi=phi, freq=freq, vx_up=cp[0], vy_up=cp[1], vxx_up=cp[2], vxy_up=cp[3],
                     vx_down=cp[4], vy_down=cp[5], vxx_down=cp[6], vxy_down=cp[7], eid=f"C{c}")
        cav.tilt = tilt
        data[f"c{c}_params"] = np.array([l, v, phi, freq, tilt, E])
        data[f"c{c}_couplers"] = np.array(cp, dtype=np.complex128)
        for k, (start, dl) in enumerate(CAVITY_SECTIONS):
            start = l - dl if start is None else start
            dl = l if dl is None else dl
            X = np.stack([rng.normal(0, 1e-3, n), rng.normal(0, 1e-4, n), rng.normal(0, 1e-3, n),
                          rng.normal(0, 1e-4, n), rng.normal(0, 1e-3, n), rng.normal(0, 1e-2, n)])
            pa = ParticleArray(n=n)
            pa.E = E
            pa.rparticles[:] = X
            for tm in cav.get_section_tms(start_l=start, delta_l=dl):
                tm.apply(pa)
            data[f"c{c}_s{k}_section"] = np.array([start, dl])
            data[f"c{c}_s{k}_in"] = X
            data[f"c{c}_s{k}_out"] = pa.rparticles.copy()
            data[f"c{c}_s{k}_E"] = np.array([E, pa.E])
    path = os.path.join(HERE, "ref_cavity.npz")
    np.savez_compressed(path, **data)
    print(f"wrote {path} ({os.path.getsize(path) / 1e6:.3f} MB)")


TWISS_KEYS = ["E", "q", "s", "p", "x", "y", "px", "py", "tau", "xx", "xpx", "pxpx", "yy", "ypy", "pypy", "tautau",
              "xy", "pxpy", "xpy", "ypx", "pp", "emit_x", "emit_y", "emit_xn", "emit_yn", "eigemit_1", "eigemit_2",
              "beta_x", "beta_y", "alpha_x", "alpha_y"]


def run_track_line(ref_root: str):
    """The reference's test_track_with_sp scenario (16 cavities, SecondTM,
    two SpaceCharge processes of step 1 and 5) tracked by the reference's own
    track(): the beam it starts from, every kick's position, length, energy
    and process, and the particles and energy at the end."""
    import_reference(ref_root)
    from ocelot.cpbd.sc import SpaceCharge
    lattice, p0, conf = build_track_scenario(ref_root)
    start = p0.rparticles.copy()
    rec = []
    base_apply = SpaceCharge.apply

    def recording_apply(self, p_array, zstep):
        rec.append((self.step, self.z0, zstep, p_array.E))
        base_apply(self, p_array, zstep)

    def make_ref(step):
        sc = SpaceCharge(step=step)
        sc.nmesh_xyz = [63, 63, 63]
        return sc

    from ocelot.cpbd.beam.analysis import get_envelope
    bounded = []

    def both_envelopes(p_array, bounds=None, slice=None, auto_disp=False):
        bounded.append(get_envelope(p_array, bounds=[-0.5, 0.5]))
        return get_envelope(p_array, bounds=bounds, slice=slice, auto_disp=auto_disp)

    SpaceCharge.apply = recording_apply
    try:
        tws, p = track_scenario(ref_root, make_ref, with_tws=True, get_twiss=both_envelopes)
    finally:
        SpaceCharge.apply = base_apply
    seq = lattice.sequence
    keys = TWISS_KEYS
    twiss = np.array([[float(np.real(getattr(t, k))) for k in keys] for t in tws])
    twiss_b = np.array([[float(np.real(getattr(t, k))) for k in keys] for t in bounded])
    twiss_b[:, keys.index("s")] = twiss[:, keys.index("s")]
    data = dict(rp_start=start, q=p0.q_array.copy(), E_start=np.array(0.0065), rp_end=p.rparticles.copy(),
                E_end=np.array(p.E), s_end=np.array(p.s),
                kick_step=np.array([r[0] for r in rec], dtype=np.int32), kick_z0=np.array([r[1] for r in rec]),
                kick_zstep=np.array([r[2] for r in rec]), kick_E=np.array([r[3] for r in rec]),
                lengths=np.array([e.l for e in seq]),
                # per element: kind (0 drift/marker, 1 quadrupole, 2 cavity), l, k1, v, phi, freq
                elements=np.array([[2 if type(e).__name__ == "Cavity" else 1 if type(e).__name__ == "Quadrupole" else 0,
                                    e.l, getattr(e, "k1", 0.0), getattr(e, "v", 0.0), getattr(e, "phi", 0.0),
                                    getattr(e, "freq", 0.0)] for e in seq]),
                indx=np.array([seq.index(conf.C_A1_1_2_I1), len(seq) - 1], dtype=np.int32),
                # get_envelope after every step (track()'s twiss list), and with bounds [-0.5, 0.5]
                twiss_keys=np.array(keys), twiss=twiss, twiss_bounds=twiss_b)
    path = os.path.join(HERE, "ref_track_line.npz")
    np.savez_compressed(path, **data)
    print(f"wrote {path} ({os.path.getsize(path) / 1e6:.2f} MB), {len(rec)} kicks")


def run_track_mixed(ref_root: str, n=5000, mesh=(31, 31, 31)):
    """A short line with first-order transport (TransferMap), an RF cavity,
    quadrupoles and two SpaceCharge processes of different step counts,
    tracked by the reference's own track(): the start and end beams, the
    energy and position at the end, every kick, and the twiss list."""
    import_reference(ref_root)
    from ocelot import (Cavity, Drift, Marker, MagneticLattice, Navigator, Quadrupole, TransferMap, track)
    from ocelot.cpbd.sc import SpaceCharge
    c = Cavity(l=0.5, v=0.005, phi=20.0, freq=1.3e9, eid="C")
    q1 = Quadrupole(l=0.2, k1=2.0, eid="Q1")
    q2 = Quadrupole(l=0.2, k1=-2.0, eid="Q2")
    m_end = Marker(eid="END")
    seq = [Marker(eid="START"), Drift(l=0.3), c, Drift(l=0.2), q1, Drift(l=0.5), q2, Drift(l=0.3), m_end]
    lat = MagneticLattice(seq, method={"global": TransferMap})
    rp, q = sc_oracle.gaussian_beam(n, seed=5, sigma_x=3e-4, sigma_px=2e-5, sigma_y=2e-4, sigma_py=3e-5,
                                    sigma_tau=5e-4, sigma_p=1e-3, charge=300e-12)
    from ocelot import ParticleArray
    pa = ParticleArray(n=n)
    pa.rparticles[:] = rp
    pa.q_array = q.copy()
    pa.E = 0.02
    start = rp.copy()
    sc_a = SpaceCharge(step=2)
    sc_a.nmesh_xyz = list(mesh)
    sc_b = SpaceCharge(step=3)
    sc_b.nmesh_xyz = list(mesh)
    navi = Navigator(lat)
    navi.add_physics_proc(sc_a, seq[0], q1)
    navi.add_physics_proc(sc_b, q1, m_end)
    navi.unit_step = 0.05
    rec = []
    base_apply = SpaceCharge.apply

    def recording_apply(self, p_array, zstep):
        rec.append((self.step, self.z0, zstep, p_array.E))
        base_apply(self, p_array, zstep)

    SpaceCharge.apply = recording_apply
    try:
        tws, p = track(lat, pa, navi, print_progress=False)
    finally:
        SpaceCharge.apply = base_apply
    keys = TWISS_KEYS
    data = dict(rp_start=start, q=q, E_start=np.array(0.02), rp_end=p.rparticles.copy(), E_end=np.array(p.E),
                s_end=np.array(p.s), nmesh=np.array(mesh), unit_step=np.array(0.05),
                kick_step=np.array([r[0] for r in rec], dtype=np.int32), kick_z0=np.array([r[1] for r in rec]),
                kick_zstep=np.array([r[2] for r in rec]), kick_E=np.array([r[3] for r in rec]),
                elements=np.array([[2 if type(e).__name__ == "Cavity" else 1 if type(e).__name__ == "Quadrupole" else 0,
                                    e.l, getattr(e, "k1", 0.0), getattr(e, "v", 0.0), getattr(e, "phi", 0.0),
                                    getattr(e, "freq", 0.0)] for e in seq]),
                indx=np.array([seq.index(q1), len(seq) - 1], dtype=np.int32),
                twiss_keys=np.array(keys), twiss=np.array([[float(np.real(getattr(t, k))) for k in keys] for t in tws]))
    path = os.path.join(HERE, "ref_track_mixed.npz")
    np.savez_compressed(path, **data)
    print(f"wrote {path} ({os.path.getsize(path) / 1e6:.2f} MB), {len(rec)} kicks")


NAVIGATOR_CASES = [
    # (element lengths, [(indx0, indx1, step)], unit_step): overlapping ranges, a gap, three processes,
    # a range ending before the lattice does
    ([0.0, 0.5, 0.3, 1.0, 0.2, 0.7, 0.0], [(0, 3, 2), (2, 6, 3)], 0.05),
    ([0.0, 0.4, 0.25, 0.6, 0.35, 0.5, 0.0], [(1, 3, 1), (4, 5, 2)], 0.1),
    ([0.0, 0.3, 0.3, 0.45, 0.15, 0.9, 0.2, 0.0], [(0, 7, 1), (0, 3, 4), (2, 5, 2)], 0.07),
    ([0.1, 0.2, 0.3, 0.4, 0.5], [(0, 3, 3)], 0.033),
]


def run_navigator(ref_root: str):
    """The reference Navigator's steps (get_next_step: step length, position
    after the step, processes applied with their step lengths) for lines with
    several processes, with passive processes (no physics)."""
    import_reference(ref_root)
    from ocelot import Drift, MagneticLattice, Marker, Navigator
    from ocelot.cpbd.physics_proc import PhysProc
    data = {"n_cases": len(NAVIGATOR_CASES)}
    for c, (lengths, procs, unit) in enumerate(NAVIGATOR_CASES):
        seq = [Marker(eid=f"M{i}") if L == 0 else Drift(l=L, eid=f"D{i}") for i, L in enumerate(lengths)]
        lat = MagneticLattice(seq)
        navi = Navigator(lat)
        objs = []
        for a, b, st in procs:
            p = PhysProc(step=st)
            navi.add_physics_proc(p, seq[a], seq[b])
            objs.append(p)
        navi.unit_step = unit
        rows = []
        for _, dz, plist, psteps in navi.get_next_step():
            ids = [next(k for k, o in enumerate(objs) if o is p) for p in plist]
            rows.append((float(dz), float(navi.z0), ids, [float(v) for v in psteps]))
        data[f"c{c}_lengths"] = np.array(lengths)
        data[f"c{c}_procs"] = np.array(procs, dtype=np.int64)
        data[f"c{c}_unit"] = np.array(unit)
        data[f"c{c}_dz"] = np.array([r[0] for r in rows])
        data[f"c{c}_z0"] = np.array([r[1] for r in rows])
        data[f"c{c}_nkick"] = np.array([len(r[2]) for r in rows], dtype=np.int64)
        data[f"c{c}_kick_proc"] = np.array([k for r in rows for k in r[2]], dtype=np.int64)
        data[f"c{c}_kick_dz"] = np.array([v for r in rows for v in r[3]])
    path = os.path.join(HERE, "ref_navigator.npz")
    np.savez_compressed(path, **data)
    print(f"wrote {path} ({os.path.getsize(path) / 1e3:.1f} kB)")


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("OCELOT_REFERENCE"),
                    help="the Ocelot checkout to import (default: $OCELOT_REFERENCE)")
    ap.add_argument("--skip-track", action="store_true")
    ap.add_argument("--only-track", action="store_true")
    ap.add_argument("--only-matrices", action="store_true")
    ap.add_argument("--only-second-order-io", action="store_true")
    ap.add_argument("--only-cavity", action="store_true")
    a = ap.parse_args()
    if not a.reference:
        ap.error("--reference (or OCELOT_REFERENCE) must name the Ocelot checkout")
    if a.only_cavity:
        run_navigator(a.reference)
        run_cavity(a.reference)
        run_track_mixed(a.reference)
        run_track_line(a.reference)
        sys.exit(0)
    if a.only_second_order_io:
        run_second_order(a.reference)
        run_io(a.reference)
        sys.exit(0)
    if a.only_matrices:
        run_matrices(a.reference)
        if not os.path.exists(os.path.join(HERE, "ref_fodo_track.npz")):
            run_fodo(a.reference)
        sys.exit(0)
    if not a.only_track:
        run_cases(a.reference)
        run_matrices(a.reference)
        run_fodo(a.reference)
        run_second_order(a.reference)
        run_io(a.reference)
        run_navigator(a.reference)
        run_cavity(a.reference)
    if not a.skip_track:
        run_track(a.reference)
        run_track_mixed(a.reference)
        run_track_line(a.reference)
