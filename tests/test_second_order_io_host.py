"""Second-order transport maps and beam files on the host, against outputs of
the reference generated by tests/golden/make_golden.py.

* second_order_tensor vs the reference's t_nnn (ocelot/cpbd/high_order.py:456-617)
  for drifts and quadrupoles of both signs at 6.5 MeV-2 GeV: within 1e-16
  absolute (the same operations; one coefficient differs by one rounding).
* a tilted, offset quadrupole slice: R, rotated T and B equal to the
  reference's SecondOrderParams (get_rotated_R, get_rotated_T, B).
* the maps applied to a small beam (R.X + T:XX + B) equal the reference's
  SecondTM.map_function outputs bit for bit.
* ASTRA and CSRtrack files written by the reference load to the reference's
  arrays bit for bit, and files written here are byte-identical to the
  reference's; npz round trips.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from ocelot_gb300 import ParticleArray
from ocelot_gb300 import io as bio
from ocelot_gb300.second_order import MAP2_DOUBLES, element_map2, pack_map, second_order_tensor
from ocelot_gb300.track import Drift, Quadrupole, lattice_order

SO = dict(np.load(os.path.join(GOLDEN, "ref_second_order.npz")))
IO = dict(np.load(os.path.join(GOLDEN, "ref_io.npz")))


def _apply(R, T, B, X):
    # SecondOrderMult.numpy_apply, then the offset (second_order.py:31-38)
    return R @ X + np.einsum("ijk,j...,k...->i...", T, X, X) + B[:, None]


@pytest.mark.parametrize("idx", range(8))
def test_tensor_matches_reference(idx):
    L, k1, E = SO["params"][idx]
    T = second_order_tensor(L, 0.0, k1, 0.0, E)
    assert np.max(np.abs(T - SO["T"][idx])) <= 1e-16


def test_tilted_offset_quadrupole_slice_matches_reference():
    L, k1, E, tilt, dx, dy = SO["quad"]
    q = Quadrupole(l=0.2, k1=k1, tilt=tilt)
    q.dx, q.dy = dx, dy
    R, T, B = element_map2(q, L, E)
    assert np.max(np.abs(R - SO["quad_Rrot"])) <= 1e-15
    assert np.max(np.abs(T - SO["quad_Trot"])) <= 1e-16
    assert np.max(np.abs(B - SO["quad_B"])) <= 1e-18


def test_maps_on_a_beam_match_reference():
    q = Quadrupole(l=0.2, k1=SO["quad"][1], tilt=SO["quad"][3])
    q.dx, q.dy = SO["quad"][4], SO["quad"][5]
    for name, (e, dl) in (("X_drift", (Drift(l=0.7), 0.7)), ("X_quad", (Quadrupole(l=0.2, k1=1.2), 0.2)),
                          ("X_tilted", (q, 0.15))):
        R, T, B = element_map2(e, dl, 0.130)
        assert np.array_equal(_apply(R, T, B, SO["X0"]), SO[name]), name


def test_packed_map_layout():
    R, T, B = element_map2(Quadrupole(l=0.2, k1=1.2), 0.2, 0.130)
    m = pack_map(R, T, B)
    assert m.shape == (MAP2_DOUBLES,)
    assert np.array_equal(m[:36], R.reshape(-1)) and np.array_equal(m[36:42], B)
    x = np.array([1e-3, 2e-4, -5e-4, 1e-4, 3e-5, -2e-4])
    q, quad = 0, np.zeros(6)
    for j in range(6):
        for k in range(j, 6):
            quad += m[42 + np.arange(6) * 21 + q] * x[j] * x[k]
            q += 1
    assert np.allclose(quad, np.einsum("ijk,j,k->i", T, x, x), rtol=1e-14, atol=1e-30)


def test_lattice_order_follows_the_method():
    class SecondTM:
        pass

    class Lat:
        method = {"global": SecondTM}

    assert lattice_order(Lat()) == 2
    assert lattice_order([Drift(l=1.0)]) == 1


def test_astra_file_loads_like_the_reference():
    p = bio.load_particle_array(os.path.join(GOLDEN, "ref_beam.ast"))
    assert np.array_equal(p.rparticles, IO["ast_rp"])
    assert np.array_equal(p.q_array, IO["ast_q"])
    assert p.E == IO["ast_E"] and p.s == IO["ast_s"]


def test_csrtrack_file_loads_like_the_reference():
    p = bio.load_particle_array(os.path.join(GOLDEN, "ref_beam.fmt1"))
    assert np.array_equal(p.rparticles, IO["fmt1_rp"])
    assert np.array_equal(p.q_array, IO["fmt1_q"])
    assert p.E == IO["fmt1_E"] and p.s == IO["fmt1_s"]


def _beam():
    pa = ParticleArray(IO["rp"].shape[1])
    pa.rparticles[:] = IO["rp"]
    pa.q_array = IO["q"].copy()
    pa.E = float(IO["E"])
    pa.s = float(IO["s"])
    return pa


@pytest.mark.parametrize("ext", [".ast", ".fmt1"])
def test_files_written_are_the_references(tmp_path, ext):
    out = tmp_path / ("beam" + ext)
    bio.save_particle_array(str(out), _beam())
    ref = os.path.join(GOLDEN, "ref_beam" + ext)
    assert out.read_bytes() == open(ref, "rb").read()


def test_npz_round_trip(tmp_path):
    out = str(tmp_path / "beam.npz")
    bio.save_particle_array(out, _beam())
    p = bio.load_particle_array(out)
    assert np.array_equal(p.rparticles, IO["rp"]) and np.array_equal(p.q_array, IO["q"])
    assert float(p.E) == float(IO["E"]) and float(p.s) == float(IO["s"])


def test_unknown_extension_raises(tmp_path):
    with pytest.raises(ValueError):
        bio.load_particle_array(str(tmp_path / "beam.txt"))
    with pytest.raises(ValueError):
        bio.save_particle_array(str(tmp_path / "beam.txt"), _beam())
