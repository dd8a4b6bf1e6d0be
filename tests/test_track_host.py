"""Host side of device tracking (CPU only): first-order matrices against the
reference's uni_matrix outputs, and the Navigator kick schedule against the
reference's own FODO run."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import sc_oracle
from ocelot_gb300 import track as T


def _fodo(cells):
    seq = []
    for _ in range(cells):
        seq += [T.Quadrupole(l=0.2, k1=1.2), T.Drift(l=1.0), T.Quadrupole(l=0.2, k1=-1.2), T.Drift(l=1.0)]
    return seq + [T.Marker()]


def test_first_order_matrix_matches_reference_uni_matrix():
    d = np.load(os.path.join(GOLDEN, "ref_uni_matrix.npz"))
    for (z, k1, E), R in zip(d["params"], d["R"]):
        M = T.first_order_matrix(z, k1, E)
        assert np.allclose(M, R, rtol=2e-15, atol=1e-17), (z, k1, E, np.abs(M - R).max())


def test_tilted_offset_quadrupole_section_matches_reference():
    d = np.load(os.path.join(GOLDEN, "ref_uni_matrix.npz"))
    dl, k1, E, tilt, dx, dy = d["tilted_params"]
    q = T.Quadrupole(l=0.2, k1=k1, tilt=tilt)
    q.dx, q.dy = dx, dy
    R, B = T.element_map(q, dl, E)
    assert np.allclose(R, d["tilted_R"], rtol=1e-14, atol=1e-17)
    assert np.allclose(B, d["tilted_B"], rtol=1e-12, atol=1e-20)


def test_oracle_matrices_bit_identical_to_reference():
    d = np.load(os.path.join(GOLDEN, "ref_uni_matrix.npz"))
    for (z, k1, E), R in zip(d["params"], d["R"]):
        assert np.array_equal(sc_oracle.uni_matrix(z, k1, E), R)


def test_kick_schedule_is_the_reference_navigators():
    f = np.load(os.path.join(GOLDEN, "ref_fodo_track.npz"))
    seq = _fodo(int(f["cells"]))
    sched = T.kick_schedule([e.l for e in seq], 0.25)
    assert np.array_equal(np.array([(z0, dz) for _, dz, z0 in sched]), f["kicks"])
    ref = sc_oracle.navigator_schedule([e.l for e in seq], 0.25)
    assert [s for s, _, _ in sched] == [s for s, _, _ in ref]


@pytest.mark.parametrize("unit_step,step", [(0.1, 1), (0.25, 2), (0.07, 3), (1.0, 1), (0.3, 5)])
def test_kick_schedule_other_steps_equal_oracle(unit_step, step):
    seq = _fodo(3)
    a = T.kick_schedule([e.l for e in seq], unit_step, step)
    b = sc_oracle.navigator_schedule([e.l for e in seq], unit_step, step)
    assert a == b
    assert abs(sum(dz for _, dz, _ in a) - 7.2) < 1e-9


def test_oracle_fodo_track_bit_identical_to_reference():
    f = dict(np.load(os.path.join(GOLDEN, "ref_fodo_track.npz")))
    els = [(e.l, e.k1) for e in _fodo(int(f["cells"]))]
    rp = f["rp_in"].copy()
    kicks = sc_oracle.track_first_order(rp, f["q"], float(f["E"]), els, 0.25, [int(v) for v in f["nmesh"]])
    assert np.array_equal(np.array(kicks), f["kicks"])
    assert np.array_equal(rp, f["rp_out"])


def test_composed_step_maps_equal_sequential_slices():
    seq = _fodo(2)
    E = 0.13
    rng = np.random.default_rng(3)
    X = rng.standard_normal((6, 50)) * 1e-4
    Y = X.copy()
    for (R, B, _, _), (slices, _, _) in zip(T.step_maps(seq, E, 0.25), T.kick_schedule([e.l for e in seq], 0.25)):
        X = R @ X + B[:, None]
        for i, dl in slices:
            if dl:
                Y = sc_oracle.uni_matrix(dl, seq[i].k1, E) @ Y
    assert np.allclose(X, Y, rtol=1e-13, atol=1e-19)


def test_unsupported_elements_and_ranges_raise():
    class SBend:
        l, angle, k1 = 1.0, 0.1, 0.0

    with pytest.raises(NotImplementedError):
        T.step_maps([T.Drift(1.0), SBend(), T.Marker()], 0.1, 0.25)
    with pytest.raises(ValueError):
        T.kick_schedule([1.0], 0.25)
    with pytest.raises(ValueError):
        T.kick_schedule([], 0.25)
