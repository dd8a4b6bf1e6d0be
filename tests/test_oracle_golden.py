"""The oracle against the reference's own outputs (CPU only).

The fixtures ``ref_*.npz`` were produced by the reference's SpaceCharge
(ocelot/cpbd/sc.py) on seeded beams; ``track_pin.json`` records the oracle
reproducing the reference's regression vectors of test_track_with_sp.
"""
import glob
import json
import os

import numpy as np
import pytest

from oracle import sc_oracle

from conftest import GOLDEN

CASES = sorted(glob.glob(os.path.join(GOLDEN, "ref_*.npz")))
# the kick fixtures (the others hold transport, tracking and beam-file outputs)
NOT_KICKS = ("ref_track_kicks.npz", "ref_uni_matrix.npz", "ref_fodo_track.npz", "ref_fodo_track2.npz",
             "ref_second_order.npz", "ref_io.npz", "ref_cavity.npz", "ref_track_line.npz",
             "ref_track_mixed.npz", "ref_navigator.npz")
CASES = [c for c in CASES if os.path.basename(c) not in NOT_KICKS]


def _load(path):
    return dict(np.load(path, allow_pickle=False))


@pytest.mark.parametrize("path", CASES, ids=[os.path.basename(c)[4:-4] for c in CASES])
def test_oracle_bit_identical_to_reference(path):
    d = _load(path)
    rp = d["rp_in"].copy()
    nmesh = [int(v) for v in d["nmesh"]]
    for k in range(int(d["kicks"])):
        rec = {}
        draws = d["mesh_draws"][k] if bool(d["random_mesh"]) else (None, None)
        sc_oracle.sc_apply(rp, d["q"], float(d["E"]), float(d["dz"]), nmesh,
                           mesh_scale=draws[0], mesh_shift=draws[1], record=rec)
        # intermediates of the reference, captured on its own instance
        assert np.array_equal(rec["steps"], d["steps"][k])
        assert np.array_equal(rec["qgrid"], d["qgrid"][k])
        assert np.array_equal(rec["phi"], d["phi"][k])
        assert np.array_equal(rec["Exyz"], d["Exyz"][k])
        assert np.array_equal(sc_oracle.igf_kernel(nmesh, rec["steps"]), d["igf"][k])
        assert np.array_equal(rp, d["rp_out"][k])


def test_oracle_pinned_to_reference_track_golden():
    """test_track_with_sp: 10k particles, 194 kicks, SecondTM transport.

    The record tests/golden/make_golden.py wrote when it ran the oracle's
    kicks inside the reference's own track() (which needs the reference
    checkout); test_oracle_retracks_the_reference_regression_line recomputes
    the line here without it.
    """
    s = json.load(open(os.path.join(GOLDEN, "track_pin.json")))
    assert s["n_kicks"] > 100 and s["n_particles"] == 10000
    for k, v in s["oracle_vs_golden_max_abs"].items():
        assert v <= s["tolerance_abs"], (k, v)
    assert s["oracle_pinned"]


def test_oracle_retracks_the_reference_regression_line():
    """test_track_with_sp's line (16 cavities, SecondTM, SpaceCharge with step
    1 up to the second cavity and step 5 after it; 10k particles, 193 kicks at
    63^3) tracked again here: the Navigator's schedule and the slice maps on
    the host (numpy), every kick by the oracle.  The particles must end within
    the reference test's own tolerance (1e-12 absolute, space_charge_test.py:65)
    of the reference's own track() of the same beam."""
    from test_cavity_host import LINE, line_elements, line_procs

    from ocelot_gb300 import cavity as CV
    from ocelot_gb300 import track as T
    seq, procs = line_elements(), line_procs()
    steps = T.navigator_steps([e.l for e in seq], procs, 0.02)
    slices, _, _ = T.step_slices(seq, float(LINE["E_start"]), steps, order=2)
    X = np.array(LINE["rp_start"], dtype=np.float64)
    kicks = 0
    for st in slices:
        if len(st.kinds):
            X = CV.apply_records_numpy(st.table, st.kinds, X)
        for _, E, zstep in st.kicks:
            sc_oracle.sc_apply(X, LINE["q"], E, zstep, [63, 63, 63])
            kicks += 1
    assert kicks == 193
    assert np.abs(X - LINE["rp_end"]).max() <= 1e-12


def test_track_kick_fixture_replays_on_oracle():
    d = _load(os.path.join(GOLDEN, "ref_track_kicks.npz"))
    for j in range(int(d["n_kept"])):
        rp = d[f"k{j}_rp_in"].copy()
        sc_oracle.sc_apply(rp, d[f"k{j}_q"], float(d[f"k{j}_E"]), float(d[f"k{j}_dz"]), [63, 63, 63])
        assert np.array_equal(rp, d[f"k{j}_rp_out"])


def test_zero_step_is_a_no_op():
    rp, q = sc_oracle.gaussian_beam(100, 1)
    r0 = rp.copy()
    sc_oracle.sc_apply(rp, q, 0.13, 0.0, [15, 15, 15])
    assert np.array_equal(rp, r0)


def test_tmap_matches_dot_plus_offset():
    rng = np.random.default_rng(5)
    rp = rng.standard_normal((6, 1000))
    R = rng.standard_normal((6, 6))
    B = rng.standard_normal((6, 1))
    ref = R @ rp + B
    sc_oracle.tmap_apply(rp, R, B)
    assert np.array_equal(rp, ref)
