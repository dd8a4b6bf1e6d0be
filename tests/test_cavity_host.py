"""RF cavity sections and the Navigator's schedule with several processes, on
the host, against the reference's own outputs (tests/golden/ref_cavity.npz,
ref_track_line.npz; tests/golden/make_golden.py wrote them)."""
from __future__ import annotations

import os

import numpy as np
import pytest

from conftest import GOLDEN
from ocelot_gb300 import cavity as CV
from ocelot_gb300 import track as T

CAV = dict(np.load(os.path.join(GOLDEN, "ref_cavity.npz")))
LINE = dict(np.load(os.path.join(GOLDEN, "ref_track_line.npz")))


def cavity_case(c):
    l, v, phi, freq, tilt, E = (float(x) for x in CAV[f"c{c}_params"])
    cp = [complex(x) for x in CAV[f"c{c}_couplers"]]
    cav = CV.Cavity(l=l, v=v, phi=phi, freq=freq, vx_up=cp[0], vy_up=cp[1], vxx_up=cp[2], vxy_up=cp[3],
                    vx_down=cp[4], vy_down=cp[5], vxx_down=cp[6], vxy_down=cp[7], tilt=tilt)
    return cav, E


def sections():
    return [(c, k) for c in range(int(CAV["n_cases"])) for k in range(int(CAV["n_sections"]))]


def close_rows(a, b, rtol):
    """max |a - b| per row within rtol of the row's largest |b|."""
    return all(np.abs(a[r] - b[r]).max() <= rtol * np.abs(b[r]).max() for r in range(6))


MIXED = dict(np.load(os.path.join(GOLDEN, "ref_track_mixed.npz")))


def line_elements(fixture=None):
    seq = []
    for kind, l, k1, v, phi, freq in (LINE if fixture is None else fixture)["elements"]:
        if kind == 2:
            seq.append(CV.Cavity(l=l, v=v, phi=phi, freq=freq))
        elif kind == 1:
            seq.append(T.Quadrupole(l=l, k1=k1))
        elif l == 0:
            seq.append(T.Marker())
        else:
            seq.append(T.Drift(l=l))
    return seq


def line_procs():
    i4, i20 = (int(v) for v in LINE["indx"])
    return [(0, i4, 1), (i4, i20, 5)]


def mixed_procs():
    i_q1, i_end = (int(v) for v in MIXED["indx"])
    return [(0, i_q1, 2), (i_q1, i_end, 3)]


@pytest.mark.parametrize("c,k", sections())
def test_cavity_section_records_match_reference(c, k):
    cav, E = cavity_case(c)
    start, dl = (float(v) for v in CAV[f"c{c}_s{k}_section"])
    recs, kinds, E1 = CV.section_records(cav, start, dl, E)
    assert E1 == CAV[f"c{c}_s{k}_E"][1]          # the energy gain, bit for bit
    out = CV.apply_records_numpy(recs, kinds, CAV[f"c{c}_s{k}_in"])
    assert close_rows(out, CAV[f"c{c}_s{k}_out"], 1e-13)


def test_cavity_sections_cover_the_branches():
    # accelerating, decelerating (180 deg), zero-crossing (90 deg: the T556/T555 limits), v = 0 (drift
    # matrix), couplers + tilt
    kinds_seen = set()
    for c in range(int(CAV["n_cases"])):
        cav, E = cavity_case(c)
        recs, kinds, _ = CV.section_records(cav, 0.0, cav.l, E)
        kinds_seen.add(tuple(kinds))
        rec = recs[kinds.index(CV.SLICE_CAVITY)]
        if c == 2:
            assert rec[CV.CAV_T556] != 0.0 and rec[CV.CAV_T555] != 0.0
        if c == 3:
            assert rec[CV.CAV_T556] == 0.0 and rec[CV.CAV_T555] == 0.0
    assert (CV.SLICE_MAP, CV.SLICE_CAVITY, CV.SLICE_MAP) in kinds_seen    # coupler kicks kept
    assert (CV.SLICE_CAVITY,) in kinds_seen                              # identity edges left out


def test_section_tms_edges_follow_reference_convention():
    cav = CV.Cavity(l=1.0, v=0.01, phi=10.0, freq=1.3e9)
    assert CV.section_tms(cav, 0.0, 1.0, True) == [("entrance", None), ("main", None), ("exit", None)]
    assert CV.section_tms(cav, 0.0, 0.2, True) == [("entrance", None), ("main", 0.2)]
    assert CV.section_tms(cav, 0.4, 0.2, True) == [("main", 0.2)]
    assert CV.section_tms(cav, 0.9, 0.2, True) == [("main", 1.0 - 0.9), ("exit", None)]


def test_navigator_steps_one_process_equals_kick_schedule():
    seq = []
    for _ in range(3):
        seq += [T.Quadrupole(l=0.2, k1=1.2), T.Drift(l=1.0), T.Quadrupole(l=0.2, k1=-1.2), T.Drift(l=1.0)]
    seq.append(T.Marker())
    lengths = [e.l for e in seq]
    for unit_step, step in ((0.25, 1), (0.1, 3), (0.07, 2)):
        a = T.kick_schedule(lengths, unit_step, step)
        b = T.navigator_steps(lengths, [(0, len(seq) - 1, step)], unit_step)
        assert len(a) == len(b)
        for (sl_a, zstep, z0a), (sec_b, kicks, z0b, _) in zip(a, b):
            assert z0a == z0b and kicks == [(0, zstep)]
            assert sl_a == [(i, T._section_length(lengths[i], s, d)) for i, s, d in sec_b]


def test_line_schedule_and_energies_are_the_reference_navigators():
    """test_track_with_sp's line: 16 cavities, SpaceCharge with step 1 up to
    the second cavity and step 5 after it -- every kick's position, length,
    energy and process equal to the reference's, bit for bit."""
    seq = line_elements()
    procs = line_procs()
    steps = T.navigator_steps([e.l for e in seq], procs, 0.02)
    slices, E_end, s_end = T.step_slices(seq, float(LINE["E_start"]), steps, order=2)
    kicks = [(procs[j][2], st.z0, zstep, E) for st in slices for j, E, zstep in st.kicks]
    assert len(kicks) == len(LINE["kick_step"]) == 193
    assert [k[0] for k in kicks] == list(LINE["kick_step"])
    assert np.array_equal([k[1] for k in kicks], LINE["kick_z0"])
    assert np.array_equal([k[2] for k in kicks], LINE["kick_zstep"])
    assert np.array_equal([k[3] for k in kicks], LINE["kick_E"])
    assert E_end == LINE["E_end"]
    assert s_end == LINE["s_end"]                   # p_array.s as Transformation.apply moves it
    assert len(slices[-1].kicks) == 0               # the last quadrupole: transport only, no process


def test_navigator_steps_reject_kick_processes_and_bad_ranges():
    with pytest.raises(NotImplementedError):
        T.navigator_steps([1.0, 1.0, 1.0], [(1, 1, 1)], 0.1)
    with pytest.raises(NotImplementedError):
        T.navigator_steps([0.0, 1.0, 1.0], [(0, 1, 1)], 0.1)
    with pytest.raises(ValueError):
        T.navigator_steps([1.0, 1.0], [(0, 5, 1)], 0.1)
    with pytest.raises(ValueError):
        T.navigator_steps([], [(0, 0, 1)], 0.1)


def _twiss_row(t, keys):
    return np.array([float(getattr(t, k)) for k in keys])


_CROSS = {"xpx": ("xx", "pxpx"), "ypy": ("yy", "pypy"), "xy": ("xx", "yy"), "pxpy": ("pxpx", "pypy"),
          "xpy": ("xx", "pypy"), "ypx": ("yy", "pxpx")}


def twiss_close(ours, ref, keys, rtol=1e-9, eig_rtol=1e-7, derived_rtol=None):
    """Twiss rows against the reference's: the means within rtol of the
    beam size and the correlations within rtol of the product of the two rms
    sizes (both are near zero), eigen-emittances within eig_rtol (they are
    computed by another method here), emittances, beta and alpha within
    derived_rtol (they amplify the moments' differences: an emittance by
    about 1 + alpha^2), the rest within rtol."""
    k = list(keys)
    bad = []
    for j, name in enumerate(k):
        a, b = ours[j], ref[j]
        if name in ("x", "px", "y", "py", "tau", "p"):
            scale = np.sqrt(abs(ref[k.index({"x": "xx", "px": "pxpx", "y": "yy", "py": "pypy", "tau": "tautau",
                                              "p": "pp"}[name])]))
            ok = abs(a - b) <= rtol * scale
        elif name.startswith("eigemit"):
            ok = abs(a - b) <= eig_rtol * abs(b)
        elif name in _CROSS:
            # a correlation: relative to the product of the two rms sizes
            u, v = _CROSS[name]
            ok = abs(a - b) <= rtol * np.sqrt(abs(ref[k.index(u)] * ref[k.index(v)]))
        elif name.startswith("alpha"):
            ok = abs(a - b) <= (derived_rtol or rtol) * (abs(b) + 1.0)
        elif name.startswith(("emit", "beta")):
            ok = abs(a - b) <= (derived_rtol or rtol) * abs(b)
        else:
            ok = abs(a - b) <= rtol * abs(b)
        if not ok:
            bad.append((name, a, b))
    return bad


def test_envelope_of_start_and_end_beams_matches_reference():
    from ocelot_gb300.envelope import moments_numpy, twiss_from_moments
    keys = [str(k) for k in LINE["twiss_keys"]]
    q = float(np.sum(LINE["q"]))
    for rp, E, row, s in ((LINE["rp_start"], float(LINE["E_start"]), 0, 0.0),
                          (LINE["rp_end"], float(LINE["E_end"]), -1, float(LINE["twiss"][-1][keys.index("s")]))):
        for bounds, table in ((None, LINE["twiss"]), ([-0.5, 0.5], LINE["twiss_bounds"])):
            t = twiss_from_moments(moments_numpy(rp, bounds), E, q, s)
            assert not twiss_close(_twiss_row(t, keys), table[row], keys, rtol=1e-12, eig_rtol=1e-8)


def test_twiss_positions_and_energies_are_the_reference_tracks():
    keys = [str(k) for k in LINE["twiss_keys"]]
    seq = line_elements()
    steps = T.navigator_steps([e.l for e in seq], line_procs(), 0.02)
    slices, _, _ = T.step_slices(seq, float(LINE["E_start"]), steps, order=2)
    L, s, E = 0., [0.0], [float(LINE["E_start"])]
    for st in slices:
        L += st.dz
        s.append(0.0 + L)
        E.append(st.E)
    assert np.array_equal(s, LINE["twiss"][:, keys.index("s")])
    assert np.array_equal(E, LINE["twiss"][:, keys.index("E")])


def test_mixed_line_schedule_energies_and_positions_are_the_reference_tracks():
    """First-order transport, a cavity and two processes (step 2 up to the
    first quadrupole, step 3 after it): kicks, energies, s and the twiss
    positions bit for bit."""
    keys = [str(k) for k in MIXED["twiss_keys"]]
    seq = line_elements(MIXED)
    procs = mixed_procs()
    steps = T.navigator_steps([e.l for e in seq], procs, float(MIXED["unit_step"]))
    slices, E_end, s_end = T.step_slices(seq, float(MIXED["E_start"]), steps, order=1)
    kicks = [(procs[j][2], st.z0, zstep, E) for st in slices for j, E, zstep in st.kicks]
    assert [k[0] for k in kicks] == list(MIXED["kick_step"])
    assert np.array_equal([k[1] for k in kicks], MIXED["kick_z0"])
    assert np.array_equal([k[2] for k in kicks], MIXED["kick_zstep"])
    assert np.array_equal([k[3] for k in kicks], MIXED["kick_E"])
    assert E_end == MIXED["E_end"] and s_end == MIXED["s_end"]
    L, s = 0., [0.0]
    for st in slices:
        L += st.dz
        s.append(0.0 + L)
    assert np.array_equal(s, MIXED["twiss"][:, keys.index("s")])
    # first-order records only: the slices carry no second-order terms
    assert all(not st.table[st.kinds != CV.SLICE_CAVITY][:, 42:].any() for st in slices)


def test_map_kinds_follow_the_element_patterns():
    from ocelot_gb300.second_order import element_map2, pack_map
    zero_t = np.zeros((6, 6, 6))
    E = 0.05
    drift = T.Drift(l=0.3)
    quad = T.Quadrupole(l=0.2, k1=1.7)
    dquad = T.Quadrupole(l=0.2, k1=-1.7)
    tilted = T.Quadrupole(l=0.2, k1=1.7, tilt=0.1)
    offset = T.Quadrupole(l=0.2, k1=1.7)
    offset.dx = 1e-4
    assert CV.map_kind(pack_map(*element_map2(drift, 0.3, E))) == CV.SLICE_MAP_DRIFT
    assert CV.map_kind(pack_map(*element_map2(quad, 0.2, E))) == CV.SLICE_MAP_PLANAR
    assert CV.map_kind(pack_map(*element_map2(dquad, 0.05, E))) == CV.SLICE_MAP_PLANAR
    assert CV.map_kind(pack_map(*element_map2(tilted, 0.2, E))) == CV.SLICE_MAP
    assert CV.map_kind(pack_map(*element_map2(offset, 0.2, E))) == CV.SLICE_MAP
    R, B = T.element_map(quad, 0.2, E)
    assert CV.map_kind(pack_map(R, zero_t, B)) == CV.SLICE_MAP_LINEAR
    R, B = T.element_map(drift, 0.3, E)
    assert CV.map_kind(pack_map(R, zero_t, B)) == CV.SLICE_MAP_LINEAR
    cav = CV.Cavity(l=1.0, v=0.01, phi=10.0, freq=1.3e9, vxx_up=1e-3)
    _, kinds, _ = CV.section_records(cav, 0.0, 1.0, E)
    assert kinds == [CV.SLICE_MAP_LINEAR, CV.SLICE_CAVITY]   # vxx: R10 and R32, inside the pattern
    cav = CV.Cavity(l=1.0, v=0.01, phi=10.0, freq=1.3e9, vxy_up=1e-3)
    _, kinds, _ = CV.section_records(cav, 0.0, 1.0, E)
    assert kinds == [CV.SLICE_MAP, CV.SLICE_CAVITY]          # vxy couples x and y


def test_navigator_steps_match_the_reference_navigator_with_several_processes():
    """Overlapping process ranges, a gap, three processes, a range that ends
    before the lattice does: every step's length, the position after it, the
    processes applied and their step lengths equal the reference Navigator's
    (ref_navigator.npz, passive processes), bit for bit."""
    nav = dict(np.load(os.path.join(GOLDEN, "ref_navigator.npz")))
    for c in range(int(nav["n_cases"])):
        procs = [tuple(int(v) for v in p) for p in nav[f"c{c}_procs"]]
        steps = T.navigator_steps(list(nav[f"c{c}_lengths"]), procs, float(nav[f"c{c}_unit"]))
        assert len(steps) == len(nav[f"c{c}_dz"]), c
        assert np.array_equal([st[3] for st in steps], nav[f"c{c}_dz"]), c
        assert np.array_equal([st[2] for st in steps], nav[f"c{c}_z0"]), c
        assert [len(st[1]) for st in steps] == list(nav[f"c{c}_nkick"]), c
        assert [j for st in steps for j, _ in st[1]] == list(nav[f"c{c}_kick_proc"]), c
        assert np.array_equal([z for st in steps for _, z in st[1]], nav[f"c{c}_kick_dz"]), c


@pytest.mark.parametrize("seed", range(12))
def test_navigator_steps_random_lines_equal_the_oracle(seed):
    """One process over random lines (zero-length elements included, the
    last a marker) and random unit steps: the Navigator restatement of the
    device loop equals the oracle's, position by position."""
    from oracle import sc_oracle
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 12))
    lengths = [0.0 if rng.random() < 0.2 else float(rng.uniform(0.01, 1.5)) for _ in range(n)] + [0.0]
    unit = float(rng.uniform(0.01, 0.4))
    step = int(rng.integers(1, 4))
    ref = sc_oracle.navigator_schedule(lengths, unit, step)
    got = T.navigator_steps(lengths, [(0, len(lengths) - 1, step)], unit)
    assert len(got) == len(ref)
    for (slices, zstep, z0), (sections, kicks, z0b, _) in zip(ref, got):
        assert z0 == z0b and kicks == [(0, zstep)]
        assert slices == [(i, T._section_length(lengths[i], s, d)) for i, s, d in sections]
