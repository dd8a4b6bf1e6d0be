"""RF cavities on the device: the cavity slice records through
``sc_slices_apply`` against the reference's sections, and the reference's
space-charge regression line (test_track_with_sp: 16 cavities, SecondTM, two
SpaceCharge processes) tracked end to end on the GPU against the reference's
own track() of it (tests/golden/ref_track_line.npz)."""
from __future__ import annotations

import ctypes as C
import types

import numpy as np
import pytest

from conftest import has_gpu
from test_cavity_host import (CAV, LINE, MIXED, cavity_case, close_rows, line_elements, line_procs, mixed_procs,
                              sections)

pytestmark = pytest.mark.gpu
if not has_gpu():
    pytest.skip("needs a CUDA device", allow_module_level=True)

import torch  # noqa: E402

from ocelot_gb300 import ParticleArray, SpaceCharge  # noqa: E402
from ocelot_gb300 import _native as N  # noqa: E402
from ocelot_gb300 import cavity as CV  # noqa: E402
from ocelot_gb300 import track as T  # noqa: E402

# the reference test's own tolerance on the particles (space_charge_test.py:65)
TOL_ABS = 1e-12


def slices_apply(recs, kinds, X):
    dev = torch.device("cuda", 0)
    rp = torch.from_numpy(np.ascontiguousarray(X)).to(dev)
    maps = torch.from_numpy(np.ascontiguousarray(recs)).to(dev)
    kd = torch.tensor(list(kinds), dtype=torch.int32, device=dev)
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    N.check(N.lib().sc_slices_apply(C.c_void_p(maps.data_ptr()), C.c_void_p(kd.data_ptr()), len(kinds),
                                    C.c_void_p(rp.data_ptr()), rp.stride(0), rp.shape[1], s))
    torch.cuda.synchronize()
    return rp.cpu().numpy()


@pytest.mark.parametrize("c,k", sections())
def test_cavity_sections_on_device_match_reference(c, k):
    cav, E = cavity_case(c)
    start, dl = (float(v) for v in CAV[f"c{c}_s{k}_section"])
    recs, kinds, _ = CV.section_records(cav, start, dl, E)
    out = slices_apply(recs, kinds, CAV[f"c{c}_s{k}_in"])
    assert close_rows(out, CAV[f"c{c}_s{k}_out"], 1e-13)


def test_cavity_record_without_positive_final_energy():
    # the branch where the energy after the slice is not positive: only the T566 term, x5 from R.x + B
    rng = np.random.default_rng(3)
    rec = np.zeros(CV.MAP2_DOUBLES)
    rec[:36] = (np.eye(6) + 1e-3 * rng.standard_normal((6, 6))).reshape(-1)
    rec[36:42] = 1e-6 * rng.standard_normal(6)
    rec[CV.CAV_T566] = 0.7
    X = 1e-3 * rng.standard_normal((6, 257))
    out = slices_apply(rec[None, :], [CV.SLICE_CAVITY], X)
    ref = CV.apply_records_numpy(rec[None, :], [CV.SLICE_CAVITY], X)
    assert close_rows(out, ref, 1e-14)


def _line_job(precision="fp64", graph=True):
    pa = ParticleArray(LINE["rp_start"].shape[1])
    pa.rparticles[:] = LINE["rp_start"]
    pa.q_array = LINE["q"].copy()
    pa.E = float(LINE["E_start"])
    procs = [(SpaceCharge(step=st, nmesh_xyz=[63, 63, 63], precision=precision), a, b) for a, b, st in line_procs()]
    job = T.DeviceTrack(line_elements(), None, 0.02, pa, graph=graph, order=2, processes=procs)
    return job, pa


def test_line_fp64_matches_reference_track():
    job, pa = _line_job("fp64", graph=False)
    assert job.nsteps == 194 and sum(len(k) for k, _ in job.steps) == 193
    assert len(job.engines) == 1          # both processes share one plan (same mesh and form)
    job.run()
    job.result(pa)
    assert pa.E == LINE["E_end"] and pa.s == LINE["s_end"]
    err = np.abs(pa.rparticles - LINE["rp_end"]).max(axis=1)
    assert (err <= TOL_ABS).all(), err


def test_line_graph_replay_equals_eager():
    job, pa = _line_job("fp64", graph=True)
    job.run()
    out = job.result().rparticles
    assert 0 < len(job._graphs) < job.nsteps
    job2, _ = _line_job("fp64", graph=False)
    job2.run()
    assert np.array_equal(out, job2.result().rparticles)


def test_line_through_navigator_like_object():
    seq = line_elements()
    procs = []
    for a, b, st in line_procs():
        sc = SpaceCharge(step=st, nmesh_xyz=[63, 63, 63])
        sc.indx0, sc.indx1 = a, b
        procs.append(sc)
    navi = types.SimpleNamespace(unit_step=0.02, process_table=types.SimpleNamespace(proc_list=procs))
    pa = ParticleArray(LINE["rp_start"].shape[1])
    pa.rparticles[:] = LINE["rp_start"]
    pa.q_array = LINE["q"].copy()
    pa.E = float(LINE["E_start"])
    tws, p = T.track(seq, pa, navi, order=2)
    assert p is pa and len(tws) == 195
    from test_cavity_host import _twiss_row, twiss_close
    keys = [str(k) for k in LINE["twiss_keys"]]
    for i, t in enumerate(tws):
        assert not twiss_close(_twiss_row(t, keys), LINE["twiss"][i], keys, rtol=1e-9, eig_rtol=1e-6,
                               derived_rtol=1e-8), i
    assert (np.abs(pa.rparticles - LINE["rp_end"]).max(axis=1) <= TOL_ABS).all()


def test_line_fp32_space_charge_part():
    job64, _ = _line_job("fp64")
    out64 = job64.run().result().rparticles
    job32, _ = _line_job("fp32")
    out32 = job32.run().result().rparticles
    # the transport alone, from the same records on the host
    lin = LINE["rp_start"].copy()
    seq = line_elements()
    steps = T.navigator_steps([e.l for e in seq], line_procs(), 0.02)
    for st in T.step_slices(seq, float(LINE["E_start"]), steps, order=2)[0]:
        lin = CV.apply_records_numpy(st.table, st.kinds, lin)
    for r in (0, 1, 2, 3, 5):
        sc64, sc32 = out64[r] - lin[r], out32[r] - lin[r]
        err = np.sqrt(np.mean((sc32 - sc64) ** 2)) / np.sqrt(np.mean(sc64 ** 2))
        assert err < 1e-4, (r, err)


def _moments_device(rp_host, bounds=None):
    dev = torch.device("cuda", 0)
    n = rp_host.shape[1]
    buf = torch.empty((6, n + 3), dtype=torch.float64, device=dev)   # a row stride other than n
    rp = buf[:, :n]
    rp.copy_(torch.from_numpy(rp_host))
    out = torch.zeros((2, 21), dtype=torch.float64, device=dev)
    scratch = torch.zeros(int(N.lib().sc_moments_scratch_bytes()), dtype=torch.uint8, device=dev)
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    lo, hi = bounds if bounds is not None else (0.0, 0.0)
    for _ in range(2):      # the ticket is reset for the next call
        N.check(N.lib().sc_moments(C.c_void_p(rp.data_ptr()), rp.stride(0), n, None, 2,
                                   1 if bounds is not None else 0, lo, hi, C.c_void_p(out.data_ptr()),
                                   C.c_void_p(scratch.data_ptr()), s))
    torch.cuda.synchronize()
    return out[0].cpu().numpy(), out[1].cpu().numpy()


@pytest.mark.parametrize("n", [5, 1000, 1_000_003])
@pytest.mark.parametrize("bounds", [None, (-0.5, 0.5), (-2.0, 1.0)])
def test_moments_match_host(n, bounds):
    from ocelot_gb300.envelope import moments_numpy
    rng = np.random.default_rng(n)
    rp = rng.standard_normal((6, n)) * np.array([1e-3, 1e-4, 2e-3, 3e-4, 1e-3, 1e-2])[:, None]
    rp += np.array([1e-5, -2e-6, 0, 1e-6, 3e-4, -1e-3])[:, None]
    dev, unused = _moments_device(rp, bounds)
    ref = moments_numpy(rp, bounds)
    assert dev[0] == ref[0]
    assert not unused.any()
    if ref[0] == 0:
        return                  # no particle within the bounds: the means are 0/0 in both
    scale = np.sqrt(np.abs(ref[[9, 12, 9, 12, 15, 20]])) + 1e-300
    assert (np.abs(dev[3:9] - ref[3:9]) <= 1e-12 * np.abs(rp).max(axis=1)[[0, 2, 1, 3, 4, 5]] + 1e-14 * scale).all()
    # second moments within 1e-12 of the product of the two rms sizes (for a variance: of itself); the
    # correlations of an uncorrelated beam are near zero, so a purely relative bound would test rounding
    var = {0: ref[9], 1: ref[12], 2: ref[11], 3: ref[14], 4: ref[15], 5: ref[20]}
    pairs = [(0, 0), (0, 2), (2, 2), (1, 1), (1, 3), (3, 3), (4, 4), (0, 1), (2, 3), (0, 3), (1, 2), (5, 5)]
    scale2 = np.array([np.sqrt(abs(var[a] * var[b])) for a, b in pairs])
    if ref[0] < 3:
        # get_envelope takes no moments of fewer than 3 particles; the spread of the whole beam is the scale
        rms = rp.std(axis=1)[[0, 2, 1, 3, 4, 5]]
        scale2 = np.array([rms[a] * rms[b] for a, b in pairs])
    assert (np.abs(dev[9:21] - ref[9:21]) <= 1e-12 * scale2 + 1e-300).all()
    if bounds is not None:
        assert abs(dev[1] - ref[1]) <= 1e-14 * abs(ref[2]) and abs(dev[2] - ref[2]) <= 1e-13 * ref[2]


@pytest.mark.parametrize("bounds", [None, [-0.5, 0.5]])
def test_line_twiss_matches_reference(bounds):
    keys = [str(k) for k in LINE["twiss_keys"]]
    pa = ParticleArray(LINE["rp_start"].shape[1])
    pa.rparticles[:] = LINE["rp_start"]
    pa.q_array = LINE["q"].copy()
    pa.E = float(LINE["E_start"])
    procs = [(SpaceCharge(step=st, nmesh_xyz=[63, 63, 63]), a, b) for a, b, st in line_procs()]
    job = T.DeviceTrack(line_elements(), None, 0.02, pa, order=2, processes=procs, twiss=True, bounds=bounds).run()
    tws = job.twiss_list()
    table = LINE["twiss"] if bounds is None else LINE["twiss_bounds"]
    assert len(tws) == table.shape[0] == 195
    from test_cavity_host import _twiss_row, twiss_close
    for i, t in enumerate(tws):
        # particles within 1e-13 of the reference's give moments within ~1e-10; the emittances amplify that by
        # 1 + alpha^2 (up to ~70 here), the eigen-emittances by up to ~1e3: the reference test's own 1e-6 for those
        bad = twiss_close(_twiss_row(t, keys), table[i], keys, rtol=1e-9, eig_rtol=1e-6, derived_rtol=1e-8)
        assert not bad, (i, bad)
    assert [t.s for t in tws] == list(LINE["twiss"][:, keys.index("s")])
    assert [t.E for t in tws] == list(LINE["twiss"][:, keys.index("E")])


def test_line_twiss_graph_equals_eager():
    runs = []
    for graph in (False, True):
        pa = ParticleArray(LINE["rp_start"].shape[1])
        pa.rparticles[:] = LINE["rp_start"]
        pa.q_array = LINE["q"].copy()
        pa.E = float(LINE["E_start"])
        procs = [(SpaceCharge(step=st, nmesh_xyz=[63, 63, 63]), a, b) for a, b, st in line_procs()]
        job = T.DeviceTrack(line_elements(), None, 0.02, pa, graph=graph, order=2, processes=procs, twiss=True).run()
        job.synchronize()
        runs.append(job.moments.cpu().numpy())
    assert np.array_equal(runs[0], runs[1])


@pytest.mark.parametrize("graph", [False, True])
def test_mixed_line_first_order_matches_reference_track(graph):
    """First-order transport through a cavity and quadrupoles with two
    processes of different step counts (the reference's TransferMap lattice)."""
    from test_cavity_host import _twiss_row, twiss_close
    pa = ParticleArray(MIXED["rp_start"].shape[1])
    pa.rparticles[:] = MIXED["rp_start"]
    pa.q_array = MIXED["q"].copy()
    pa.E = float(MIXED["E_start"])
    mesh = [int(v) for v in MIXED["nmesh"]]
    procs = [(SpaceCharge(step=st, nmesh_xyz=mesh), a, b) for a, b, st in mixed_procs()]
    job = T.DeviceTrack(line_elements(MIXED), None, float(MIXED["unit_step"]), pa, graph=graph, order=1,
                        processes=procs, twiss=True).run()
    tws = job.twiss_list()
    job.result(pa)
    assert not job.composed and sum(len(k) for k, _ in job.steps) == len(MIXED["kick_step"])
    assert pa.E == MIXED["E_end"] and pa.s == MIXED["s_end"]
    err = np.abs(pa.rparticles - MIXED["rp_end"]).max(axis=1)
    assert (err <= TOL_ABS).all(), err
    keys = [str(k) for k in MIXED["twiss_keys"]]
    for i, t in enumerate(tws):
        assert not twiss_close(_twiss_row(t, keys), MIXED["twiss"][i], keys, rtol=1e-9, eig_rtol=1e-6,
                               derived_rtol=1e-8), i


def test_pattern_map_forms_equal_the_general_form():
    """The straight-line drift/quadrupole forms give the general form's
    result bit for bit (same FMAs in the same order over the pattern)."""
    from ocelot_gb300.second_order import element_map2, pack_map
    E = 0.05
    elems = [(T.Drift(l=0.3), 0.3), (T.Quadrupole(l=0.2, k1=1.7), 0.2), (T.Quadrupole(l=0.2, k1=-1.7), 0.05),
             (T.Quadrupole(l=0.2, k1=1.7, tilt=0.1), 0.2), (T.Marker(), 0.0)]
    recs = [pack_map(*element_map2(e, L, E)) for e, L in elems]
    R, B = T.element_map(T.Quadrupole(l=0.2, k1=2.5), 0.2, E)
    recs.append(pack_map(R, np.zeros((6, 6, 6)), B))
    recs = np.array(recs)
    kinds = [CV.map_kind(r) for r in recs]
    assert kinds == [CV.SLICE_MAP_DRIFT, CV.SLICE_MAP_PLANAR, CV.SLICE_MAP_PLANAR, CV.SLICE_MAP,
                     CV.SLICE_MAP_LINEAR, CV.SLICE_MAP_LINEAR]
    rng = np.random.default_rng(7)
    X = rng.standard_normal((6, 4099)) * np.array([1e-3, 1e-4, 1e-3, 1e-4, 1e-3, 1e-2])[:, None]
    fast = slices_apply(recs, kinds, X)
    general = slices_apply(recs, [CV.SLICE_MAP] * len(kinds), X)
    assert np.array_equal(fast, general)
    assert close_rows(fast, CV.apply_records_numpy(recs, kinds, X), 1e-13)


@pytest.mark.parametrize("bounds", [None, [-0.5, 0.5]])
def test_get_envelope_matches_reference(bounds):
    """get_envelope on the device, for a host and a device beam, against the
    reference's get_envelope of the same beam (the last row of the twiss list
    its track() returned)."""
    from ocelot_gb300.beam import DeviceParticleArray
    from ocelot_gb300.envelope import get_envelope
    from test_cavity_host import _twiss_row, twiss_close
    keys = [str(k) for k in LINE["twiss_keys"]]
    table = LINE["twiss"] if bounds is None else LINE["twiss_bounds"]
    pa = ParticleArray(LINE["rp_end"].shape[1])
    pa.rparticles[:] = LINE["rp_end"]
    pa.q_array = LINE["q"].copy()
    pa.E = float(LINE["E_end"])
    ref = table[-1].copy()
    ref[keys.index("s")] = 0.0        # get_envelope leaves s at 0; track() adds the position
    for beam in (pa, DeviceParticleArray.from_host(pa, torch.device("cuda", 0))):
        t = get_envelope(beam, bounds=bounds)
        assert not twiss_close(_twiss_row(t, keys), ref, keys, rtol=1e-12, eig_rtol=1e-8, derived_rtol=1e-11)
    with pytest.raises(NotImplementedError):
        get_envelope(pa, auto_disp=True)
