"""Device-resident tracking on the GPU: the reference's FODO run (first-order
maps between kicks every 0.25 m) reproduced with the particles kept on the
device, eager and graph-replayed; the indexed map table; jobs interleaved on
separate streams give the results they give alone.

Tolerances: FP64 form 1e-10 relative per row against the reference's tracked
particles (the composed step maps differ from sequential slices by rounding
only); graph replay and interleaving are bit-identical to eager, alone runs
(both forms are deterministic).  FP32 form: the space-charge part of the
momentum change (tracked minus transport-only) within 1e-4 relative RMS of
the FP64 form's over 20 kicks.
"""
import os
import types

import numpy as np
import pytest

from conftest import GOLDEN, has_gpu
from oracle import sc_oracle

pytestmark = pytest.mark.gpu

if not has_gpu():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import ctypes as C  # noqa: E402

import torch  # noqa: E402

from ocelot_gb300 import ParticleArray, SpaceCharge  # noqa: E402
from ocelot_gb300 import _native as N  # noqa: E402
from ocelot_gb300 import track as T  # noqa: E402

DEV = torch.device("cuda", 0)
FODO = dict(np.load(os.path.join(GOLDEN, "ref_fodo_track.npz")))


def _fodo(cells):
    seq = []
    for _ in range(cells):
        seq += [T.Quadrupole(l=0.2, k1=1.2), T.Drift(l=1.0), T.Quadrupole(l=0.2, k1=-1.2), T.Drift(l=1.0)]
    return seq + [T.Marker()]


def _pa(rp, q, E):
    pa = ParticleArray(rp.shape[1])
    pa.rparticles[:] = rp
    pa.q_array = q.copy()
    pa.E = E
    return pa


def rel_rows(a, b):
    return max(np.linalg.norm(a[r] - b[r]) / np.linalg.norm(b[r]) for r in range(a.shape[0]))


def _run(precision="fp64", graph=True, rp=None, q=None, E=None, mesh=None, cells=None):
    rp = FODO["rp_in"] if rp is None else rp
    q = FODO["q"] if q is None else q
    E = float(FODO["E"]) if E is None else E
    mesh = [int(v) for v in FODO["nmesh"]] if mesh is None else mesh
    sc = SpaceCharge(step=1, nmesh_xyz=mesh, precision=precision)
    job = T.DeviceTrack(_fodo(int(FODO["cells"]) if cells is None else cells), sc, 0.25, _pa(rp, q, E), graph=graph)
    job.run()
    return job, job.result().rparticles


def test_fodo_track_fp64_matches_reference():
    job, out = _run("fp64", graph=False)
    assert job.nsteps == len(FODO["kicks"])
    assert rel_rows(out, FODO["rp_out"]) < 1e-10


def test_fodo_track_graph_replay_equals_eager():
    _, eager = _run("fp64", graph=False)
    job, replay = _run("fp64", graph=True)
    # the 0.25 m steps replay one graph; the truncated last step runs once and is launched directly
    assert len(job._graphs) == 1
    assert np.array_equal(eager, replay)
    _, e32 = _run("fp32", graph=False)
    _, g32 = _run("fp32", graph=True)
    assert np.array_equal(e32, g32)


def test_fodo_track_fp32_space_charge_part():
    _, out64 = _run("fp64")
    _, out32 = _run("fp32")
    lin = FODO["rp_in"].copy()
    for R, B, _, _ in T.step_maps(_fodo(int(FODO["cells"])), float(FODO["E"]), 0.25):
        lin = R @ lin + B[:, None]
    for r in (1, 3, 5):
        sc64, sc32 = out64[r] - lin[r], out32[r] - lin[r]
        err = np.sqrt(np.mean((sc32 - sc64) ** 2)) / np.sqrt(np.mean(sc64 ** 2))
        assert err < 1e-4, (r, err)


def test_track_function_with_navigator_like_object():
    sc = SpaceCharge(step=1, nmesh_xyz=[int(v) for v in FODO["nmesh"]])
    navi = types.SimpleNamespace(unit_step=0.25, process_table=types.SimpleNamespace(proc_list=[sc]))
    pa = _pa(FODO["rp_in"], FODO["q"], float(FODO["E"]))
    tws, p = T.track(_fodo(int(FODO["cells"])), pa, navi)
    assert p is pa and len(tws) == len(FODO["kicks"]) + 1
    assert rel_rows(pa.rparticles, FODO["rp_out"]) < 1e-10


def test_tmap_indexed_applies_table_in_order_and_advances():
    rng = np.random.default_rng(5)
    n = 10_001
    X = rng.standard_normal((6, n))
    maps = [(np.eye(6) + 0.1 * rng.standard_normal((6, 6)), rng.standard_normal(6)) for _ in range(3)]
    table = torch.tensor(np.stack([np.r_[R.reshape(-1), B] for R, B in maps]), device=DEV)
    counter = torch.zeros(1, dtype=torch.int32, device=DEV)
    d = torch.tensor(X, device=DEV)
    lib = N.lib()
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for _ in range(4):   # the fourth index is past the table: no transport, counter still moves
        N.check(lib.sc_tmap_apply_indexed(C.c_void_p(table.data_ptr()), C.c_void_p(counter.data_ptr()), 3,
                                          C.c_void_p(d.data_ptr()), n, n, s))
    for R, B in maps:
        X = R @ X + B[:, None]
    assert int(counter.item()) == 4
    assert np.allclose(d.cpu().numpy(), X, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_interleaved_jobs_equal_alone(precision):
    """Three jobs of different size and mesh stepped round-robin on their own
    streams give bit-identical particles to each job run alone."""
    specs = [(3000, 7, [15, 15, 15]), (20_000, 8, [32, 32, 32]), (7000, 9, [16, 24, 32])]
    alone, jobs = [], []
    for n, seed, mesh in specs:
        rp, q = sc_oracle.gaussian_beam(n, seed, sigma_x=200e-6, sigma_y=200e-6, charge=300e-12)
        alone.append(_run(precision, rp=rp, q=q, E=0.05, mesh=mesh, cells=2)[1])
        sc = SpaceCharge(step=1, nmesh_xyz=mesh, precision=precision)
        jobs.append(T.DeviceTrack(_fodo(2), sc, 0.25, _pa(rp, q, 0.05)))
    while not all(j.finished for j in jobs):
        for j in jobs:
            j.step(1)
    for j, ref in zip(jobs, alone):
        assert np.array_equal(j.result().rparticles, ref)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_random_mesh_track_equals_plugin_step_by_step(precision):
    """random_mesh: the device loop takes the two draws per kick from numpy's
    global generator in kick order, as SpaceCharge.apply does inside the
    reference's track() -- so a seeded device track equals the plugin
    applied after each step's map, bit for bit, and leaves the generator in
    the same state."""
    mesh = [int(v) for v in FODO["nmesh"]]
    E = float(FODO["E"])
    seq = _fodo(int(FODO["cells"]))
    np.random.seed(10)
    sc = SpaceCharge(step=1, nmesh_xyz=mesh, precision=precision, random_mesh=True)
    job = T.DeviceTrack(seq, sc, 0.25, _pa(FODO["rp_in"], FODO["q"], E), graph=True)
    after_job = np.random.random()
    out = job.run().result().rparticles
    assert len(job._graphs) == 0           # every kick has its own mesh: no step repeats

    np.random.seed(10)
    sc2 = SpaceCharge(step=1, nmesh_xyz=mesh, precision=precision, random_mesh=True)
    dev = torch.device("cuda", 0)
    # the job's row layout (the FP32 form is bit-reproducible for a given layout)
    rp = torch.empty_like(job.beam.rparticles)
    assert rp.stride() == job.beam.rparticles.stride()
    rp.copy_(torch.from_numpy(FODO["rp_in"]))
    q = torch.from_numpy(FODO["q"]).to(dev)
    lib = N.lib()
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    for R, B, zstep, _ in T.step_maps(seq, E, 0.25):
        Rc = np.ascontiguousarray(R, dtype=np.float64)
        Bc = np.ascontiguousarray(B, dtype=np.float64)
        N.check(lib.sc_tmap_apply(Rc.ctypes.data_as(C.POINTER(C.c_double)), Bc.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.c_void_p(rp.data_ptr()), rp.stride(0), rp.shape[1], s))
        sc2.apply_device(rp, q, E, zstep)
    sc2.check()
    assert np.random.random() == after_job
    assert np.array_equal(out, rp.cpu().numpy())
