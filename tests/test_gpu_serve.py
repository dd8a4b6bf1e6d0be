"""The tracking server: continuous batching of FODO tracking jobs.

A job's result must not depend on the company it ran in: the tests compare
each job served among others (admitted at different ticks, so their steps
interleave at different lattice positions) with the same job served alone,
bit for bit, and with DeviceTrack (plain launches) bit for bit.  Against the
reference's own FODO run (FP64) the FP32 form's space-charge part is within
1e-4 relative RMS after 20 kicks, as for DeviceTrack.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, has_gpu

pytestmark = pytest.mark.gpu

if not has_gpu():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch  # noqa: E402

from ocelot_gb300 import ParticleArray, SpaceCharge  # noqa: E402
from ocelot_gb300 import serve as S  # noqa: E402
from ocelot_gb300 import track as T  # noqa: E402

DEV = torch.device("cuda", 0)
FODO = dict(np.load(os.path.join(GOLDEN, "ref_fodo_track.npz")))


def _req(n, seed, mesh, cells=2, **kw):
    return S.Request(S.BeamSpec(n=n, seed=seed, **kw), S.fodo(cells), tuple(mesh), 0.25, 1)


JOBS = [(3000, 1, (15, 15, 15)), (20_000, 2, (32, 32, 32)), (7001, 3, (24, 24, 24)), (12_000, 4, (16, 16, 32))]


def _alone(n, seed, mesh):
    srv = S.Server(DEV, max_active=4)
    jid = srv.submit(_req(n, seed, mesh))
    srv.drain()
    return srv.result(jid)


def test_job_in_the_mix_equals_job_alone():
    srv = S.Server(DEV, max_active=8)
    ids = [srv.submit(_req(*JOBS[0]))]
    for _ in range(3):
        srv.pump()
    ids.append(srv.submit(_req(*JOBS[1])))
    for _ in range(5):
        srv.pump()
    ids += [srv.submit(_req(*JOBS[2])), srv.submit(_req(*JOBS[3]))]
    srv.drain()
    assert srv.ticks > 20          # 20 steps per job, staggered starts
    for jid, spec in zip(ids, JOBS):
        assert np.array_equal(srv.result(jid), _alone(*spec)), spec


def test_server_equals_device_track():
    pa = ParticleArray(FODO["rp_in"].shape[1])
    pa.rparticles[:] = FODO["rp_in"]
    pa.q_array = FODO["q"].copy()
    pa.E = float(FODO["E"])
    mesh = tuple(int(v) for v in FODO["nmesh"])
    srv = S.Server(DEV)
    jid = srv.submit(S.Request(pa, S.fodo(int(FODO["cells"])), mesh, 0.25, 1))
    srv.drain()
    out = srv.result(jid)
    sc = SpaceCharge(step=1, nmesh_xyz=list(mesh), precision="fp32")
    ref = T.DeviceTrack(S.fodo(int(FODO["cells"])), sc, 0.25, pa).run().result().rparticles
    assert np.array_equal(out, ref)
    # and against the reference's FP64 run: the space-charge part
    lin = FODO["rp_in"].copy()
    for R, B, _, _ in T.step_maps(S.fodo(int(FODO["cells"])), float(FODO["E"]), 0.25):
        lin = R @ lin + B[:, None]
    for r in (1, 3, 5):
        sc_ref, sc_out = FODO["rp_out"][r] - lin[r], out[r] - lin[r]
        assert np.sqrt(np.mean((sc_out - sc_ref) ** 2)) / np.sqrt(np.mean(sc_ref ** 2)) < 1e-4


def test_admission_keeps_within_the_hbm_budget():
    srv0 = S.Server(DEV)
    eng = srv0._engine((32, 32, 32))
    one = srv0._footprint(eng, 20_000)
    srv = S.Server(DEV, hbm_budget=int(2.5 * one), max_active=8)
    ids = [srv.submit(_req(20_000, 10 + i, (32, 32, 32))) for i in range(5)]
    most = 0
    while srv.busy():
        srv.pump()
        assert srv.used <= srv.budget
        most = max(most, len(srv.active))
    assert most == 2
    for i, jid in enumerate(ids):
        assert np.array_equal(srv.result(jid), _alone(20_000, 10 + i, (32, 32, 32)))


def test_failing_job_reports_its_error_and_spares_the_others():
    srv = S.Server(DEV)
    bad = ParticleArray(64)
    bad.rparticles[5] = 1e-4            # every particle at one point: no extent
    bad.q_array = np.full(64, 1e-12)
    bad.E = 0.13
    ids = [srv.submit(_req(*JOBS[0])), srv.submit(S.Request(bad, S.fodo(2), (15, 15, 15))),
           srv.submit(_req(*JOBS[1]))]
    srv.drain()
    with pytest.raises(ValueError, match=r"\[sc error 4\]"):
        srv.result(ids[1])
    assert np.array_equal(srv.result(ids[0]), _alone(*JOBS[0]))
    assert np.array_equal(srv.result(ids[2]), _alone(*JOBS[1]))


def test_poisson_run_serves_everything():
    srv = S.Server(DEV, max_active=16)
    reqs = [_req(2000 + 500 * i, 50 + i, (16, 16, 16), cells=1) for i in range(8)]
    lat, wall, kicks, ids = S.poisson_run(srv, reqs, rate_hz=200.0, seed=1)
    assert len(lat) == 8 and (lat > 0).all() and wall > 0
    assert kicks == sum((2000 + 500 * i) * 10 for i in range(8))   # 10 kicks of 0.25 m per 2.4 m cell
    for jid, r in zip(ids, reqs):
        assert srv.result(jid).shape == (6, r.beam.n)


def test_line_without_steps_is_refused():
    # a zero-length section (only a Marker) gives no tracking step: the server
    # refuses it at submit instead of admitting a job that never finishes
    srv = S.Server(DEV)
    with pytest.raises(ValueError, match="no tracking steps"):
        srv.submit(S.Request(S.BeamSpec(n=1000, seed=1), S.fodo(0), (15, 15, 15), 0.25, 1))
    assert not srv.busy()
    jid = srv.submit(_req(*JOBS[0], cells=1))
    srv.drain(timeout_s=60.0)
    assert srv.result(jid).shape == (6, JOBS[0][0])


def test_request_refused_at_submit_leaves_the_server_idle():
    # validate_request runs at submit: a beam whose q_array does not match its
    # particles never reaches the batched kernels
    srv = S.Server(DEV)
    pa = ParticleArray(64)
    pa.rparticles[:] = np.random.default_rng(3).standard_normal((6, 64)) * 1e-4
    pa.q_array = np.full(32, 1e-12)
    pa.E = 0.13
    with pytest.raises(ValueError, match="q_array has"):
        srv.submit(S.Request(pa, S.fodo(1), (15, 15, 15)))
    assert not srv.busy()
