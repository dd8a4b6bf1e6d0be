"""Batched kicks (sc_kick_batched): many beams of uneven size and mesh in one
launch per stage.  Each beam keeps the grids and reductions of a single kick,
so the tests require bit-identical particles against kicking each beam alone
(FP32 form with the exact fixed-point deposit), in eager and graph-replayed
batches, across repeated kicks (the cached Green's tables), with odd sizes,
unaligned rows, zero-length kicks and a degenerate beam in the mix."""
import numpy as np
import pytest

from conftest import has_gpu
from oracle import sc_oracle

pytestmark = pytest.mark.gpu

if not has_gpu():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch  # noqa: E402

from ocelot_gb300 import SpaceCharge  # noqa: E402
from ocelot_gb300.batch import BeamBatch  # noqa: E402

DEV = torch.device("cuda", 0)

SPECS = [  # n, mesh, E [GeV], charge [C], sigma_x, sigma_tau, zstep
    (2, [8, 8, 8], 0.05, 1e-12, 1e-4, 1e-4, 0.1),
    (3001, [15, 15, 15], 0.13, 250e-12, 50e-6, 100e-6, 0.1),
    (20_000, [32, 32, 32], 0.0065, 500e-12, 200e-6, 300e-6, 0.05),
    (100_000, [16, 24, 32], 0.3, 100e-12, 30e-6, 400e-6, 0.2),
    (257, [32, 32, 128], 0.02, 20e-12, 300e-6, 30e-6, 0.1),
    (50_001, [48, 48, 48], 0.5, 400e-12, 80e-6, 80e-6, 0.15),
]


def _beam(i, spec):
    n, _, _, charge, sx, st, _ = spec
    rp, q = sc_oracle.gaussian_beam(n, 100 + i, sigma_x=sx, sigma_y=sx, sigma_tau=st, charge=charge)
    return rp, q


def _dev(rp, q, odd_stride=False):
    n = rp.shape[1]
    ld = (n if n % 2 else n + 1) if odd_stride else n + (n & 1)
    buf = torch.zeros((6, ld), dtype=torch.float64, device=DEV)
    buf[:, :n] = torch.from_numpy(rp).to(DEV)
    return buf[:, :n], torch.from_numpy(q).to(DEV)


def _alone(rp, q, spec, kicks=1, odd_stride=False, fields="spectral"):
    d_rp, d_q = _dev(rp, q, odd_stride)
    sc = SpaceCharge(nmesh_xyz=spec[1], precision="fp32", fields=fields)
    for _ in range(kicks):
        sc.apply_device(d_rp, d_q, spec[2], spec[6])
    sc.check()
    return d_rp.cpu().numpy()


def _batch(beams, kicks=1, graph=False, odd=(), fields="spectral"):
    b = BeamBatch(DEV, fields=fields)
    tensors = []
    for i, (rp, q, spec) in enumerate(beams):
        d_rp, d_q = _dev(rp, q, i in odd)
        tensors.append((d_rp, d_q))
        b.add(d_rp, d_q, spec[2], spec[1], spec[6])
    b.commit()
    if graph:
        g = b.graph()
        for _ in range(kicks):
            g.replay()
    else:
        for _ in range(kicks):
            b.kick()
    torch.cuda.synchronize()
    return b, [t[0].cpu().numpy() for t in tensors]


@pytest.mark.parametrize("kicks,graph,fields", [(1, False, "spectral"), (3, False, "spectral"), (3, True, "spectral"),
                                                (2, False, "difference"), (2, True, "difference")])
def test_batched_equals_alone(kicks, graph, fields):
    beams = [(*_beam(i, s), s) for i, s in enumerate(SPECS)]
    b, outs = _batch(beams, kicks, graph, fields=fields)
    b.check()
    assert b.launches == 15
    for (rp, q, spec), out in zip(beams, outs):
        ref = _alone(rp, q, spec, kicks, fields=fields)
        assert np.array_equal(out, ref), spec
        assert not np.array_equal(out, rp)


def test_batched_unaligned_rows_match_alone():
    """Odd row strides take the one-particle-per-thread loop; inlined into the
    batched kernels its FP32 products may be contracted into FMAs differently
    than in the plain kernels, so the result is compared to 1e-12 of each
    row's scale (the FP32 kick itself is accurate to 1e-5)."""
    beams = [(*_beam(i, s), s) for i, s in enumerate(SPECS[1:4])]
    _, outs = _batch(beams, 2, odd=(0, 2))
    for i, ((rp, q, spec), out) in enumerate(zip(beams, outs)):
        ref = _alone(rp, q, spec, 2, odd_stride=i in (0, 2))
        for r in range(6):
            assert np.abs(out[r] - ref[r]).max() <= 1e-12 * np.abs(ref[r]).max(), (i, r)


def test_batch_result_does_not_depend_on_the_mix():
    """The same beam kicked in batches of different company is bit-identical
    (each beam's grids and reductions are its own), aligned or not."""
    beams = [(*_beam(i, s), s) for i, s in enumerate(SPECS)]
    _, mixed = _batch(beams, 2, odd=(1, 3))
    for j in (1, 3, 5):
        _, solo = _batch([beams[j]], 2, odd=(0,) if j in (1, 3) else ())
        assert np.array_equal(solo[0], mixed[j]), j


def test_zero_step_beam_is_left_alone_and_degenerate_beam_latches():
    good = (*_beam(1, SPECS[1]), SPECS[1])
    still = (*_beam(2, SPECS[2]), SPECS[2][:6] + (0.0,))
    rp_deg = np.zeros((6, 64))
    rp_deg[5] = 1e-4
    deg = (rp_deg, np.full(64, 1e-12), SPECS[1])
    b, outs = _batch([good, still, deg])
    assert np.array_equal(outs[0], _alone(good[0], good[1], good[2]))
    assert np.array_equal(outs[1], still[0])
    b.beams[0][0].check_status()
    with pytest.raises(ValueError, match=r"\[sc error 4\]"):
        b.beams[2][0].check_status()


def test_batch_rejects_fp64_plans_and_shared_buffers():
    from ocelot_gb300.sc import Engine
    rp, q = _beam(1, SPECS[1])
    d_rp, d_q = _dev(rp, q)
    b = BeamBatch(DEV)
    b.add(d_rp, d_q, 0.13, [15, 15, 15], 0.1, engine=Engine((15, 15, 15), "fp64", DEV))
    with pytest.raises(ValueError, match=r"\[sc error 6\]"):
        b.commit()
    b2 = BeamBatch(DEV)
    b2.add(d_rp, d_q, 0.13, [15, 15, 15], 0.1)
    b2.add(d_rp, d_q, 0.13, [15, 15, 15], 0.1)
    with pytest.raises(ValueError, match=r"\[sc error 1\]"):
        b2.commit()


def test_batch_of_many_small_beams():
    """96 beams of a few thousand particles on mixed meshes: the launch count
    stays 15 and every beam equals its solo kick."""
    meshes = [[32, 32, 32], [16, 16, 16], [32, 32, 64], [24, 24, 24]]
    rng = np.random.default_rng(9)
    beams = []
    for i in range(96):
        n = int(rng.integers(500, 5000))
        spec = (n, meshes[i % 4], float(rng.uniform(0.005, 0.5)), float(rng.uniform(20e-12, 500e-12)),
                float(rng.uniform(20e-6, 500e-6)), float(rng.uniform(20e-6, 500e-6)), 0.1)
        beams.append((*_beam(1000 + i, spec), spec))
    b, outs = _batch(beams)
    assert b.launches == 15
    for (rp, q, spec), out in list(zip(beams, outs))[::7]:
        assert np.array_equal(out, _alone(rp, q, spec))


def test_zero_step_beam_with_a_map_is_transported():
    """A step whose kick has zero length still applies its transport map (the
    reference returns early from apply only, sc.py:210-212): the beam stays in
    the table for sc_tmap_batched alone, beside a beam that is also kicked."""
    R = np.eye(6)
    R[0, 1] = R[2, 3] = 0.7      # a drift of 0.7 m (first order)
    B = np.zeros(6)
    good = (*_beam(1, SPECS[1]), SPECS[1])
    still = (*_beam(2, SPECS[2]), SPECS[2])
    b = BeamBatch(DEV)
    d0, q0 = _dev(good[0], good[1])
    d1, q1 = _dev(still[0], still[1])
    b.add(d0, q0, good[2][2], good[2][1], good[2][6], tmap=(R, B))
    b.add(d1, q1, still[2][2], still[2][1], 0.0, tmap=(R, B))
    b.commit()
    b.transport()
    b.kick()
    torch.cuda.synchronize()
    b.beams[0][0].check_status()
    # the same maps and kick, one beam at a time through the plain entry points
    from ocelot_gb300.transfer import tmap_apply
    e1, _ = _dev(still[0], still[1])
    tmap_apply(R, B, e1)
    assert np.array_equal(d1.cpu().numpy(), e1.cpu().numpy())
    assert not np.array_equal(d1.cpu().numpy(), still[0])
    e0, eq0 = _dev(good[0], good[1])
    tmap_apply(R, B, e0)
    sc = SpaceCharge(nmesh_xyz=good[2][1], precision="fp32")
    sc.apply_device(e0, eq0, good[2][2], good[2][6])
    sc.check()
    assert np.array_equal(d0.cpu().numpy(), e0.cpu().numpy())


def test_workspace_allocated_anew_after_commit():
    """A beam's engine whose workspace grows after the table was uploaded (a
    solo kick of more particles) no longer matches the table: the C entry
    point refuses to kick with the old workspace, and BeamBatch uploads the
    table again before its next kick, whose result equals the solo kick."""
    import ctypes as C
    from ocelot_gb300 import _native as N
    from ocelot_gb300.sc import Engine
    spec = SPECS[2]
    rp, q = _beam(2, spec)
    d_rp, d_q = _dev(rp, q)
    eng = Engine(tuple(spec[1]), "fp32", DEV)
    b = BeamBatch(DEV)
    b.add(d_rp, d_q, spec[2], spec[1], spec[6], engine=eng)
    b.commit()
    old = eng.ws.data_ptr()
    eng.ensure(4 * eng.cap)
    assert eng.ws.data_ptr() != old
    stream = C.c_void_p(torch.cuda.current_stream(DEV).cuda_stream)
    assert b.lib.sc_kick_batched(b.handle, stream) == N.SC_ERR_WORKSPACE
    assert b.launches == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_rp.cpu().numpy(), rp)          # nothing ran
    b.kick()
    torch.cuda.synchronize()
    b.check()
    assert np.array_equal(d_rp.cpu().numpy(), _alone(rp, q, spec))


def test_graph_fixes_the_table_shape():
    """After a kick is recorded as a graph, a table of another shape (a beam's
    kick length set to zero removes it from the kick stages) is refused;
    a table of the same shape with other kick lengths is accepted, and a
    replay kicks with the new lengths."""
    beams = [(*_beam(i, s), s) for i, s in enumerate(SPECS[:3])]
    b = BeamBatch(DEV)
    tensors = []
    for rp, q, spec in beams:
        d_rp, d_q = _dev(rp, q)
        tensors.append(d_rp)
        b.add(d_rp, d_q, spec[2], spec[1], spec[6])
    g = b.graph()
    b.set_step(1, 0.0)
    with pytest.raises(ValueError, match=r"\[sc error 1\]"):
        b.commit()
    half = [s[:6] + (s[6] / 2,) for _, _, s in beams]
    for i, s in enumerate(half):
        b.set_step(i, s[6])
    g.replay()
    torch.cuda.synchronize()
    b.check()
    for (rp, q, _), s, t in zip(beams, half, tensors):
        assert np.array_equal(t.cpu().numpy(), _alone(rp, q, s))
