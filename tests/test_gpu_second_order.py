"""Second-order transport on the GPU (SecondTM of drift/quadrupole slices).

* sc_tmap2_apply through the C ABI on a seeded beam: several maps (drift,
  quadrupole, tilted offset quadrupole) applied in one pass equal the host's
  R.X + T:XX + B applied map after map, within 1e-13 relative per row (the
  device accumulates the combined coefficients as an FMA chain).
* DeviceTrack with order=2 (FP64 form) reproduces the reference's track()
  through FODO cells with SecondTM and SpaceCharge (ref_fodo_track2.npz)
  within 1e-10 relative per row -- the tolerance of the first-order run.
* graph replay equals eager launches bit for bit.
"""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN, has_gpu
from oracle import sc_oracle

pytestmark = pytest.mark.gpu

if not has_gpu():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch  # noqa: E402

from ocelot_gb300 import ParticleArray, SpaceCharge  # noqa: E402
from ocelot_gb300 import _native as N  # noqa: E402
from ocelot_gb300 import track as T  # noqa: E402
from ocelot_gb300.second_order import MAP2_DOUBLES, element_map2, pack_map  # noqa: E402

DEV = torch.device("cuda", 0)
FODO2 = dict(np.load(os.path.join(GOLDEN, "ref_fodo_track2.npz")))


def rel_rows(a, b):
    return max(np.linalg.norm(a[r] - b[r]) / np.linalg.norm(b[r]) for r in range(a.shape[0]))


def test_tmap2_apply_matches_host():
    q = T.Quadrupole(l=0.2, k1=-1.2, tilt=0.3)
    q.dx, q.dy = 1e-3, -2e-3
    slices = [(T.Drift(l=0.7), 0.7), (T.Quadrupole(l=0.2, k1=1.2), 0.2), (q, 0.15)]
    rp, _ = sc_oracle.gaussian_beam(100_003, 31, sigma_x=1e-3, sigma_px=1e-4, sigma_y=1e-3, sigma_py=1e-4,
                                    sigma_tau=1e-4, sigma_p=1e-3)
    host = rp.copy()
    maps = []
    for e, dl in slices:
        R, Tt, B = element_map2(e, dl, 0.130)
        host = R @ host + np.einsum("ijk,j...,k...->i...", Tt, host, host) + B[:, None]
        maps.append(pack_map(R, Tt, B))
    maps = np.array(maps)
    d_maps = torch.from_numpy(maps).to(DEV)
    d_rp = torch.from_numpy(rp).to(DEV)
    lib = N.lib()
    s = C.c_void_p(torch.cuda.current_stream(DEV).cuda_stream)
    N.check(lib.sc_tmap2_apply(C.c_void_p(d_maps.data_ptr()), len(slices), C.c_void_p(d_rp.data_ptr()),
                               d_rp.stride(0), d_rp.shape[1], s))
    out = d_rp.cpu().numpy()
    assert maps.shape[1] == MAP2_DOUBLES
    assert rel_rows(out, host) < 1e-13


def _fodo(cells):
    seq = []
    for _ in range(cells):
        seq += [T.Quadrupole(l=0.2, k1=1.2), T.Drift(l=1.0), T.Quadrupole(l=0.2, k1=-1.2), T.Drift(l=1.0)]
    return seq + [T.Marker()]


def _run(graph):
    rp, q = FODO2["rp_in"], FODO2["q"]
    pa = ParticleArray(rp.shape[1])
    pa.rparticles[:] = rp
    pa.q_array = q.copy()
    pa.E = float(FODO2["E"])
    sc = SpaceCharge(step=1, nmesh_xyz=[int(v) for v in FODO2["nmesh"]], precision="fp64")
    job = T.DeviceTrack(_fodo(int(FODO2["cells"])), sc, 0.25, pa, graph=graph, order=2)
    job.run()
    return job.result().rparticles


def test_fodo_second_order_track_matches_reference():
    assert rel_rows(_run(graph=False), FODO2["rp_out"]) < 1e-10


def test_second_order_graph_replay_equals_eager():
    assert np.array_equal(_run(graph=False), _run(graph=True))
