"""The record-field mode: the field each particle was kicked with, stored
by the kick itself (SC_PARAM_RECORD_FIELD, SC_REGION_FIELD) -- the
measurement behind the stated errors of E at the particles.  The FP64 form's
record equals the oracle's el_field at the particles (sc.py:201-204) to
1e-11, and recording changes no particle in either form."""
import numpy as np
import pytest

from conftest import has_gpu
from oracle import sc_oracle

pytestmark = pytest.mark.gpu

if not has_gpu():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch  # noqa: E402

from ocelot_gb300 import SpaceCharge, _native as N  # noqa: E402

DEV = torch.device("cuda", 0)


def _kick(rp, q, precision, record, mesh=(32, 32, 32)):
    n = rp.shape[1]
    d = torch.zeros((6, n + (n & 1)), dtype=torch.float64, device=DEV)[:, :n]
    d.copy_(torch.from_numpy(rp))
    sc = SpaceCharge(nmesh_xyz=list(mesh), precision=precision, device=DEV)
    eng = sc.engine()
    eng.set_param(N.SC_PARAM_RECORD_FIELD, int(record))
    sc.apply_device(d, torch.from_numpy(q).to(DEV), 0.130, 0.1)
    sc.check()
    return d.cpu().numpy(), (eng.region("field", n).double().cpu().numpy() if record else None)


@pytest.mark.parametrize("n", [50_000, 50_001])
def test_recorded_field_equals_the_oracle_and_changes_nothing(n):
    rp, q = sc_oracle.gaussian_beam(n, 8, charge=1e-9)
    rec = {}
    ref = rp.copy()
    sc_oracle.sc_apply(ref, q, 0.130, 0.1, [32, 32, 32], record=rec)
    g0 = float(rec["gamma0"])
    out64, f64 = _kick(rp, q, "fp64", True)
    plain64, _ = _kick(rp, q, "fp64", False)
    assert np.array_equal(out64, plain64)
    E = rec["Exyz"]
    for c, scale in ((0, g0), (1, g0), (2, 1.0)):
        got = f64[c] * scale
        assert np.linalg.norm(got - E[:, c]) <= 1e-11 * np.linalg.norm(E[:, c]), c
    out32, f32 = _kick(rp, q, "fp32", True)
    plain32, _ = _kick(rp, q, "fp32", False)
    assert np.array_equal(out32, plain32)
    for c in range(3):
        assert np.linalg.norm(f32[c] - f64[c]) <= 1e-4 * np.linalg.norm(f64[c]), c
