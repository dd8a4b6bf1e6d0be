"""Failure detection of the device-side waits, without a fault or a hang.

The FP32 form's frame, extent and kick kernels wait for their bulk copies on
mbarriers with an iteration limit.  Here a test-only limit of zero tries makes
the first wait of one kernel give up at once: the kernel latches
SC_ERR_TIMEOUT, waits (with the normal limit) for the copies it has in flight
and returns, the rest of the kick skips its work, sc_read_status reports the
timeout, the particles are unchanged, and the next kick with the normal limit
is bit-identical to a kick that never timed out.  (The reference has no
device waits; its only failure reports are Python exceptions, sc.py:104-107.)
"""
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


def _beam(n, seed=5):
    rp, q = sc_oracle.gaussian_beam(n, seed, charge=250e-12)
    buf = torch.zeros((6, n + (n & 1)), dtype=torch.float64, device=DEV)   # 16-byte rows: the bulk-copy kernels
    buf[:, :n] = torch.from_numpy(rp).to(DEV)
    return buf[:, :n], torch.from_numpy(q).to(DEV)


@pytest.mark.parametrize("kernel", [N.SC_WAIT_FRAME, N.SC_WAIT_EXTENT, N.SC_WAIT_KICK])
@pytest.mark.parametrize("n", [20_001, 300_000])
def test_wait_that_runs_out_reports_timeout_and_leaves_particles(kernel, n):
    d_rp, d_q = _beam(n)
    ref_rp, ref_q = _beam(n)
    sc = SpaceCharge(nmesh_xyz=[32, 32, 32], precision="fp32", device=DEV)
    ref = SpaceCharge(nmesh_xyz=[32, 32, 32], precision="fp32", device=DEV)
    eng = sc.engine()
    before = d_rp.clone()
    eng.set_wait_limit(kernel, 0)
    sc.apply_device(d_rp, d_q, 0.13, 0.1)
    with pytest.raises(N.ScError) as exc:
        sc.check()
    assert exc.value.code == N.SC_ERR_TIMEOUT
    assert "gave up" in str(exc.value)
    assert torch.equal(d_rp, before)
    # the normal limit again: the context is usable and the kick is exact
    eng.set_wait_limit(-1, -1)
    sc.apply_device(d_rp, d_q, 0.13, 0.1)
    sc.check()
    ref.apply_device(ref_rp, ref_q, 0.13, 0.1)
    ref.check()
    assert torch.equal(d_rp, ref_rp)
    assert not torch.equal(d_rp, before)
    # the first-error word still holds the timeout of the earlier kick
    assert int(eng.region("first_error")[0]) == N.SC_ERR_TIMEOUT


def test_wait_limit_arguments():
    sc = SpaceCharge(nmesh_xyz=[16, 16, 16], precision="fp32", device=DEV)
    eng = sc.engine()
    with pytest.raises(ValueError, match=r"\[sc error 1\]"):
        eng.set_wait_limit(3, 0)
    eng.set_wait_limit(-1, 10 ** 12)   # clamped to the default
