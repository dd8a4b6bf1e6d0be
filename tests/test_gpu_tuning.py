"""Launch shapes chosen by the autotuner change no result: every kick tiling
(tile size, tile buffers, particles per thread, blocks per SM) gives the same
bits as the default, for even and odd particle counts (the odd last particle
is kicked outside the bulk copies) and several meshes; the tuner itself
refuses a candidate that changes a bit."""
import numpy as np
import pytest

from conftest import has_gpu
from oracle import sc_oracle

pytestmark = pytest.mark.gpu

if not has_gpu():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch  # noqa: E402

from ocelot_gb300 import _native as N  # noqa: E402
from ocelot_gb300 import tuning  # noqa: E402
from ocelot_gb300.sc import Engine  # noqa: E402

DEV = torch.device("cuda", 0)


@pytest.mark.parametrize("n,mesh", [(300_000, (64, 64, 64)), (100_001, (32, 32, 64)), (1_537, (16, 16, 16))])
def test_every_kick_variant_gives_the_same_bits(n, mesh):
    rp, q = sc_oracle.gaussian_beam(n, 21, charge=1e-9)
    buf = torch.zeros((6, n + (n & 1)), dtype=torch.float64, device=DEV)
    r0 = torch.from_numpy(rp).to(DEV)
    dq = torch.from_numpy(q).to(DEV)
    d = buf[:, :n]
    eng = Engine(mesh, "fp32", DEV, tuned=False)
    outs = []
    for v in range(N.SC_KICK_NVARIANTS):
        eng.set_param(N.SC_PARAM_KICK_VARIANT, v)
        assert eng.get_param(N.SC_PARAM_KICK_VARIANT) == v
        for _ in range(2):          # the second kick reuses the cached Green's function
            d.copy_(r0)
            eng.kick(d, dq, n, 0.130, 0.1)
        eng.check_status()
        outs.append(d.cpu().numpy())
    for v in range(1, N.SC_KICK_NVARIANTS):
        assert np.array_equal(outs[v], outs[0]), v
    assert not np.array_equal(outs[0], rp)


def test_tuner_picks_an_identical_variant_and_records_it(tmp_path):
    path = str(tmp_path / "t.json")
    res = tuning.tune((32, 32, 32), 200_000, "fp32", DEV, reps=2, warmup=1, save=True, path=path)
    assert res["identical"]
    v = res["params"]["kick_variant"]
    assert 0 <= v < N.SC_KICK_NVARIANTS
    assert set(res["us"]["kick_variant"]) == {str(i) for i in range(N.SC_KICK_NVARIANTS)}
    assert tuning.lookup("fp32", (32, 32, 32), 200_000, path)[N.SC_PARAM_KICK_VARIANT] == v
    assert set(res["params"]) == {"kick_variant", "fft_plane_fwd", "fft_plane_inv", "fft_cols_x", "fft_cols_y"}


def test_bad_variant_is_refused():
    eng = Engine((16, 16, 16), "fp32", DEV, tuned=False)
    with pytest.raises(ValueError, match=r"\[sc error 1\]"):
        eng.set_param(N.SC_PARAM_KICK_VARIANT, N.SC_KICK_NVARIANTS)


@pytest.mark.parametrize("precision,fields", [("fp32", "spectral"), ("fp32", "difference"), ("fp64", "difference")])
def test_fft_plane_parameters_give_the_same_bits(precision, fields):
    """Plane-fused or separate FFT passes, forward and inverse: the same lines
    through the same transform code, so the kick is bit-identical."""
    from ocelot_gb300.sc import plan_mode
    n, mesh = 100_001, (48, 48, 48)
    rp, q = sc_oracle.gaussian_beam(n, 23, charge=1e-9)
    r0 = torch.from_numpy(rp).to(DEV)
    dq = torch.from_numpy(q).to(DEV)
    d = torch.zeros((6, n + 1), dtype=torch.float64, device=DEV)[:, :n]
    eng = Engine(mesh, precision, DEV, plan_mode(precision, fields=fields), tuned=False)
    outs = []
    for fwd, inv in ((1, 1), (0, 1), (1, 0), (0, 0)):
        eng.set_param(N.SC_PARAM_FFT_PLANE_FWD, fwd)
        eng.set_param(N.SC_PARAM_FFT_PLANE_INV, inv)
        d.copy_(r0)
        eng.kick(d, dq, n, 0.130, 0.1)
        eng.check_status()
        outs.append(d.cpu().numpy())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])


@pytest.mark.parametrize("precision,fields,mesh", [("fp32", "spectral", (48, 48, 48)), ("fp32", "difference", (96, 96, 96)),
                                                   ("fp64", "difference", (48, 48, 48))])
def test_fft_columns_per_block_give_the_same_bits(precision, fields, mesh):
    """Columns per block of the x pass and of the separate y passes group
    independent lines into blocks: every choice gives the same bits."""
    from ocelot_gb300.sc import plan_mode
    n = 100_001
    rp, q = sc_oracle.gaussian_beam(n, 29, charge=1e-9)
    r0 = torch.from_numpy(rp).to(DEV)
    dq = torch.from_numpy(q).to(DEV)
    d = torch.zeros((6, n + 1), dtype=torch.float64, device=DEV)[:, :n]
    eng = Engine(mesh, precision, DEV, plan_mode(precision, fields=fields), tuned=False)
    eng.set_param(N.SC_PARAM_FFT_PLANE_FWD, 0)  # the separate y pass forward too
    eng.set_param(N.SC_PARAM_FFT_PLANE_INV, 0)
    outs = []
    for cx, cy in ((0, 0), (16, 4), (2, 16), (8, 8), (4, 2)):
        eng.set_param(N.SC_PARAM_FFT_COLS_X, cx)
        eng.set_param(N.SC_PARAM_FFT_COLS_Y, cy)
        assert (eng.get_param(N.SC_PARAM_FFT_COLS_X), eng.get_param(N.SC_PARAM_FFT_COLS_Y)) == (cx, cy)
        d.copy_(r0)
        eng.kick(d, dq, n, 0.130, 0.1)
        eng.check_status()
        outs.append(d.cpu().numpy())
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    with pytest.raises(ValueError, match=r"\[sc error 1\]"):
        eng.set_param(N.SC_PARAM_FFT_COLS_X, 3)
