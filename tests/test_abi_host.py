"""CPU checks: the C-ABI library loads and exports every declared symbol, and
the host-side plugin surface behaves like the reference's (no GPU calls)."""
import os
import re
import shutil

import numpy as np
import pytest

from conftest import REPO

HEADER = os.path.join(REPO, "include", "ocelot_sc.h")


def _declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:[\w\s\*]+?)\b(sc_\w+)\s*\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def native():
    from ocelot_gb300 import _native
    if not os.path.exists(_native.LIB_PATH):
        if shutil.which("nvcc") is None and not os.path.exists("/usr/local/cuda/bin/nvcc"):
            pytest.skip("library not built and no nvcc to build it")
        from ocelot_gb300 import build
        build.build()
    return _native


def test_header_declares_the_api():
    names = _declared()
    for must in ("sc_plan_create", "sc_kick", "sc_el_field", "sc_potential", "sc_sym_kernel",
                 "sc_sort_keys", "sc_tmap_apply", "sc_read_status", "sc_last_error"):
        assert must in names


def test_header_constants_match_the_bindings():
    """Every integer constant the header defines (modes, status codes,
    parameters, regions, limits) has the same value in the Python bindings."""
    from ocelot_gb300 import _native
    text = re.sub(r"/\*.*?\*/", "", open(HEADER).read(), flags=re.S)
    defs = dict(re.findall(r"^#define\s+(SC_\w+)\s+(0x[0-9a-fA-F]+|\d+)\s*$", text, flags=re.M))
    assert len(defs) > 20
    regions = {k: int(v, 0) for k, v in defs.items() if k.startswith("SC_REGION_")}
    for name, value in defs.items():
        if name.startswith("SC_REGION_"):
            continue
        assert hasattr(_native, name), f"{name} is not in the bindings"
        assert getattr(_native, name) == int(value, 0), name
    assert sorted(_native.REGIONS.values()) == sorted(regions.values())
    assert len({v for k, v in defs.items() if k.startswith("SC_ERR_")}) == \
        len([k for k in defs if k.startswith("SC_ERR_")])       # distinct status codes


def test_library_exports_every_declared_symbol(native):
    lib = native.lib()
    names = _declared()
    assert names
    for name in names:
        assert hasattr(lib, name), name
        assert name in native.SIGNATURES, f"{name} has no ctypes signature"
    assert set(native.SIGNATURES) == set(names)
    assert lib.sc_abi_version() == native.SC_ABI_VERSION


def test_library_argument_checks_without_gpu(native):
    """Host-side validation answers before any CUDA call."""
    import ctypes as C
    lib = native.lib()
    plan = C.c_void_p()
    assert lib.sc_plan_create(C.byref(plan), 3, 63, 63, 0) == native.SC_ERR_ARG
    assert "must be >= 4" in native.last_error()
    assert lib.sc_plan_create(C.byref(plan), 63, 63, 63, 7) == native.SC_ERR_ARG
    assert lib.sc_sort_keys(None, 10, 0, None, None, None, 0, None) == native.SC_ERR_ARG


def test_spacecharge_surface_matches_reference():
    from ocelot_gb300 import SpaceCharge
    sc = SpaceCharge()
    assert sc.step == 1 and sc.nmesh_xyz == [63, 63, 63] and sc.random_mesh is False
    assert sc.random_seed == 10 and sc.debug is False and sc.low_order_kick is True
    for attr in ("indx0", "indx1", "s_start", "s_stop", "start_elem", "end_elem", "z0", "energy"):
        assert getattr(sc, attr) is None
    sc2 = SpaceCharge(step=5, nmesh_xyz=[31, 31, 63], random_mesh=True)
    assert repr(sc2) == "<SpaceCharge: step=5, nmesh_xyz=[31, 31, 63], random_mesh=True>"


def test_prepare_seeds_global_rng_like_reference():
    from ocelot_gb300 import SpaceCharge
    np.random.seed(123)
    SpaceCharge().prepare(None)
    a = np.random.uniform()
    np.random.seed(10)
    assert a == np.random.uniform()


def test_random_mesh_draw_order():
    from ocelot_gb300 import SpaceCharge
    sc = SpaceCharge(random_mesh=True)
    sc.prepare(None)
    s, o = sc._mesh_draws()
    np.random.seed(10)
    assert s == np.random.uniform(low=1, high=1.1)
    assert o == np.random.uniform(low=-0.5, high=0.5)


def test_zero_step_returns_without_touching_particles():
    from ocelot_gb300 import ParticleArray, SpaceCharge
    pa = ParticleArray(10)
    pa.rparticles[:] = 1.0
    SpaceCharge().apply(pa, 0.0)  # sc.py:210-212: no GPU needed
    assert np.all(pa.rparticles == 1.0)


def test_empty_beam_raises_value_error():
    from ocelot_gb300 import ParticleArray, SpaceCharge
    pa = ParticleArray(0)
    pa.E = 0.13
    with pytest.raises(ValueError):
        SpaceCharge().apply(pa, 0.1)


def test_bad_precision_rejected():
    from ocelot_gb300 import SpaceCharge
    with pytest.raises(ValueError):
        SpaceCharge(precision="fp16")
