"""The autotuner's table on the CPU: entries keyed by form and mesh, the
nearest particle count on a log scale, and launch-shape parameters only."""
import json

from ocelot_gb300 import _native as N
from ocelot_gb300 import tuning


def test_record_and_lookup_nearest_particle_count(tmp_path):
    path = str(tmp_path / "table.json")
    assert tuning.lookup("fp32", (64, 64, 64), 2_000_000, path) == {}
    tuning.record("fp32", (64, 64, 64), 200_000, {N.SC_PARAM_KICK_VARIANT: 2}, {"kick_variant": {"2": 10.0}}, path)
    tuning.record("fp32", (64, 64, 64), 2_000_000, {N.SC_PARAM_KICK_VARIANT: 1}, None, path)
    assert tuning.lookup("fp32", (64, 64, 64), 150_000, path) == {N.SC_PARAM_KICK_VARIANT: 2}
    assert tuning.lookup("fp32", (64, 64, 64), 5_000_000, path) == {N.SC_PARAM_KICK_VARIANT: 1}
    assert tuning.lookup("fp32", (64, 64, 64), 500_000, path) == {N.SC_PARAM_KICK_VARIANT: 2}
    assert tuning.lookup("fp32", (64, 64, 64), 700_000, path) == {N.SC_PARAM_KICK_VARIANT: 1}
    assert tuning.lookup("fp64", (64, 64, 64), 2_000_000, path) == {}
    assert tuning.lookup("fp32", (63, 63, 63), 2_000_000, path) == {}
    # re-recording a particle count replaces its entry
    tuning.record("fp32", (64, 64, 64), 2_000_000, {N.SC_PARAM_KICK_VARIANT: 4}, None, path)
    table = json.load(open(path))
    assert [e["n"] for e in table["fp32/64x64x64"]] == [200_000, 2_000_000]
    assert tuning.lookup("fp32", (64, 64, 64), 2_000_000, path) == {N.SC_PARAM_KICK_VARIANT: 4}


def test_committed_table_holds_valid_parameters():
    table = tuning.load_table(tuning.TABLE_PATH)
    for k, entries in table.items():
        form, mesh = k.split("/")
        assert form in ("fp32", "fp64")
        assert len(mesh.split("x")) == 3
        for e in entries:
            assert e["n"] >= 1
            for name, v in e["params"].items():
                assert name in tuning.PARAM_NAMES.values()
                if name == "kick_variant":
                    assert 0 <= v < N.SC_KICK_NVARIANTS
                elif name in ("fft_plane_fwd", "fft_plane_inv"):
                    assert v in (0, 1)
                elif name in ("fft_cols_x", "fft_cols_y"):
                    assert v in (0, 2, 4, 8, 16)
            # every candidate the tuner timed is recorded with its time
            for name, times in e.get("us", {}).items():
                assert name in tuning.PARAM_NAMES.values()
                assert str(e["params"][name]) in times
