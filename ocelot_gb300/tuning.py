"""Autotuner of the kick's launch shapes, keyed by (form, mesh, particle count).

The plan's launch-shape parameters (``sc_plan_set_param``) change how the
work is cut into blocks and tiles, never the arithmetic: every candidate must
give bit-identical particles, and the tuner checks that before it times
anything.  For one (form, mesh, N) it kicks a seeded Gaussian beam on the
GPU with each candidate, times the stages the candidate changes with the
library's stage events (L2 flushed before each kick), and keeps the fastest.  Results go to a small JSON table -- by
default ``tuning_table.json`` beside this module, or the file named by
``OCELOT_SC_TUNING`` -- that ``Engine`` reads: before a kick of N particles
it applies the entry of its form and mesh whose particle count is nearest to
N on a log scale.  A mesh without an entry keeps the defaults.

The reference has no counterpart; its only knob is the FFT thread count
(ocelot/cpbd/sc.py:152-160).
"""
from __future__ import annotations

import json
import math
import os
import threading

from . import _native as N

TABLE_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_table.json")

# parameter -> candidate values (the plan's launch-shape knobs)
def candidates():
    return {N.SC_PARAM_KICK_VARIANT: list(range(N.SC_KICK_NVARIANTS)),
            N.SC_PARAM_FFT_PLANE_FWD: [1, 0], N.SC_PARAM_FFT_PLANE_INV: [1, 0],
            N.SC_PARAM_FFT_COLS_X: [0, 8, 4], N.SC_PARAM_FFT_COLS_Y: [0, 8, 4]}


PARAM_NAMES = {N.SC_PARAM_KICK_VARIANT: "kick_variant", N.SC_PARAM_FFT_PLANE_FWD: "fft_plane_fwd",
               N.SC_PARAM_FFT_PLANE_INV: "fft_plane_inv", N.SC_PARAM_FFT_COLS_X: "fft_cols_x",
               N.SC_PARAM_FFT_COLS_Y: "fft_cols_y"}
# the stages (sc_profile_read) each parameter changes: a candidate is timed by
# the sum of these stage times, which a few-microsecond difference does not
# drown in the rest of the kick
PARAM_STAGES = {N.SC_PARAM_KICK_VARIANT: ("kick",), N.SC_PARAM_FFT_PLANE_FWD: ("convolve", "join_wait"),
                N.SC_PARAM_FFT_PLANE_INV: ("convolve", "field"),
                N.SC_PARAM_FFT_COLS_X: ("convolve", "join_wait", "field"),
                N.SC_PARAM_FFT_COLS_Y: ("convolve", "join_wait", "field")}
_NAME_TO_PARAM = {v: k for k, v in PARAM_NAMES.items()}

_lock = threading.Lock()
_cache: dict = {}


def table_path() -> str:
    return os.environ.get("OCELOT_SC_TUNING", TABLE_PATH)


def load_table(path: str | None = None) -> dict:
    path = path or table_path()
    with _lock:
        if path in _cache:
            return _cache[path]
        try:
            with open(path) as f:
                table = json.load(f)
        except (OSError, ValueError):
            table = {}
        _cache[path] = table
        return table


def key(precision: str, shape) -> str:
    return f"{precision}/{'x'.join(str(int(v)) for v in shape)}"


def lookup(precision: str, shape, n: int, path: str | None = None) -> dict:
    """{param: value} of the table entry of this form and mesh nearest to n
    (log scale); {} when there is none."""
    entries = load_table(path).get(key(precision, shape))
    if not entries or n < 1:
        return {}
    best = min(entries, key=lambda e: abs(math.log(max(int(e["n"]), 1)) - math.log(n)))
    return {_NAME_TO_PARAM[k]: int(v) for k, v in best["params"].items() if k in _NAME_TO_PARAM}


def record(precision: str, shape, n: int, params: dict, timings: dict | None = None, path: str | None = None):
    """Store a tuned entry (replacing one of the same particle count)."""
    path = path or table_path()
    table = dict(load_table(path))
    k = key(precision, shape)
    entries = [e for e in table.get(k, []) if int(e["n"]) != int(n)]
    e = {"n": int(n), "params": {PARAM_NAMES[p]: int(v) for p, v in params.items()}}
    if timings:
        e["us"] = timings
    entries.append(e)
    table[k] = sorted(entries, key=lambda e: e["n"])
    tmp = path + ".tmp"
    with open(tmp, "w") as f:
        json.dump(table, f, indent=1, sort_keys=True)
    os.replace(tmp, path)
    with _lock:
        _cache[path] = table


def _beam(n: int, device, seed: int = 1):
    """A seeded Gaussian beam (the benchmark's shape) on the device, rows on
    an even stride so that the bulk-copy kernels run."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    buf = torch.empty((6, n + (n & 1)), dtype=torch.float64, device=device)
    for row, sig in enumerate((50e-6, 1e-5, 50e-6, 1e-5, 100e-6, 1e-4)):
        buf[row].normal_(0.0, sig, generator=g)
    return buf[:, :n], torch.full((n,), 1e-9 / n, dtype=torch.float64, device=device)


def tune(shape, n: int, precision: str = "fp32", device=None, energy_gev: float = 0.130, zstep: float = 0.1,
         reps: int = 5, warmup: int = 2, save: bool = False, path: str | None = None) -> dict:
    """Time every candidate of every parameter (one parameter at a time, the
    others at their current best) on a seeded beam of n particles, by the
    stages the parameter changes (library stage events); returns
    {"params": best, "us": {param name: {value: us of those stages}}, "identical": True}.
    Raises if a candidate changes a single bit of the result."""
    import torch
    from .sc import Engine, cuda_device
    dev = cuda_device(device)
    eng = Engine(tuple(int(v) for v in shape), precision, dev, tuned=False)
    eng.ensure(n)
    rp0, q = _beam(n, dev)
    rp = torch.empty_like(rp0)
    flush_w = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)

    def kick_once(stages=None):
        rp.copy_(rp0)
        flush_w.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.kick(rp, q, n, energy_gev, zstep)
        b.record(stream)
        b.synchronize()
        if stages is None:
            return a.elapsed_time(b) * 1e3
        ms, _ = eng.profile_read()
        return sum(ms[k] for k in stages) * 1e3

    best = {p: eng.get_param(p) for p in candidates()}
    ref = None
    timings = {}
    for p, values in candidates().items():
        us = {}
        for v in values:
            eng.set_param(p, v)
            for _ in range(warmup):
                kick_once()
            eng.check_status()
            if ref is None:
                ref = rp.clone()
            elif not torch.equal(rp, ref):
                raise RuntimeError(f"{PARAM_NAMES[p]}={v} changed the kick's result: launch shapes must not")
            eng.profile(True)
            us[v] = min(kick_once(PARAM_STAGES[p]) for _ in range(reps))
            eng.profile(False)
            eng.check_status()
        best[p] = min(us, key=us.get)
        eng.set_param(p, best[p])
        timings[PARAM_NAMES[p]] = {str(k): round(t, 2) for k, t in us.items()}
    if save:
        record(precision, shape, n, best, timings, path)
    return {"params": {PARAM_NAMES[p]: v for p, v in best.items()}, "us": timings, "identical": True,
            "n": n, "mesh": list(shape), "form": precision}
