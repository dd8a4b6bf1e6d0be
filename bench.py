"""Benchmark of the GB300 3D space-charge kick (Ocelot SpaceCharge.apply).

Workload: the 2M-particle / 64^3 precision-form configuration -- a seeded
uncorrelated 6D Gaussian beam (sigma_x = sigma_y = 50 um, sigma_x' = sigma_y'
= 1e-5, sigma_tau = 100 um, sigma_delta = 1e-4), 130 MeV, 1 nC split equally,
one kick of dz = 0.1 m per step.  Synthetic data, no dataset involved.

A step is one kick.  ``value`` is particle-kicks/s of the FP32 form (spectral
fields, the library's default; the headline) with the particles resident in
HBM, timed with CUDA events around each kick; L2 (129 MB, larger than the
112 MB of particles and charges) is flushed between timed kicks by writing a
256 MB buffer and then reading another 256 MB buffer (the read writes the
flush's dirty lines back to HBM before the kick starts, so the kick does not
pay for them).  Timed the same way and reported beside it: the FP32 form with
the reference's difference fields and the FP64 form, each with its stage
times; the errors of phi, of E at the particles (recorded by the kick itself)
and of the momentum kicks of both FP32 forms against the FP64 form.  ``e2e``
is the same metric through ``SpaceCharge.apply`` on a host ``ParticleArray``
in pinned memory: the host->device copy of rparticles and q_array and the
device->host copy of rparticles are inside the timed region of every step;
``e2e_pageable`` the same with pageable numpy arrays, and ``e2e_roofline``
the step's copies at the measured host-link bandwidth against the e2e step.
``config1`` (the plain FP64 form: 200k particles, 63^3, 10 kicks per step)
and ``config3`` (the FP32 stress workload: 10M particles at 6.5 MeV on
128x128x256, 20 kicks per step) are timed with their rooflines, CPU baselines
and errors; ``batched`` (96 uneven beams, one graph-replayed batched kick per
step, with its stage times) and ``serving`` (Poisson-arriving FODO tracking
jobs, latency percentiles) complete the line.

Modes that print their own line and exit: --kick-only (the FP32 kick alone),
--profile-form fp32|fp64 with --n and --mesh (one form's kicks on a chosen
size: the small cases of the ncu captures), --transport N (the tracking
kernels), --tune [--tune-save] (the autotuner on this GPU).

--impl reference times the CPU restatement of the reference's algorithm
(oracle/sc_oracle.py: numpy, scipy.ndimage and scipy.fft on all host cores)
on the same workload; the reference itself is pure Python and does not run
on the GPU machine.

N > 1 (torchrun): replicas only -- each rank kicks its own beam, no
collective on the data path; value = all ranks' particle-kicks / max time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "particle-kicks/s, 2M p/64^3 grid: FP32 vs FP64 form at <=1e-5 rel err; p99 latency"
N_PART = 2_000_000
MESH = [64, 64, 64]
E_GEV = 0.130
CHARGE = 1e-9
DZ = 0.1
SEED = 2024

# algorithmic HBM bytes: rparticles read + write (2 x 48 B) + q read (8 B) per particle,
# plus the charge grid written and the potential read once (2 x w x N_g)
B_PER_PARTICLE = 104
B_KICK_KERNEL_PER_PARTICLE = 96  # gather+kick: rparticles read + write
# DRAM traffic of one k_kick32_tma launch per particle, from the ncu capture
# summarised in profiles/k_kick32_tma_4M_64cube.txt (200.39 MB read + 132.49 MB
# written at 4M particles); traffic grows with the particles, so it is scaled
# to the bench's n
KICK_TRAFFIC_PER_PARTICLE = (200.39e6 + 132.49e6) / 4e6


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def beam(n, seed=SEED):
    from oracle.sc_oracle import gaussian_beam  # seeded synthetic input generator (numpy)
    return gaussian_beam(n, seed, charge=CHARGE)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        # the raw samples go to OCELOT_SC_CLOCKS_DIR when set (the summary is in the JSON line either way)
        self.path = os.path.join(os.environ.get("OCELOT_SC_CLOCKS_DIR", "/tmp"), f"clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def peaks():
    try:
        d = json.load(open(os.path.join(REPO, "MEASURED_PEAKS.json")))
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def time_form(precision, n, steps, warmup, dev, flush, fields="spectral", mesh=MESH):
    """Device-resident kicks; per-kick CUDA events; per-stage events from the library."""
    import torch
    from ocelot_gb300 import SpaceCharge
    rp, q = beam(n)
    d_rp = torch.from_numpy(rp).to(dev)
    d_q = torch.from_numpy(q).to(dev)
    sc = SpaceCharge(nmesh_xyz=mesh, precision=precision, device=dev, fields=fields)
    eng = sc.engine()
    eng.ensure(n)
    stream = torch.cuda.current_stream(dev)
    for _ in range(warmup):  # the timed step's sequence, untimed
        flush()
        sc.apply_device(d_rp, d_q, E_GEV, DZ)
    sc.check()
    kick_ms, stages, launches = [], {}, 0
    for _ in range(steps):
        flush()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        sc.apply_device(d_rp, d_q, E_GEV, DZ)
        b.record(stream)
        b.synchronize()
        kick_ms.append(a.elapsed_time(b))
        launches += eng.launches()
    sc.check()
    # the stage split comes from separate kicks: the library's stage events
    # sit between the kernels and keep consecutive kernels from overlapping
    # their launch (programmatic dependent launch), so they are not recorded
    # during the timed kicks
    eng.profile(True)
    for _ in range(steps):
        flush()
        sc.apply_device(d_rp, d_q, E_GEV, DZ)
        st, _ = eng.profile_read()
        for k, v in st.items():
            stages.setdefault(k, []).append(v)
    sc.check()
    eng.profile(False)
    return kick_ms, {k: sum(v) / len(v) for k, v in stages.items()}, launches


def time_e2e(precision, n, steps, warmup, dev, pinned=True):
    """Through SpaceCharge.apply on a host ParticleArray; the host->device copy
    of rparticles and q_array and the device->host copy of rparticles are
    inside the timed region.  pinned=False: plain numpy arrays (pageable), as
    Ocelot's track() hands them to SpaceCharge.apply (track.py:476-478)."""
    import numpy as np
    import torch
    from ocelot_gb300 import ParticleArray, SpaceCharge
    rp, q = beam(n)
    pa = ParticleArray(0)
    if pinned:
        h_rp = torch.empty((6, n), dtype=torch.float64).pin_memory()
        h_q = torch.empty(n, dtype=torch.float64).pin_memory()
        h_rp.numpy()[:] = rp
        h_q.numpy()[:] = q
        pa.rparticles = h_rp.numpy()
        pa.q_array = h_q.numpy()
    else:
        pa.rparticles = rp
        pa.q_array = q
    pa.E = E_GEV
    sc = SpaceCharge(nmesh_xyz=MESH, precision=precision, device=dev)
    for _ in range(warmup):
        sc.apply(pa, DZ)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    for _ in range(steps):
        sc.apply(pa, DZ)  # H2D, kick, status check, D2H: synchronous per step
    torch.cuda.synchronize(dev)
    dt = time.perf_counter() - t0
    assert np.isfinite(pa.rparticles).all()
    return dt, 6 * n * 8 + n * 8, 6 * n * 8


def host_link(dev, h2d_bytes, d2h_bytes):
    """Pinned host<->device copy bandwidth (GB/s, best of 5 CUDA-event timed
    copies of the e2e step's own sizes) -- the bound of an end-to-end step."""
    import torch
    hi = torch.empty(h2d_bytes, dtype=torch.uint8).pin_memory()
    ho = torch.empty(d2h_bytes, dtype=torch.uint8).pin_memory()
    di = torch.empty(h2d_bytes, dtype=torch.uint8, device=dev)
    do = torch.empty(d2h_bytes, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    best = [math.inf, math.inf]
    for _ in range(5):
        for k, (dst, src) in enumerate(((di, hi), (ho, do))):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            dst.copy_(src, non_blocking=True)
            b.record(stream)
            b.synchronize()
            best[k] = min(best[k], a.elapsed_time(b) * 1e-3)
    return h2d_bytes / best[0] / 1e9, d2h_bytes / best[1] / 1e9


# Configurations of the metric timed beside the headline (each a sequence of
# kicks on a seeded synthetic beam; a step is the whole sequence)
PLAIN_200K_63 = {"key": "config1", "form": "fp64", "n": 200_000, "mesh": [63, 63, 63], "E": 0.130,
                 "charge": 250e-12, "dz": 0.1, "kicks": 10, "beam": "gauss",
                 "workload": "plain FP64 form: 200k particles, 6D Gaussian (sigma_x = sigma_y = 50 um, "
                             "sigma_x' = sigma_y' = 1e-5, sigma_tau = 100 um, sigma_delta = 1e-4), 130 MeV, "
                             "250 pC, 63^3 mesh, 10 kicks of 0.1 m"}
STRESS_10M_128X128X256 = {
    "key": "config3", "form": "fp32", "fields": "spectral", "n": 10_000_000, "mesh": [128, 128, 256],
    "E": 0.0065, "charge": 500e-12, "dz": 0.05, "kicks": 20, "beam": "flat",
    "workload": "low-energy stress case, FP32 form with spectral fields: 10M particles at 6.5 MeV, 500 pC, "
                "flat-top tau of 2 mm with 100 um Gaussian edges, chirp delta += -10 tau, transverse "
                "Gaussian 200 um with a 1 mrad x-tau tilt, 128x128x256 mesh, 20 kicks of 0.05 m"}


def config_beam(cfg, seed=SEED):
    from oracle.sc_oracle import flat_top_beam, gaussian_beam  # seeded synthetic input generators (numpy)
    if cfg["beam"] == "gauss":
        return gaussian_beam(cfg["n"], seed, charge=cfg["charge"])
    return flat_top_beam(cfg["n"], seed, charge=cfg["charge"])


def form_errors(cfg, dev, seed=SEED + 1, fp32_mode=None):
    """The FP32 form against the FP64 form on one kick of the same beam --
    relative RMS errors of the grid potential, of the field at the particles
    as the kick used it (both forms record it, SC_PARAM_RECORD_FIELD) and of
    the momentum kicks (x', y', delta).  The FP64 form is itself within 1e-10
    of the oracle (tests), so these are the FP32 form's errors."""
    import torch
    from ocelot_gb300 import SpaceCharge, _native as N
    rp, q = config_beam(cfg, seed)
    n, mesh = rp.shape[1], cfg["mesh"]
    r0 = torch.from_numpy(rp).to(dev)
    d_q = torch.from_numpy(q).to(dev)
    out, phi, field = {}, {}, {}
    for prec in ("fp64", "fp32"):
        d = torch.empty((6, n + (n & 1)), dtype=torch.float64, device=dev)[:, :n]
        d.copy_(r0)
        kw = {} if (prec == "fp64" or not fp32_mode) else fp32_mode
        sc = SpaceCharge(nmesh_xyz=mesh, precision=prec, device=dev, **kw)
        eng = sc.engine()
        eng.set_param(N.SC_PARAM_RECORD_FIELD, 1)
        sc.apply_device(d, d_q, cfg["E"], cfg["dz"])
        sc.check()
        out[prec] = d
        phi[prec] = eng.region("phi").to(torch.float64)
        field[prec] = eng.region("field", n).to(torch.float64)
        del sc, eng
    rel = lambda a, b: float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b))  # noqa: E731
    dp = {}
    for r, name in ((1, "dxp"), (3, "dyp"), (5, "ddelta")):
        k64 = out["fp64"][r] - r0[r]
        k32 = out["fp32"][r] - r0[r]
        dp[name] = float(torch.sqrt(torch.mean((k32 - k64) ** 2)) / torch.sqrt(torch.mean(k64 ** 2)))
    e_at = {c: rel(field["fp32"][k], field["fp64"][k]) for k, c in enumerate(("Ex", "Ey", "Ez"))}
    res = {"phi": rel(phi["fp32"], phi["fp64"]), "E_at_particles": e_at, "kick": dp,
           "vs": "FP64 form (itself within 1e-10 of the oracle), one kick, same beam", "beam_seed": seed}
    del out, phi, field
    torch.cuda.empty_cache()
    return res


def padded_length(n: int) -> int:
    """The FFT length the library pads a mesh axis of n cells to: the smallest
    2^k or 3 * 2^k (8 .. 512) holding the linear convolution (>= 2n - 1)."""
    fits = [L for L in [8 << k for k in range(7)] + [12 << k for k in range(6)] if L >= 2 * n - 1]
    return min(fits) if fits else 0


def fp64_work_per_kick(mesh):
    """Algorithmic FP64 work of one kick of the plain form, counted by the
    reference's operations: its potential is three complex 3D FFTs of the
    padded grid (sc.py:135-168), 5 M log2 M flops each, and its Green's function
    evaluates 3 arctangents, 3 logarithms and a square root per corner of the
    (nx+1)(ny+1)(nz+1) lattice (sc.py:109-133).  The library's passes do less
    than the FFT count (real-to-half-complex transforms, lines that are all
    padding skipped), so the count is not a rate to hold against the FP64 peak."""
    M = math.prod(padded_length(int(v)) for v in mesh)
    return {"fft_flops_reference_count": 3 * 5 * M * math.log2(M),
            "padded_grid": [padded_length(int(v)) for v in mesh],
            "igf_transcendentals": 7 * math.prod(int(v) + 1 for v in mesh)}


def time_config(cfg, steps, warmup, dev, flush, cpu_threads=None):
    """A configuration's kick sequence, device-resident: every step restores
    the initial beam (outside the timed region), flushes L2 and times the
    whole sequence with CUDA events on the launching stream."""
    import torch
    from ocelot_gb300 import SpaceCharge
    rp, q = config_beam(cfg)
    n, mesh = cfg["n"], cfg["mesh"]
    r0 = torch.from_numpy(rp).to(dev)
    d_rp = torch.empty((6, n + (n & 1)), dtype=torch.float64, device=dev)[:, :n]
    d_q = torch.from_numpy(q).to(dev)
    sc = SpaceCharge(nmesh_xyz=mesh, precision=cfg["form"], device=dev, fields=cfg.get("fields", "difference"))
    eng = sc.engine()
    eng.ensure(n)
    stream = torch.cuda.current_stream(dev)
    ms, launches = [], 0
    for it in range(warmup + steps):
        d_rp.copy_(r0)
        flush()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for _ in range(cfg["kicks"]):
            sc.apply_device(d_rp, d_q, cfg["E"], cfg["dz"])
            if it >= warmup:
                launches += eng.launches()
        b.record(stream)
        b.synchronize()
        if it >= warmup:
            ms.append(a.elapsed_time(b))
    sc.check()
    eng.profile(True)
    d_rp.copy_(r0)
    flush()
    sc.apply_device(d_rp, d_q, cfg["E"], cfg["dz"])
    stages, _ = eng.profile_read()
    eng.profile(False)
    sc.check()
    del sc, eng, d_rp, r0
    torch.cuda.empty_cache()
    t = statistics.mean(ms) * 1e-3
    w = 8 if cfg["form"] == "fp64" else 4
    ncell = math.prod(mesh)
    b_kick = B_PER_PARTICLE * n + 2 * w * ncell
    peak, kind = peaks()
    achieved = b_kick * cfg["kicks"] / t / 1e9
    out = {"workload": cfg["workload"], "form": cfg["form"], "fields": cfg.get("fields", "difference"),
           "n_particles": n, "mesh": mesh,
           "kicks_per_step": cfg["kicks"], "steps": steps, "warmup": warmup,
           "value": n * cfg["kicks"] / t, "unit": "particle-kicks/s", "ms_per_step": t * 1e3,
           "ms_per_kick": t * 1e3 / cfg["kicks"], "gpu_launches": launches, "stages_ms_one_kick": stages,
           "l2": "flushed before each step; the kicks of a step run back to back",
           "roofline": {"bound": "hbm" if cfg["form"] == "fp32" else
                        "fp64 pipe: every FP64-form kernel with arithmetic keeps it 65-85% busy (ncu); the bytes "
                        "below are far from the HBM bound",
                        "algorithmic_bytes_per_kick": b_kick, "achieved": achieved, "unit": "GB/s",
                        "peak": peak, "frac": achieved / peak, "peak_kind": peak_kind_text(kind)}}
    if cfg["form"] == "fp64":
        out["fp64_work_per_kick"] = fp64_work_per_kick(mesh)
    if cpu_threads:
        from oracle import sc_oracle
        rp_c, q_c = config_beam(cfg)
        t0 = time.perf_counter()
        sc_oracle.sc_apply(rp_c, q_c, cfg["E"], cfg["dz"], mesh, fft_workers=cpu_threads)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": n / dt, "unit": "particle-kicks/s", "cores": cpu_threads, "kind": "port",
                               "sample": f"1 kick of the same {n}-particle beam and mesh, oracle/sc_oracle.py "
                                         f"(numpy + scipy.ndimage, scipy.fft with {cpu_threads} workers)"}
    return out


def peak_kind_text(kind):
    return "of measured (MEASURED_PEAKS.json hbm_gbs)" if kind == "measured" else "of fallback"


def cpu_port(n, kicks_max, budget_s, threads):
    """The oracle (numpy/scipy restatement of the reference) on the host cores."""
    from oracle import sc_oracle
    rp, q = beam(n)
    sc_oracle.sc_apply(rp, q, E_GEV, DZ, MESH, fft_workers=threads)  # warm-up
    times = []
    t_start = time.perf_counter()
    while len(times) < kicks_max and (time.perf_counter() - t_start < budget_s or len(times) < 1):
        t0 = time.perf_counter()
        sc_oracle.sc_apply(rp, q, E_GEV, DZ, MESH, fft_workers=threads)
        times.append(time.perf_counter() - t0)
    return n * len(times) / sum(times), len(times)


# batched workload: 96 seeded Gaussian beams, N log-uniform in [1e4, 4e6], mesh
# drawn from these five, E uniform 5-500 MeV, charge uniform 20-500 pC,
# sigma_x (= sigma_y) and sigma_tau each log-uniform in 20-500 um
BATCH_MESHES = [(32, 32, 32), (48, 48, 48), (64, 64, 64), (96, 96, 96), (32, 32, 128)]


def batch_specs(nbeams=96, seed=SEED + 4):
    import numpy as np
    rng = np.random.default_rng(seed)
    lg = lambda a, b: float(10 ** rng.uniform(math.log10(a), math.log10(b)))  # noqa: E731
    out = []
    for i in range(nbeams):
        out.append({"n": int(round(lg(1e4, 4e6))), "mesh": BATCH_MESHES[int(rng.integers(len(BATCH_MESHES)))],
                    "E": float(rng.uniform(0.005, 0.5)), "Q": float(rng.uniform(20e-12, 500e-12)),
                    "sx": lg(20e-6, 500e-6), "st": lg(20e-6, 500e-6), "seed": seed * 1000 + i})
    return out


def device_beam(spec, dev):
    """Seeded Gaussian beam generated on the device (rows padded to an even stride)."""
    import torch
    n = spec["n"]
    g = torch.Generator(device=dev)
    g.manual_seed(spec["seed"])
    buf = torch.empty((6, n + (n & 1)), dtype=torch.float64, device=dev)
    for row, sig in enumerate((spec["sx"], 1e-5, spec["sx"], 1e-5, spec["st"], 1e-4)):
        buf[row].normal_(0.0, sig, generator=g)
    q = torch.full((n,), spec["Q"] / n, dtype=torch.float64, device=dev)
    return buf[:, :n], q


def time_batched(steps, warmup, dev, nbeams=96):
    """The 96-beam workload kicked by sc_kick_batched (one launch per stage,
    recorded once as a CUDA graph and replayed), against the same beams
    kicked one sc_kick after another on one stream.  nbeams < 96: the first
    nbeams beams of the same draw (the small case of the batch's profiles)."""
    import torch
    from ocelot_gb300.batch import BeamBatch
    specs = batch_specs()[:nbeams]
    batch = BeamBatch(dev)
    beams = []
    for sp in specs:
        rp, q = device_beam(sp, dev)
        batch.add(rp, q, sp["E"], sp["mesh"], DZ)
        beams.append((rp, q, sp))
    batch.commit()
    g = batch.graph()
    stream = torch.cuda.current_stream(dev)
    for _ in range(warmup):
        g.replay()
    torch.cuda.synchronize(dev)
    ms = []
    for _ in range(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        g.replay()
        b.record(stream)
        b.synchronize()
        ms.append(a.elapsed_time(b))
    batch.check()
    # stage split of the batched kick (events between the launches: separate kicks)
    batch.profile(True)
    stage_ms = {}
    for _ in range(3):
        batch.kick()
        for k, v in batch.profile_read().items():
            stage_ms.setdefault(k, []).append(v)
    batch.profile(False)
    stage_ms = {k: sum(v) / len(v) for k, v in stage_ms.items()}
    batch.check()
    # the same beams, one plain kick each, on one stream (same plans and workspaces)
    seq_ms = []
    for it in range(warmup + steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for (eng, rp, q, E, dz, _) in batch.beams:
            eng.kick(rp, q, int(rp.shape[1]), E, dz)
        b.record(stream)
        b.synchronize()
        if it >= warmup:
            seq_ms.append(a.elapsed_time(b))
    batch.check()
    ntot = sum(sp["n"] for sp in specs)
    cells = sum(math.prod(sp["mesh"]) for sp in specs)
    t = statistics.mean(ms)
    ts = statistics.mean(seq_ms)
    alg = B_PER_PARTICLE * ntot + 2 * 4 * cells
    return {
        "workload": "96 seeded Gaussian beams, N log-uniform 1e4-4e6, meshes from 32^3/48^3/64^3/96^3/32x32x128, "
                    "E 5-500 MeV, Q 20-500 pC, sigma_x and sigma_tau log-uniform 20-500 um; one 0.1 m kick "
                    "per beam per step (FP32 form); 15 launches per step recorded as one CUDA graph",
        "beams": len(specs), "particles": ntot, "value": ntot / (t * 1e-3), "unit": "particle-kicks/s",
        "ms_per_step": t, "launches_per_step": 15, "stages_ms": stage_ms,
        "sequential": {"value": ntot / (ts * 1e-3), "ms_per_step": ts, "launches_per_step": 15 * len(specs),
                       "how": "one sc_kick per beam, one stream, same plans and workspaces"},
        "batched_over_sequential": ts / t,
        "hbm": {"algorithmic_bytes_per_step": alg, "achieved_gbs": alg / (t * 1e-3) / 1e9},
        "l2": "not flushed: the 96 beams' particles (several GB) exceed L2",
    }


# serving workload: Poisson-arriving tracking jobs, each a seeded Gaussian beam
# (sigma_x = sigma_y = 200 um, sigma_x' = sigma_y' = 2e-5, sigma_tau = 100 um,
# sigma_delta = 1e-4, 130 MeV, 250 pC) with N log-uniform in [5e4, 5e6] on a
# mesh of 32^3, 48^3, 64^3 or 96^3, tracked through 10 FODO cells with a kick
# every 0.25 m (96 kicks) and first-order transport between kicks
SERVE_MESHES = [(32, 32, 32), (48, 48, 48), (64, 64, 64), (96, 96, 96)]
SERVE_RATES = [4.0, 12.0, 24.0, 36.0, 48.0]
SERVE_JOBS = 30


def serve_requests(count, seed):
    import numpy as np
    from ocelot_gb300 import serve as S
    rng = np.random.default_rng(seed)
    lattice = S.fodo(10)
    out = []
    for i in range(count):
        n = int(round(10 ** rng.uniform(math.log10(5e4), math.log10(5e6))))
        mesh = SERVE_MESHES[int(rng.integers(len(SERVE_MESHES)))]
        out.append(S.Request(S.BeamSpec(n=n, seed=seed * 1000 + i), lattice, mesh, 0.25, 1))
    return out


def time_serving(dev, rates=SERVE_RATES, jobs=SERVE_JOBS):
    import numpy as np
    from ocelot_gb300 import serve as S
    srv = S.Server(dev, max_active=64)
    S.poisson_run(srv, serve_requests(4, SEED + 50), rate_hz=100.0, seed=0)   # warm-up
    results = []
    for k, rate in enumerate(rates):
        reqs = serve_requests(jobs, SEED + 60 + k)
        ticks0 = srv.ticks
        lat, wall, kicks, _ = S.poisson_run(srv, reqs, rate_hz=rate, seed=k + 1)
        results.append({"rate_hz": rate, "jobs": len(reqs), "p50_s": float(np.percentile(lat, 50)),
                        "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()),
                        "max_s": float(lat.max()), "throughput": kicks / wall, "unit": "particle-kicks/s",
                        "wall_s": wall, "ticks": srv.ticks - ticks0,
                        "offered_particle_kicks_per_s": rate * float(np.mean([r.beam.n for r in reqs])) * 96})
    sustained = [r for r in results if r["throughput"] >= 0.9 * r["offered_particle_kicks_per_s"]]
    return {"workload": "Poisson-arriving FODO tracking jobs (10 cells, kick every 0.25 m = 96 kicks, first-order "
                        "transport between kicks), N log-uniform 5e4-5e6, mesh 32^3/48^3/64^3/96^3, FP32 form; "
                        "latency = arrival to tracked particles in pinned host memory",
            "rates": results, "peak_hbm_bytes": srv.peak_used,
            "sustained_rate_hz": max((r["rate_hz"] for r in sustained), default=None),
            "p99_at_sustained_s": (max(sustained, key=lambda r: r["rate_hz"])["p99_s"] if sustained else None)}


def headline_config(n, ws):
    """The workload of the headline line (the same dict in both arms)."""
    return {"workload": "2M particles, 64^3 mesh, 130 MeV, 1 nC, one 0.1 m kick per step (FP32 form, spectral "
                        "fields)",
            "n_particles": n, "mesh": MESH, "form": "fp32",
            "l2": "flushed between kicks (256 MB write, then 256 MB read)", "parallelism": f"replicas x{ws}"}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    n = N_PART
    from oracle import sc_oracle
    rp, q = beam(n)
    for _ in range(args.warmup):
        sc_oracle.sc_apply(rp, q, E_GEV, DZ, MESH, fft_workers=threads)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        sc_oracle.sc_apply(rp, q, E_GEV, DZ, MESH, fft_workers=threads)
    dt = time.perf_counter() - t0
    value = n * args.steps / dt
    sample = (f"{n} particles of the 2M/64^3 workload per step, {args.steps} kicks; oracle/sc_oracle.py "
              f"(numpy + scipy.ndimage, scipy.fft with {threads} workers)")
    out = {"metric": METRIC, "value": value, "unit": "particle-kicks/s", "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
           "data": "synthetic seeded 6D Gaussian beam",
           "config": headline_config(n, ws),
           "reference_arithmetic": "FP64 (the reference's own; it has no FP32 form)",
           "impl": "reference",
           "cpu_baseline": {"value": value, "unit": "particle-kicks/s", "cores": threads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": value, "unit": "particle-kicks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def time_transport(n: int, steps: int, warmup: int):
    """The tracking transport kernels alone on a seeded device beam of n
    particles: one slice of each record form (sc_slices_apply) and the beam
    moments (sc_moments), CUDA-event time per launch.  Prints one JSON line;
    the launch order (per form: warmup, then steps launches) is fixed, so a
    profiler can pick a form's last launch by its index."""
    import ctypes as C
    import numpy as np
    import torch
    from ocelot_gb300 import _native as N
    from ocelot_gb300 import cavity as CV
    from ocelot_gb300 import track as T
    from ocelot_gb300.second_order import element_map2, pack_map
    dev = torch.device("cuda", 0)
    lib = N.lib()
    g = torch.Generator(device=dev).manual_seed(1)
    rp = torch.randn((6, n), generator=g, device=dev, dtype=torch.float64) * 1e-3
    s = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    E = 0.05
    cav = CV.Cavity(l=1.0377, v=0.0195, phi=18.7, freq=1.3e9)
    rec_c, kinds_c, _ = CV.section_records(cav, 0.3, 0.02, E)
    rec_d = pack_map(*element_map2(T.Drift(l=0.02), 0.02, E))
    rec_q = pack_map(*element_map2(T.Quadrupole(l=0.02, k1=1.5), 0.02, E))
    R1, B1 = T.element_map(T.Quadrupole(l=0.02, k1=1.5), 0.02, E)
    rec_1 = pack_map(R1, np.zeros((6, 6, 6)), B1)
    forms = [("cavity", rec_c, list(kinds_c)),
             ("drift_general", rec_d[None], [CV.SLICE_MAP]), ("quad_general", rec_q[None], [CV.SLICE_MAP]),
             ("drift", rec_d[None], [CV.map_kind(rec_d)]), ("quad", rec_q[None], [CV.map_kind(rec_q)]),
             ("quad_first_order", rec_1[None], [CV.map_kind(rec_1)])]
    out = {"workload": f"tracking transport kernels, {n} particles (rows {48 * n / 1e6:.0f} MB; above L2 from 2.7M)",
           "unit": "us per launch"}

    def timed(fn):
        for _ in range(warmup):
            fn()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record()
        for _ in range(steps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps * 1e3

    for name, recs, kinds in forms:
        maps = torch.from_numpy(np.ascontiguousarray(recs)).to(dev)
        kd = torch.tensor(kinds, dtype=torch.int32, device=dev)
        us = timed(lambda: N.check(lib.sc_slices_apply(C.c_void_p(maps.data_ptr()), C.c_void_p(kd.data_ptr()),
                                                       len(kinds), C.c_void_p(rp.data_ptr()), rp.stride(0), n, s)))
        out[name] = {"us": round(us, 2), "kinds": kinds, "rows_read_written_GBs": round(96 * n / (us * 1e-6) / 1e9, 1)}
    # the composed first-order map of the FODO tracking loop and the batched serving path (sc_tmap_apply)
    for name, e in (("tmap_quad", T.Quadrupole(l=0.2, k1=1.5)), ("tmap_tilted_quad", T.Quadrupole(l=0.2, k1=1.5,
                                                                                                 tilt=0.1))):
        R, B = T.element_map(e, 0.2, E)
        Rc = np.ascontiguousarray(R, dtype=np.float64)
        Bc = np.ascontiguousarray(B, dtype=np.float64)
        us = timed(lambda: N.check(lib.sc_tmap_apply(Rc.ctypes.data_as(C.POINTER(C.c_double)),
                                                     Bc.ctypes.data_as(C.POINTER(C.c_double)),
                                                     C.c_void_p(rp.data_ptr()), rp.stride(0), n, s)))
        out[name] = {"us": round(us, 2), "rows_read_written_GBs": round(96 * n / (us * 1e-6) / 1e9, 1)}
    mom = torch.zeros((1, 21), dtype=torch.float64, device=dev)
    scr = torch.zeros(int(lib.sc_moments_scratch_bytes()), dtype=torch.uint8, device=dev)
    for bounds in (0, 1):
        us = timed(lambda: N.check(lib.sc_moments(C.c_void_p(rp.data_ptr()), rp.stride(0), n, None, 1, bounds,
                                                  -0.5, 0.5, C.c_void_p(mom.data_ptr()), C.c_void_p(scr.data_ptr()),
                                                  s)))
        out["moments" + ("_bounds" if bounds else "")] = {"us": round(us, 2), "launches": 4 if bounds else 2}
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=N_PART)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip timing the FP64 form")
    ap.add_argument("--no-batch", action="store_true", help="skip the 96-beam batched leg")
    ap.add_argument("--no-serve", action="store_true", help="skip the serving leg")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the plain 200k / 63^3 FP64 and the 10M / 128x128x256 FP32 legs")
    ap.add_argument("--kick-only", action="store_true",
                    help="time the FP32 kick alone (no other leg): the small case for profiling")
    ap.add_argument("--transport", type=int, default=0, metavar="N",
                    help="time the tracking transport kernels (slice forms, moments) on N particles and exit")
    ap.add_argument("--profile-form", choices=["fp32", "fp64"], default=None,
                    help="time kicks of one form alone on --n particles and a --mesh^3 mesh, print one line and exit "
                         "(the small cases of the profiles)")
    ap.add_argument("--mesh", default="64", help="mesh cells per axis, or nx,ny,nz")
    ap.add_argument("--batch-only", type=int, default=0, metavar="BEAMS",
                    help="time the batched leg alone on the first BEAMS beams of its draw, print one line and exit")
    ap.add_argument("--tune", action="store_true",
                    help="autotune the launch shapes on the benchmark meshes and particle counts, print the "
                         "timings (and store them in the tuning table with --tune-save) and exit")
    ap.add_argument("--tune-save", action="store_true")
    args = ap.parse_args()
    mesh = [int(v) for v in str(args.mesh).split(",")]
    mesh = mesh * 3 if len(mesh) == 1 else mesh
    if len(mesh) != 3:
        ap.error("--mesh takes one size or nx,ny,nz")
    if args.profile_form:
        import torch
        dev = torch.device("cuda", 0)
        flush_buf = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
        kick, stages, launches = time_form(args.profile_form, args.n, args.steps, max(args.warmup, 3), dev,
                                           flush_buf.zero_, mesh=mesh)
        print(json.dumps({"form": args.profile_form, "n": args.n, "mesh": mesh, "ms_per_kick": kick,
                          "stages_ms": stages, "launches": launches}), flush=True)
        return
    if args.batch_only:
        import torch
        dev = torch.device("cuda", 0)
        print(json.dumps(time_batched(args.steps, max(args.warmup, 3), dev, args.batch_only)), flush=True)
        return
    if args.tune:
        from ocelot_gb300 import tuning
        cases = [((64, 64, 64), 2_000_000), ((64, 64, 64), 200_000), ((63, 63, 63), 200_000),
                 ((128, 128, 256), 10_000_000), ((32, 32, 32), 100_000), ((96, 96, 96), 4_000_000),
                 ((48, 48, 48), 1_000_000), ((32, 32, 128), 500_000)]
        for shape, n in cases:
            print(json.dumps(tuning.tune(shape, n, "fp32", save=args.tune_save)), flush=True)
        return
    if args.transport:
        time_transport(args.transport, args.steps, max(args.warmup, 3))
        return
    if args.kick_only:
        args.no_cpu = args.no_fp64 = args.no_batch = args.no_serve = args.no_configs = True
    args.warmup = max(args.warmup, 3)

    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    n = args.n
    l2_w = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    l2_r = torch.ones(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    l2_sum = torch.empty((), dtype=torch.float32, device=dev)

    def flush():
        # evict L2 (129 MB): write 256 MB, then read 256 MB so that the written
        # lines are back in HBM and L2 holds only clean lines of l2_r
        l2_w.zero_()
        torch.sum(l2_r, dim=0, out=l2_sum)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    barrier()
    with ClockSampler(local) as clk:
        kick32, stages32, launches32 = time_form("fp32", n, args.steps, args.warmup, dev, flush)
        barrier()
    kick64, stages64, _ = ([], {}, 0) if args.no_fp64 else time_form("fp64", n, args.steps, 3, dev, flush)
    kickdf, stagesdf, _ = ([], {}, 0) if args.kick_only else time_form("fp32", n, args.steps, 3, dev, flush,
                                                                     fields="difference")
    e2e_dt, h2d, d2h = (math.nan, 0, 0) if args.kick_only else time_e2e("fp32", n, args.steps, args.warmup, dev)
    e2e_page_dt = math.nan if args.kick_only else time_e2e("fp32", n, args.steps, args.warmup, dev, pinned=False)[0]
    e2e64_dt = math.nan if (args.kick_only or args.no_fp64) else time_e2e("fp64", n, args.steps, args.warmup, dev)[0]
    link = None if args.kick_only else host_link(dev, h2d, d2h)
    threads = os.cpu_count() or 1
    cpu_threads = None if (args.no_cpu or rank != 0) else threads
    configs = {}
    if not args.no_configs:
        for cfg in (PLAIN_200K_63, STRESS_10M_128X128X256):
            configs[cfg["key"]] = time_config(cfg, 3, 1, dev, flush, cpu_threads)
        configs["config3"]["fp32_errors_vs_fp64"] = form_errors(STRESS_10M_128X128X256, dev,
                                                                 fp32_mode={"fields": "spectral"})
        configs["config3"]["fp32_difference_fields_errors_vs_fp64"] = form_errors(STRESS_10M_128X128X256, dev,
                                                                                   fp32_mode={"fields": "difference"})
    batched = None if args.no_batch else time_batched(args.steps, args.warmup, dev)
    serving = None if args.no_serve else time_serving(dev)
    head_cfg = {"n": n, "mesh": MESH, "E": E_GEV, "dz": DZ, "charge": CHARGE, "beam": "gauss"}
    errors = None if args.kick_only else form_errors(head_cfg, dev, fp32_mode={"fields": "spectral"})
    errors_df = None if args.kick_only else form_errors(head_cfg, dev, fp32_mode={"fields": "difference"})
    barrier()

    t32 = sum(kick32) / 1e3
    if ws > 1:
        tt = torch.tensor([t32, e2e_dt], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t32, e2e_dt = float(tt[0]), float(tt[1])
    value = ws * n * args.steps / t32
    e2e_value = ws * n * args.steps / e2e_dt

    peak, peak_kind = peaks()
    # dominant kernel: the stage with the largest share of the FP32 kick
    top = max(stages32, key=stages32.get)
    kick_ms = stages32["kick"]
    achieved_kick = B_KICK_KERNEL_PER_PARTICLE * n / (kick_ms * 1e-3) / 1e9
    whole_ms = statistics.mean(kick32)
    achieved_whole = (B_PER_PARTICLE * n + 2 * 4 * math.prod(MESH)) / (whole_ms * 1e-3) / 1e9

    out = None
    if rank == 0:
        cpu = None
        if not args.no_cpu:
            v, k = cpu_port(N_PART, 5, 10.0, threads)
            cpu = {"value": v, "unit": "particle-kicks/s", "cores": threads, "kind": "port",
                   "sample": f"2M particles, 64^3, {k} kicks of oracle/sc_oracle.py (numpy + scipy.ndimage, "
                             f"scipy.fft with {threads} workers; the rest single-threaded)"}
        e2e_step_ms = e2e_dt / args.steps * 1e3
        link_ms = (h2d / (link[0] * 1e9) + d2h / (link[1] * 1e9)) * 1e3 if link else math.nan
        out = {
            "metric": METRIC, "value": value, "unit": "particle-kicks/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(kick32),
            "ms_each_step": [round(v, 4) for v in kick32],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic seeded 6D Gaussian beam (no dataset)",
            "config": headline_config(n, ws),
            "fp64_form": ({"value": n * args.steps / (sum(kick64) / 1e3), "ms_per_step": statistics.mean(kick64),
                           "stages_ms": stages64,
                           "e2e": ({"value": n * args.steps / e2e64_dt, "unit": "particle-kicks/s",
                                    "ms_per_step": e2e64_dt / args.steps * 1e3, "h2d_bytes_per_step": h2d,
                                    "d2h_bytes_per_step": d2h, "host_memory": "pinned"}
                                   if e2e64_dt == e2e64_dt else None)} if kick64 else None),
            "fp32_over_fp64": (statistics.mean(kick64) / statistics.mean(kick32)) if kick64 else None,
            "fp32_difference_form": ({"value": n * args.steps / (sum(kickdf) / 1e3),
                                      "ms_per_step": statistics.mean(kickdf), "stages_ms": stagesdf,
                                      "errors_vs_fp64": errors_df,
                                      "over_fp64": (statistics.mean(kick64) / statistics.mean(kickdf)) if kick64 else None,
                                      "what": "the FP32 form with the reference's differences of the FP32 potential "
                                              "(fields='difference'); the headline form takes them in Fourier space"}
                                     if kickdf else None),
            "fp32_kick_rel_rms_err_vs_fp64": errors["kick"] if errors else None,
            "fp32_errors_vs_fp64": errors,
            "stages_ms": stages32,
            "roofline": {"bound": "hbm", "kernel": "k_kick32_tma (gather+kick+FP64 accumulate)",
                         "achieved": achieved_kick, "peak": peak, "unit": "GB/s", "frac": achieved_kick / peak,
                         "traffic": KICK_TRAFFIC_PER_PARTICLE * n, "peak_kind": peak_kind_text(peak_kind),
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of k_kick32_tma at 4M "
                                           "particles (profiles/k_kick32_tma_4M_64cube.txt), scaled by particles",
                         "algorithmic_bytes_per_launch": B_KICK_KERNEL_PER_PARTICLE * n,
                         "top_stage": top, "top_stage_ms": stages32[top]},
            "kick_roofline": {"achieved": achieved_whole, "frac": achieved_whole / peak, "unit": "GB/s",
                              "algorithmic_bytes_per_kick": B_PER_PARTICLE * n + 2 * 4 * math.prod(MESH)},
            "e2e": (None if args.kick_only else
                    {"value": e2e_value, "unit": "particle-kicks/s", "h2d_bytes_per_step": h2d,
                     "d2h_bytes_per_step": d2h, "host_memory": "pinned", "ms_per_step": e2e_step_ms}),
            "e2e_pageable": (None if args.kick_only else
                             {"value": n * args.steps / e2e_page_dt, "unit": "particle-kicks/s",
                              "ms_per_step": e2e_page_dt / args.steps * 1e3, "h2d_bytes_per_step": h2d,
                              "d2h_bytes_per_step": d2h,
                              "host_memory": "pageable numpy arrays, as track() passes them"}),
            "e2e_roofline": (None if not link else
                             {"bound": "host link", "h2d_gbs": link[0], "d2h_gbs": link[1], "link_ms": link_ms,
                              "e2e_ms": e2e_step_ms, "frac": link_ms / e2e_step_ms,
                              "how": "the step's copies at the measured pinned copy bandwidth (best of 5, CUDA "
                                     "events) over the measured pinned e2e step"}),
            "e2e_link_frac": (link_ms / e2e_step_ms) if link else None,
            "gpu_launches": launches32,
            "config1": configs.get("config1"),
            "config3": configs.get("config3"),
            "batched": batched,
            "serving": serving,
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
        }
        print(json.dumps(out), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
