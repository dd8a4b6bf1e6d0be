"""Serving space-charge tracking jobs on one GPU with continuous batching.

A request is a beam (a host ParticleArray, or a seeded Gaussian generated on
the device), a lattice section of drifts, quadrupoles and markers, and the
space-charge settings (mesh, Navigator unit step, process step) -- what the
reference runs as ``track(lat, p_array, navi)`` with a SpaceCharge process
(ocelot/cpbd/track.py:431-505).  The server keeps every admitted job's
particles, plan and workspace (its Green's table included) resident in HBM
and advances all of them together: each tick uploads one work table holding
every job's next transport map and kick length, then runs one batched
transport launch and the batched kick (sc_tmap_batched, sc_kick_batched).
Requests that arrive while others are on the GPU wait in a FIFO queue and are
admitted at the next tick once the HBM budget and the slot limit allow; their
steps then share launches with jobs that are already part way down their
lattice.  A finished job's particles are copied to pinned host memory and its
device memory is released.

Every job's arithmetic is its own (per-beam grids, reductions and fixed-point
deposit inside the batched kernels), so a job's result is bit-identical
whether it runs alone or among others, and equal to ``DeviceTrack`` in the
FP32 form.
"""
from __future__ import annotations

import collections
import dataclasses
import math
import time

import numpy as np

from . import _native as N
from .batch import BeamBatch
from .globals import m_e_GeV
from .sc import Engine, cuda_device, plan_mode
from .track import _lattice_sequence, step_maps


@dataclasses.dataclass
class BeamSpec:
    """A seeded, uncorrelated 6D Gaussian beam generated on the device."""
    n: int
    seed: int
    energy_gev: float = 0.130
    charge: float = 250e-12
    sigma_x: float = 200e-6
    sigma_px: float = 2e-5
    sigma_y: float = 200e-6
    sigma_py: float = 2e-5
    sigma_tau: float = 100e-6
    sigma_p: float = 1e-4


@dataclasses.dataclass
class Request:
    beam: object                 # BeamSpec or a host ParticleArray
    elements: object             # lattice (``.sequence``) or element list
    nmesh: tuple = (63, 63, 63)
    unit_step: float = 0.25
    sc_step: int = 1


def fodo(cells: int):
    """``cells`` FODO cells: QF(0.2 m, k1 = +1.2), D(1 m), QD(0.2 m, k1 = -1.2),
    D(1 m), then a Marker so that a process can end on the last element."""
    from .track import Drift, Marker, Quadrupole
    seq = []
    for _ in range(cells):
        seq += [Quadrupole(l=0.2, k1=1.2), Drift(l=1.0), Quadrupole(l=0.2, k1=-1.2), Drift(l=1.0)]
    return seq + [Marker()]


def device_gaussian(spec: BeamSpec, device):
    """rparticles [6, n] (rows on an even stride) and q_array on ``device``."""
    import torch
    n = int(spec.n)
    g = torch.Generator(device=device)
    g.manual_seed(int(spec.seed))
    buf = torch.empty((6, n + (n & 1)), dtype=torch.float64, device=device)
    for row, sig in enumerate((spec.sigma_x, spec.sigma_px, spec.sigma_y, spec.sigma_py, spec.sigma_tau,
                               spec.sigma_p)):
        buf[row].normal_(0.0, float(sig), generator=g)
    return buf[:, :n], torch.full((n,), spec.charge / n, dtype=torch.float64, device=device)


def validate_request(request: Request):
    """Check a request before it is queued and return its step list.

    Everything a job needs is checked here, on the host, so that no admitted
    job can fail a later tick for all the jobs batched with it: the beam's
    shape (rparticles (6, N), q_array of N entries, N >= 1) and energy (above
    the electron's rest energy, as the kick's gamma needs), the mesh (three
    dimensions >= 4), and the step list -- the transport map and kick length
    of every step, which depend only on the line and the energy -- so that a
    line without steps (a zero-length section) is refused instead of being
    admitted as a job that never finishes."""
    b = request.beam
    if isinstance(b, BeamSpec):
        n, E = int(b.n), float(b.energy_gev)
    else:
        shape = np.shape(b.rparticles)
        if len(shape) != 2 or shape[0] != 6:
            raise ValueError(f"rparticles must have shape (6, N), not {shape}")
        n, E = int(shape[1]), float(b.E)
        if np.size(b.q_array) != n:
            raise ValueError(f"q_array has {np.size(b.q_array)} entries for {n} particles")
    if n < 1:
        raise ValueError("zero-size array: the space-charge kick needs at least one particle")
    if not (math.isfinite(E) and E > m_e_GeV):
        raise ValueError(f"beam energy {E} GeV: must be finite and above the electron rest energy")
    if len(request.nmesh) != 3 or min(int(v) for v in request.nmesh) < 4:
        raise ValueError(f"nmesh {request.nmesh}: three dimensions >= 4 needed")
    steps = step_maps(_lattice_sequence(request.elements), E, request.unit_step, int(request.sc_step))
    if not steps:
        raise ValueError("the lattice section has no tracking steps (zero length): nothing to track")
    return steps


class _Job:
    __slots__ = ("id", "req", "t_arrive", "t_admit", "t_done", "n", "E", "mesh", "steps", "next", "engine", "rp",
                 "q", "host", "status", "tick_event", "copy_event", "bytes", "result", "error")

    def __init__(self, jid, req, t_arrive):
        self.id = jid
        self.req = req
        self.t_arrive = t_arrive
        self.t_admit = self.t_done = None
        self.next = 0
        self.steps = None
        self.engine = self.rp = self.q = self.host = self.status = None
        self.tick_event = self.copy_event = self.result = self.error = None
        self.bytes = 0


class Server:
    """Continuous-batching tracking server on one GPU (FP32 form).

    ``hbm_budget``: bytes of device memory the jobs may hold together
    (default: 80% of the free memory when the server starts); ``max_active``:
    jobs kicked together at most; ``inflight``: ticks queued on the GPU
    ahead of the host at most.
    """

    def __init__(self, device=None, hbm_budget=None, max_active: int = 64, inflight: int = 2, igf: str = "hybrid",
                 fields: str = "spectral"):
        import torch
        self.torch = torch
        self.device = cuda_device(device)
        if hbm_budget is None:
            free, _ = torch.cuda.mem_get_info(self.device)
            hbm_budget = int(free * 0.8)
        self.budget = int(hbm_budget)
        self.max_active = int(max_active)
        self.inflight = max(1, int(inflight))
        self.mode = plan_mode("fp32", "fixed", igf, fields)
        self.batch = BeamBatch(self.device, igf=igf, max_beams=self.max_active, fields=fields)
        self.stream = torch.cuda.Stream(self.device)
        self.copy_stream = torch.cuda.Stream(self.device)
        self.pending = collections.deque()
        self.active = []
        self.finishing = []
        self.done = {}
        self.outstanding = collections.deque()
        self.used = 0
        self.peak_used = 0
        self.ticks = 0
        self.kicks = 0               # particle-kicks completed
        self._pool = {}              # mesh -> idle Engines (plans kept, workspaces released)
        self._next_id = 0

    # ---- requests ---------------------------------------------------------
    def submit(self, request: Request, t_arrive: float | None = None) -> int:
        """Queue a request; returns its job id.  ``t_arrive``: its arrival
        time (time.perf_counter()), now by default.  Raises ValueError for a
        request that ``validate_request`` refuses."""
        steps = validate_request(request)
        jid = self._next_id
        self._next_id += 1
        job = _Job(jid, request, time.perf_counter() if t_arrive is None else t_arrive)
        job.steps = steps
        self.pending.append(job)
        return jid

    def busy(self) -> bool:
        return bool(self.pending or self.active or self.finishing)

    def result(self, jid: int):
        """Tracked rparticles (host float64 [6, n]) of a finished job; raises
        ValueError if one of its kicks latched an error on the device."""
        job = self.done[jid]
        if job.error is not None:
            raise ValueError(f"[sc error {job.error}] job {jid}: {N.ERROR_TEXT.get(job.error, 'device error')}")
        return job.result

    def latencies(self):
        return {j.id: j.t_done - j.t_arrive for j in self.done.values()}

    # ---- memory -------------------------------------------------------------
    def _engine(self, mesh):
        pool = self._pool.setdefault(mesh, [])
        return pool.pop() if pool else Engine(mesh, "fp32", self.device, self.mode)

    def _footprint(self, engine, n):
        return int(engine.lib.sc_workspace_bytes(engine.plan, n)) + 6 * 8 * (n + (n & 1)) + 8 * n

    def _admit(self):
        torch = self.torch
        while self.pending and len(self.active) < self.max_active:
            job = self.pending[0]
            req = job.req
            n = int(req.beam.n) if isinstance(req.beam, BeamSpec) else int(np.shape(req.beam.rparticles)[1])
            mesh = tuple(int(v) for v in req.nmesh)
            eng = self._engine(mesh)
            need = self._footprint(eng, n)
            if self.used + need > self.budget and (self.active or self.finishing):
                self._pool[mesh].append(eng)
                return                      # FIFO: wait for memory to be released
            self.pending.popleft()
            job.t_admit = time.perf_counter()
            job.n, job.mesh, job.engine, job.bytes = n, mesh, eng, need
            with torch.cuda.device(self.device), torch.cuda.stream(self.stream):
                eng.ensure(n)
                if isinstance(req.beam, BeamSpec):
                    job.rp, job.q = device_gaussian(req.beam, self.device)
                    job.E = float(req.beam.energy_gev)
                else:
                    pa = req.beam
                    buf = torch.empty((6, n + (n & 1)), dtype=torch.float64, device=self.device)
                    job.rp = buf[:, :n]
                    job.rp.copy_(torch.from_numpy(np.ascontiguousarray(pa.rparticles, dtype=np.float64)).pin_memory(),
                                 non_blocking=True)
                    job.q = torch.from_numpy(np.ascontiguousarray(pa.q_array, dtype=np.float64)).pin_memory().to(
                        self.device, non_blocking=True)
                    job.E = float(pa.E)
            self.used += need
            self.peak_used = max(self.peak_used, self.used)
            self.active.append(job)

    def _release(self, job):
        job.engine.ws = None
        job.engine.cap = -1
        self._pool.setdefault(job.mesh, []).append(job.engine)
        job.engine = job.rp = job.q = None
        self.used -= job.bytes

    # ---- the GPU side -------------------------------------------------------
    def _tick(self) -> bool:
        torch = self.torch
        ready = [j for j in self.active if j.next < len(j.steps)]
        if not ready:
            return False
        while len(self.outstanding) >= self.inflight:
            self.outstanding.popleft().synchronize()
        b = self.batch
        b.clear()
        for j in ready:
            R, B, zstep, _ = j.steps[j.next]
            b.add(j.rp, j.q, j.E, j.mesh, zstep, engine=j.engine, tmap=(R, B))
        with torch.cuda.device(self.device), torch.cuda.stream(self.stream):
            b.commit()
            b.transport()
            b.kick()
            ev = torch.cuda.Event()
            ev.record(self.stream)
        self.outstanding.append(ev)
        self.ticks += 1
        for j in ready:
            j.next += 1
            self.kicks += j.n
            if j.next == len(j.steps):
                j.tick_event = ev
        still = []
        for j in self.active:
            if j.next >= len(j.steps):
                self._copy_back(j)
                self.finishing.append(j)
            else:
                still.append(j)
        self.active = still
        return True

    def _copy_back(self, job):
        torch = self.torch
        with torch.cuda.device(self.device), torch.cuda.stream(self.copy_stream):
            self.copy_stream.wait_event(job.tick_event)
            job.host = torch.empty((6, job.n), dtype=torch.float64).pin_memory()
            job.host.copy_(job.rp, non_blocking=True)
            # the device status of the last kick and the first error of any kick
            job.status = torch.empty(2, dtype=torch.int32).pin_memory()
            job.status[0:1].copy_(job.engine.region("status"), non_blocking=True)
            job.status[1:2].copy_(job.engine.region("first_error"), non_blocking=True)
            job.copy_event = torch.cuda.Event()
            job.copy_event.record(self.copy_stream)

    def _retire(self) -> bool:
        moved = False
        keep = []
        for j in self.finishing:
            if j.copy_event.query():
                j.t_done = time.perf_counter()
                code = int(j.status[1]) or int(j.status[0])
                j.error = code or None
                j.result = j.host.numpy()
                self._release(j)
                self.done[j.id] = j
                moved = True
            else:
                keep.append(j)
        self.finishing = keep
        while self.outstanding and self.outstanding[0].query():
            self.outstanding.popleft()
        return moved

    def pump(self) -> bool:
        """One scheduling round: retire finished copies, admit waiting
        requests, launch a tick.  Returns whether anything happened."""
        a = self._retire()
        self._admit()
        t = self._tick()
        return a or t

    def drain(self, timeout_s: float = 600.0):
        """Run until every submitted request has finished."""
        t0 = time.perf_counter()
        while self.busy():
            if not self.pump():
                time.sleep(0.0002)
            if time.perf_counter() - t0 > timeout_s:
                raise TimeoutError("serving did not drain")


def poisson_run(server: Server, requests, rate_hz: float, seed: int = 0):
    """Submit ``requests`` at Poisson arrival times of ``rate_hz`` (wall clock)
    while serving; returns per-job latencies [s], the wall time from the first
    arrival to the last completion and the particle-kicks done."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_hz, len(requests))
    gaps[0] = 0.0
    arrive = np.cumsum(gaps)
    kicks0 = server.kicks
    ids = []
    t0 = time.perf_counter()
    i = 0
    while i < len(requests) or server.busy():
        now = time.perf_counter() - t0
        while i < len(requests) and arrive[i] <= now:
            ids.append(server.submit(requests[i], t0 + arrive[i]))
            i += 1
        if not server.pump():
            nxt = arrive[i] - (time.perf_counter() - t0) if i < len(requests) else 0.0
            time.sleep(min(max(nxt, 0.0), 0.0005) if nxt > 0 else 0.0002)
    t_end = max(server.done[j].t_done for j in ids)
    lat = np.array([server.done[j].t_done - server.done[j].t_arrive for j in ids])
    return lat, t_end - t0, server.kicks - kicks0, ids
