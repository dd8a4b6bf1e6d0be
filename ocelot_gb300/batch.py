"""Many beams kicked together: one launch per stage for all of them.

``BeamBatch`` holds a set of GPU-resident beams, each with its own mesh, plan
and workspace (its Green's-function table stays there between kicks), and
kicks them all through ``sc_kick_batched``: 15 kernel launches per kick
whatever the number of beams, every launch a concatenation of the beams'
grids driven by a device work table.  Each beam's arithmetic is that of a
single kick (``SpaceCharge.apply`` in the FP32 form with the exact
fixed-point deposit), so its result is bit-identical to kicking it alone.

The reference kicks one beam per ``SpaceCharge.apply`` call
(ocelot/cpbd/sc.py:208-251, called from track(), ocelot/cpbd/track.py:476-478);
this is the same operation for many beams at once.
"""
from __future__ import annotations

import ctypes as C
import math

from . import _native as N
from .sc import Engine, check_beam_tensors, cuda_device, plan_mode


class BeamBatch:
    """Beams kicked together on one GPU (FP32 form, fixed-point deposit).

    ``add(rparticles, q_array, energy_gev, nmesh_xyz, zstep)`` registers a
    beam (torch CUDA tensors, float64 [6, N] with contiguous rows and [N]);
    ``commit()`` uploads the work table; ``kick()`` kicks every beam
    (asynchronous, current stream); ``graph()`` records one batched kick as
    a CUDA graph to replay.  ``igf="exact"`` uses the FP64 8-corner IGF on
    the whole octant instead of the hybrid table; ``fields`` as in
    ``SpaceCharge`` (spectral by default).

    The table holds each beam's workspace: when an engine's workspace is
    allocated anew (a solo kick of more particles grew it), ``kick()``,
    ``transport()`` and a graph's ``replay()`` upload the table again first.
    After ``graph()`` the batch's launch shape is fixed (see ``graph``).
    """

    def __init__(self, device=None, igf: str = "hybrid", max_beams: int = 1024, fields: str = "spectral"):
        import torch
        if not torch.cuda.is_available():
            raise N.NativeLibraryError("ocelot_gb300 needs a CUDA device; there is no CPU fallback")
        self.lib = N.lib()
        self.device = cuda_device(device)
        self.mode = plan_mode("fp32", "fixed", igf, fields)
        self.max_beams = int(max_beams)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            N.check(self.lib.sc_batch_create(C.byref(h), self.max_beams))
        self.handle = h
        self.beams = []      # (engine, rp, q, E, zstep, tmap or None)
        self._table = None
        self._maps = None
        self._ws = None      # the workspaces the uploaded table holds

    def __del__(self):
        try:
            if getattr(self, "handle", None) is not None and self.handle.value:
                self.lib.sc_batch_destroy(self.handle)
        except Exception:
            pass

    def __len__(self):
        return len(self.beams)

    def add(self, rparticles, q_array, energy_gev: float, nmesh_xyz, zstep: float, engine: Engine | None = None,
            tmap=None):
        """Register a beam; returns its index.  A new plan and workspace are
        made for it unless ``engine`` (an FP32 Engine of the same mesh, not
        used by another beam) is given.  ``tmap`` = (R [6x6], B [6]): the
        transport ``transport()`` applies before the kick, or None."""
        if len(self.beams) >= self.max_beams:
            raise ValueError(f"batch is full ({self.max_beams} beams)")
        if rparticles.dim() != 2 or rparticles.shape[0] != 6 or rparticles.stride(1) != 1:
            raise ValueError("rparticles must be [6, N] with contiguous rows")
        n = int(rparticles.shape[1])
        if n == 0:
            raise ValueError("zero-size array: the space-charge kick needs at least one particle")
        check_beam_tensors(rparticles, q_array, n, self.device)
        if engine is None:
            engine = Engine(tuple(int(v) for v in nmesh_xyz), "fp32", self.device, self.mode)
        engine.ensure(n)
        engine.apply_tuning(n)  # the beam's FFT tiling in the batched passes
        self.beams.append((engine, rparticles, q_array, float(energy_gev), float(zstep), tmap))
        self._table = None
        return len(self.beams) - 1

    def set_step(self, index: int, zstep: float, tmap=None):
        """Kick length and transport map of beam ``index`` for the next step."""
        e, rp, q, E, _, _ = self.beams[index]
        self.beams[index] = (e, rp, q, E, float(zstep), tmap)
        self._table = None

    def clear(self):
        """Forget every beam (their engines are not touched)."""
        self.beams = []
        self._table = None

    def commit(self):
        """Upload the work table (asynchronous copy on the current stream)."""
        import torch
        import numpy as np
        arr = (N.ScBeam * max(1, len(self.beams)))()
        maps = []
        for i, (e, rp, q, E, dz, tm) in enumerate(self.beams):
            mp = None
            if tm is not None:
                m = np.ascontiguousarray(np.concatenate([np.asarray(tm[0], dtype=np.float64).reshape(36),
                                                         np.asarray(tm[1], dtype=np.float64).reshape(6)]))
                maps.append(m)
                mp = m.ctypes.data_as(C.POINTER(C.c_double))
            arr[i] = N.ScBeam(e.plan.value, e.ws.data_ptr(), e.ws.numel(), rp.data_ptr(), rp.stride(0),
                              q.data_ptr(), int(rp.shape[1]), E, dz, math.nan, math.nan, mp)
        with torch.cuda.device(self.device):
            N.check(self.lib.sc_batch_set(self.handle, arr, len(self.beams),
                                          C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)))
        self._table, self._maps = arr, maps   # copied by sc_batch_set; kept for inspection
        self._ws = self._workspaces()

    def _workspaces(self):
        return [(e.ws.data_ptr(), e.ws.numel()) if e.ws is not None else None for e, *_ in self.beams]

    def _refresh(self):
        """Upload the table if it changed or a beam's workspace was allocated anew."""
        if self._table is None or self._ws != self._workspaces():
            self.commit()

    def kick(self):
        """Kick every beam once (asynchronous on the current stream)."""
        import torch
        self._refresh()
        with torch.cuda.device(self.device):
            N.check(self.lib.sc_kick_batched(self.handle,
                                             C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)))

    def transport(self):
        """Apply every beam's transport map (one launch, current stream)."""
        import torch
        self._refresh()
        with torch.cuda.device(self.device):
            N.check(self.lib.sc_tmap_batched(self.handle,
                                             C.c_void_p(torch.cuda.current_stream(self.device).cuda_stream)))

    def profile(self, enable: bool = True):
        """Stage events between the batched launches (read with profile_read)."""
        N.check(self.lib.sc_batch_profile_enable(self.handle, 1 if enable else 0))

    def profile_read(self):
        """{stage: ms} of the last batched kick (synchronous)."""
        ms = (C.c_float * N.SC_NSTAGES)()
        N.check(self.lib.sc_batch_profile_read(self.handle, ms))
        names = [self.lib.sc_profile_stage_name(i).decode() for i in range(N.SC_NSTAGES)]
        return dict(zip(names, [float(v) for v in ms]))

    @property
    def launches(self) -> int:
        return int(self.lib.sc_batch_launches(self.handle))

    def graph(self, stream=None):
        """Record one batched kick as a CUDA graph; ``.replay()`` kicks the
        beams of the table current at replay time.

        The recorded launches fix the batch's shape: afterwards ``commit()``
        accepts new kick lengths, energies and maps for the same beams, but
        raises for other particle counts or meshes, an added or removed beam,
        or a kick length set to zero (kick those beams with a new batch)."""
        import torch
        self._refresh()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.device(self.device):
            torch.cuda.synchronize(self.device)
            with torch.cuda.graph(g, stream=stream):
                self.kick()
        return BatchGraph(self, g)

    def check(self):
        """Wait for the GPU and raise if any beam latched an error."""
        for e, *_ in self.beams:
            e.check_status()


class BatchGraph:
    """A batched kick recorded as a CUDA graph (``BeamBatch.graph``)."""

    def __init__(self, batch: BeamBatch, graph):
        self.batch = batch
        self.graph = graph

    def replay(self):
        """Kick the beams of the batch's current table again (current
        stream); the table is uploaded first if it changed since."""
        self.batch._refresh()
        self.graph.replay()
