"""Particle containers.

``ParticleArray`` is the data layout the kick mutates, as in Ocelot
(ocelot/cpbd/beam/particle.py:79-84): ``rparticles`` is a float64 [6, N]
array of MAD coordinates (x, x', y, y', tau, delta), ``q_array`` float64 [N]
charges in coulomb, ``E`` the reference energy in GeV and ``s`` the position.
Only those fields are provided here; any object with them (including Ocelot's
own ParticleArray) works with ``SpaceCharge.apply``.

``DeviceParticleArray`` keeps the same fields resident on the GPU as torch
tensors so that kicks and transfer maps run back to back without host copies.
"""
from __future__ import annotations

import numpy as np


class ParticleArray:
    def __init__(self, n=0):
        self.rparticles = np.zeros((6, n))
        self.q_array = np.zeros(n)
        self.s = 0.0
        self.E = 0.0

    def size(self):
        return self.rparticles.shape[1]

    def x(self):
        return self.rparticles[0]

    def px(self):
        return self.rparticles[1]

    def y(self):
        return self.rparticles[2]

    def py(self):
        return self.rparticles[3]

    def tau(self):
        return self.rparticles[4]

    def p(self):
        return self.rparticles[5]


class DeviceParticleArray:
    """GPU-resident twin of a ParticleArray (torch float64 tensors)."""

    def __init__(self, rparticles, q_array, E: float, s: float = 0.0):
        import torch
        self.rparticles = rparticles
        self.q_array = q_array
        self.E = float(E)
        self.s = float(s)
        if not (isinstance(rparticles, torch.Tensor) and rparticles.is_cuda and rparticles.dtype == torch.float64):
            raise TypeError("rparticles must be a CUDA float64 tensor")
        if rparticles.dim() != 2 or rparticles.shape[0] != 6:
            raise ValueError(f"rparticles must have shape (6, N), not {tuple(rparticles.shape)}")
        if not (isinstance(q_array, torch.Tensor) and q_array.dtype == torch.float64 and
                q_array.device == rparticles.device and q_array.dim() == 1 and
                q_array.numel() == rparticles.shape[1]):
            raise ValueError(f"q_array must be a float64 vector of {rparticles.shape[1]} charges on "
                             f"{rparticles.device}")

    @classmethod
    def from_host(cls, p_array, device=None, pinned_staging=True):
        import torch
        dev = torch.device(device or "cuda")
        rp = torch.from_numpy(np.ascontiguousarray(p_array.rparticles))
        q = torch.from_numpy(np.ascontiguousarray(p_array.q_array, dtype=np.float64))
        if pinned_staging:
            rp = rp.pin_memory()
            q = q.pin_memory()
        return cls(rp.to(dev, non_blocking=True), q.to(dev, non_blocking=True), p_array.E, getattr(p_array, "s", 0.0))

    def to_host(self, p_array=None):
        host = self.rparticles.cpu().numpy()
        if p_array is None:
            p_array = ParticleArray(host.shape[1])
            p_array.q_array = self.q_array.cpu().numpy()
        p_array.rparticles[...] = host
        p_array.E = self.E
        p_array.s = self.s
        return p_array

    def size(self):
        return int(self.rparticles.shape[1])
