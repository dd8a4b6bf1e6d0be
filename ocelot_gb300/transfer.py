"""First-order transport of GPU-resident particles between kicks.

``TransferMapDevice`` applies X <- R.X + B to the 6 x N rparticles of a
``DeviceParticleArray`` in place, as Ocelot's TransferMap.mul_p_array does to
host arrays (ocelot/cpbd/transformations/transfer_map.py:40-50).  The 6x6
matrix must already include the element tilt (FirstOrderParams.get_rotated_R,
ocelot/cpbd/tm_params/first_order_params.py:26-28).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N


def tmap_apply(R, B, rparticles) -> None:
    """rparticles (CUDA float64 [6, N], rows contiguous) <- R.rparticles + B."""
    import torch
    R = np.ascontiguousarray(np.asarray(R, dtype=np.float64).reshape(6, 6))
    B = np.ascontiguousarray(np.asarray(B, dtype=np.float64).reshape(6))
    if not (isinstance(rparticles, torch.Tensor) and rparticles.is_cuda and rparticles.dtype == torch.float64):
        raise TypeError("rparticles must be a CUDA float64 tensor")
    if rparticles.dim() != 2 or rparticles.shape[0] != 6 or rparticles.stride(1) != 1:
        raise ValueError("rparticles must be [6, N] with contiguous rows")
    lib = N.lib()
    stream = C.c_void_p(torch.cuda.current_stream(rparticles.device).cuda_stream)
    with torch.cuda.device(rparticles.device):
        N.check(lib.sc_tmap_apply(R.ctypes.data_as(C.POINTER(C.c_double)), B.ctypes.data_as(C.POINTER(C.c_double)),
                                  C.c_void_p(rparticles.data_ptr()), rparticles.stride(0), rparticles.shape[1], stream))


class TransferMapDevice:
    """A first-order map (R, B) applied to device particle arrays."""

    def __init__(self, R, B=None):
        self.R = np.asarray(R, dtype=np.float64).reshape(6, 6)
        self.B = np.zeros(6) if B is None else np.asarray(B, dtype=np.float64).reshape(6)

    def apply(self, p_array):
        tmap_apply(self.R, self.B, p_array.rparticles)
