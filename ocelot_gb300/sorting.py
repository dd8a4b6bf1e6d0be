"""Stable radix sort of NGP cell keys on the GPU (the deposit's order).

``stable_sort_keys`` exposes the sort that orders the charge deposit
(sc_sort_keys in include/ocelot_sc.h): equal to
``numpy.argsort(keys, kind='stable')`` bit for bit.
"""
from __future__ import annotations

import ctypes as C

from . import _native as N


def stable_sort_keys(keys, key_bits: int):
    """Sort a CUDA uint32 (or int32) tensor of keys; returns (sorted_keys, perm) as int64 tensors."""
    import torch
    if keys.dtype not in (torch.int32, torch.uint32):
        raise TypeError("keys must be a 32-bit integer tensor")
    lib = N.lib()
    n = int(keys.numel())
    keys = keys.contiguous()
    out_k = torch.empty(n, dtype=torch.int32, device=keys.device)
    out_p = torch.empty(n, dtype=torch.int32, device=keys.device)
    nbytes = int(lib.sc_sort_workspace_bytes(n, int(key_bits)))
    if nbytes < 0:
        raise ValueError("bad sort size")
    ws = torch.empty(max(nbytes, 1), dtype=torch.uint8, device=keys.device)
    stream = C.c_void_p(torch.cuda.current_stream(keys.device).cuda_stream)
    with torch.cuda.device(keys.device):
        N.check(lib.sc_sort_keys(C.c_void_p(keys.data_ptr()), n, int(key_bits), C.c_void_p(out_k.data_ptr()),
                                 C.c_void_p(out_p.data_ptr()), C.c_void_p(ws.data_ptr()), nbytes, stream))
    return out_k.to(torch.int64) & 0xFFFFFFFF, out_p.to(torch.int64) & 0xFFFFFFFF
