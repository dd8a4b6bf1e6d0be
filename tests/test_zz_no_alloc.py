"""The Green's-function table without any device allocation.

sc_sym_kernel_static serves callers that cannot allocate device memory where
they need the table: a process whose device memory is reserved up front by
another allocator or a fixed budget, or a latency-critical loop that must not
call cudaMalloc/cudaFree.  Its scratch is a static device array inside the
library.  Here it is called through the C ABI twice in a row (two meshes, the
second reusing the array the first one filled) and each result is compared
with sc_sym_kernel, the entry point that takes a caller-allocated workspace
(both run the same kernels, so the tables must be identical), and with the
oracle's table (the reference's sym_kernel, sc.py:109-133): against an
extended-precision evaluation of the same formula, the static table's error
is at most twice the oracle's own, the bound the workspace entry point meets
on the reference's fixtures.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import has_gpu, igf_extended
from oracle import sc_oracle

pytestmark = pytest.mark.gpu

if not has_gpu():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

import torch  # noqa: E402

from ocelot_gb300 import SpaceCharge, _native  # noqa: E402

CASES = [((63, 63, 63), (6.97e-06, 7.05e-06, 4.15e-03)),  # 64^3 corners: the default mesh
         ((20, 31, 40), (1.0e-03, 2.0e-03, 5.0e-04))]


def _static_table(lib, shape, h, stream):
    out = torch.empty(shape, dtype=torch.float64, device="cuda")
    rc = lib.sc_sym_kernel_static(*shape, *h, C.c_void_p(out.data_ptr()), stream)
    assert rc == _native.SC_OK, _native.last_error()
    return out


def test_static_table_matches_workspace_table_two_calls_in_a_row():
    torch.cuda.set_device(0)
    lib = _native.lib()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    outs = [_static_table(lib, shape, h, stream) for shape, h in CASES]
    torch.cuda.synchronize()
    for (shape, h), out in zip(CASES, outs):
        got = out.cpu().numpy()
        ref = SpaceCharge(nmesh_xyz=list(shape)).sym_kernel(shape, h)
        assert np.array_equal(got, ref), shape
        exact = igf_extended(shape, h)
        oracle = sc_oracle.igf_kernel(shape, h)
        e_oracle = float(np.linalg.norm(oracle.astype(np.longdouble) - exact) / np.linalg.norm(exact))
        e_static = float(np.linalg.norm(got.astype(np.longdouble) - exact) / np.linalg.norm(exact))
        assert e_static <= 2 * e_oracle + 1e-14, (shape, e_static, e_oracle)


def test_static_table_rejects_a_mesh_beyond_its_limit():
    lib = _native.lib()
    out = torch.empty(1, dtype=torch.float64, device="cuda")
    rc = lib.sc_sym_kernel_static(128, 128, 128, 1e-5, 1e-5, 1e-5, C.c_void_p(out.data_ptr()), None)
    assert rc == _native.SC_ERR_UNSUPPORTED
    assert "exceeds the static table" in _native.last_error()
