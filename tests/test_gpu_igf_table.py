"""The FP32 form's Green's function table against an extended-precision IGF.

SpaceCharge.sym_kernel (ocelot/cpbd/sc.py:109-133) integrates 1/r over each
cell of the lag octant by the 8-corner difference of its antiderivative.  The
FP32 form keeps that difference, in FP64, only near the origin; beyond it the
cell integral is the 4th-order multipole form, and for cells long along z
(the relativistic case) the cells of the first z planes away from the z axis
take the line form (exact along z, Gauss-Legendre across), so that the FP64
work does not grow with the transverse mesh.  The table of the last call
(SC_REGION_IGF) is compared entry by entry with sym_kernel's formula in
np.longdouble, on meshes and steps from cells 500 times longer than wide to
cubic and flat ones.
"""
import numpy as np
import pytest

from conftest import has_gpu, igf_extended

pytestmark = pytest.mark.gpu

if not has_gpu():
    pytest.skip("needs a CUDA GPU", allow_module_level=True)

from ocelot_gb300 import SpaceCharge  # noqa: E402

CASES = [
    ((64, 64, 64), (8.7e-6, 8.7e-6, 4.5e-3)),  # the 2M / 64^3 130 MeV beam's rest-frame cells
    ((32, 32, 64), (1e-5, 1.2e-5, 5e-4)),      # long, unequal transverse steps
    ((48, 48, 48), (1e-5, 1e-5, 3e-5)),        # mildly long
    ((40, 40, 40), (1e-5, 1e-5, 1e-5)),        # cubic
    ((48, 48, 32), (2e-5, 2e-5, 5e-6)),        # flat: the multipole form beyond the near box
]


@pytest.mark.parametrize("shape,h", CASES, ids=["long500", "long50", "long3", "cubic", "flat"])
def test_hybrid_table_against_extended_precision(shape, h):
    sc = SpaceCharge(nmesh_xyz=list(shape), precision="fp32", igf="hybrid")
    sc.potential(np.zeros(shape), h)  # builds the table for these steps
    k = sc.engine(shape).region("igf").cpu().numpy().astype(np.float64)
    exact = igf_extended(shape, h).astype(np.float64)
    rel = np.abs(k - exact) / np.abs(exact)
    # each form within a few FP32 roundings: 8-corner FP64 differences near
    # the origin, the multipole form (5e-8) and the line form (2.6e-7 worst,
    # 7e-8 rms) beyond, then rounded to FP32
    assert rel.max() <= 4e-7, (shape, h, float(rel.max()), np.unravel_index(int(rel.argmax()), shape))
    assert np.sqrt(np.mean(rel ** 2)) <= 1.5e-7, (shape, h, float(np.sqrt(np.mean(rel ** 2))))
