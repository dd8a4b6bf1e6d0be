"""The checks every kick entry makes on its tensors before launching (host
logic, run here on CPU tensors): the kernels read n particles from
rparticles [6, >= n] and n charges from q_array, float64, on the kick's
device; anything else must raise before a launch, never read out of bounds."""
import pytest
import torch

from ocelot_gb300.sc import check_beam_tensors, cuda_device

CPU = torch.device("cpu")


def _t(n=100, nq=None, rows=6, dtype=torch.float64):
    return torch.zeros((rows, n), dtype=dtype), torch.zeros(n if nq is None else nq, dtype=dtype)


def test_matching_tensors_pass():
    rp, q = _t()
    check_beam_tensors(rp, q, 100, CPU)
    buf = torch.zeros((6, 101), dtype=torch.float64)
    check_beam_tensors(buf[:, :100], q, 100, CPU)     # a row stride other than n
    check_beam_tensors(rp, q, 50, CPU)                 # the first 50 particles


@pytest.mark.parametrize("nq", [99, 0])
def test_short_charge_vector_is_refused(nq):
    rp, q = _t(nq=nq)
    with pytest.raises(ValueError, match="q_array"):
        check_beam_tensors(rp, q, 100, CPU)


def test_wrong_shapes_dtypes_and_layouts_are_refused():
    rp, q = _t(rows=5)
    with pytest.raises(ValueError, match=r"shape \(6, N\)"):
        check_beam_tensors(rp, q, 100, CPU)
    rp, q = _t()
    with pytest.raises(ValueError, match=r"shape \(6, N\)"):
        check_beam_tensors(rp, q, 101, CPU)
    with pytest.raises(ValueError, match="rows must be contiguous"):
        check_beam_tensors(torch.zeros((100, 6), dtype=torch.float64).t(), q, 100, CPU)
    with pytest.raises(ValueError, match="q_array"):
        check_beam_tensors(rp, torch.zeros((100, 2), dtype=torch.float64)[:, 0], 100, CPU)
    rp32, q32 = _t(dtype=torch.float32)
    with pytest.raises(TypeError, match="float64"):
        check_beam_tensors(rp32, q, 100, CPU)
    with pytest.raises(TypeError, match="float64"):
        check_beam_tensors(rp, q32, 100, CPU)
    with pytest.raises(TypeError, match="torch tensors"):
        check_beam_tensors(rp.numpy(), q, 100, CPU)


def test_tensors_on_another_device_are_refused():
    rp, q = _t()
    with pytest.raises(ValueError, match="must be on"):
        check_beam_tensors(rp, q, 100, torch.device("cuda", 0))


def test_only_cuda_devices_are_accepted():
    with pytest.raises(ValueError, match="CUDA device"):
        cuda_device("cpu")
    assert cuda_device("cuda:1") == torch.device("cuda", 1)
