"""The tensor-core (tcgen05) building block of the network kernels on one
tile: BF16 operands staged as K-major core matrices in shared memory, the
FP32 accumulator in tensor memory, read back with tcgen05.ld.  Checked
against an FP32 matrix product of the same BF16 values (the products are
exact in FP32; only the summation order differs)."""
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N", [16, 48, 64, 128])
@pytest.mark.parametrize("K", [16, 64, 256])
def test_umma_tile_matches_matmul(cuda, N, K):
    from serac_gb300 import _lib

    g = torch.Generator(device="cpu").manual_seed(N * 1000 + K)
    A = torch.randn(128, K, generator=g).to(torch.bfloat16).to(cuda)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).to(cuda)
    D = torch.full((128, N), float("nan"), dtype=torch.float32, device=cuda)
    _lib.call("sfx_selftest_umma_tile", A.data_ptr(), B.data_ptr(), N, K, D.data_ptr())
    ref = A.float() @ B.float().T
    assert torch.isfinite(D).all()
    assert (D - ref).abs().max().item() <= 1e-5 * ref.abs().max().item()
