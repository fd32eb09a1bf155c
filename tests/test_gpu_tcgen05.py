"""The fifth-generation tensor-core path (tcgen05.mma with TMEM accumulators,
diffrax_gb300/csrc/gbdx_tc.cuh) on the GPU: a BF16 128 x 128 x 64 product
against torch's FP32 product of the same BF16-rounded operands."""
import pytest
import torch

from diffrax_gb300 import _lib

pytestmark = pytest.mark.gpu


def test_tcgen05_product_matches_torch():
    lib = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(0)
    A = torch.randn(128, 64, device="cuda", generator=g)
    B = torch.randn(128, 64, device="cuda", generator=g)
    D = torch.full((128, 128), float("nan"), device="cuda")
    status = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    rc = lib.gbdx_selftest_tcgen05(A.data_ptr(), B.data_ptr(), D.data_ptr(), status.data_ptr(),
                                   torch.cuda.current_stream().cuda_stream)
    _lib.check(rc, "gbdx_selftest_tcgen05")
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    want = A.bfloat16().float() @ B.bfloat16().float().T
    # FP32 accumulation of exact BF16 products: only the summation order differs
    assert torch.allclose(D, want, rtol=1e-5, atol=1e-4), (D - want).abs().max()
