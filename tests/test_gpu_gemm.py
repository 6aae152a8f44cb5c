"""The tensor-core GEMM (tcgen05, BF16 in, FP32 accumulate) against a
PyTorch fp32 matmul of the same bf16 operands."""
import ctypes

import numpy as np
import pytest

from rtac_simulation_gb300 import _lib

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
if not torch.cuda.is_available():
    pytest.skip("needs a GPU", allow_module_level=True)


# 128 x 256 tiles (N a multiple of 256) and 128 x 128 tiles, two CTAs per SM
# (N = 384: a multiple of 128 only).
@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (256, 512, 192), (384, 256, 1024), (256, 384, 128),
                                   (4096, 1024, 3072), (8192, 2048, 256)])
def test_gemm_bf16_matches_fp32_reference(M, N, K):
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.full((M, N), float("nan"), device="cuda")
    lib = _lib.load()
    st = lib.rtacx_gemm_bf16_tn(A.data_ptr(), B.data_ptr(), C.data_ptr(), M, N, K,
                                torch.cuda.current_stream().cuda_stream)
    assert st == _lib.RTACX_OK
    ref = A.float() @ B.float().T
    err = (C - ref).norm() / ref.norm()
    assert torch.isfinite(C).all()
    assert err.item() < 1e-5, err.item()


def test_gemm_rejects_bad_shapes():
    lib = _lib.load()
    A = torch.zeros(128, 64, dtype=torch.bfloat16, device="cuda")
    C = torch.zeros(128, 256, device="cuda")
    assert lib.rtacx_gemm_bf16_tn(A.data_ptr(), A.data_ptr(), C.data_ptr(), 100, 256, 64, None) == \
        _lib.RTACX_ERR_INVALID_ARGUMENT
