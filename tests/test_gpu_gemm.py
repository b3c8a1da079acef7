"""The tcgen05 BF16 GEMM building block against torch (fp32 math on the
same bf16 inputs)."""
import ctypes

import numpy as np
import pytest

from create_rate_subs_gb300 import _lib

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


@pytest.mark.parametrize("M,N,K,bn", [(128, 64, 64, 64), (256, 128, 256, 128),
                                      (384, 192, 512, 192), (512, 256, 320, 256),
                                      (1024, 576, 1024, 192)])
def test_gemm_matches_torch(M, N, K, bn):
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn((M, K), device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn((N, K), device="cuda", generator=g).to(torch.bfloat16)
    D = torch.full((M, N), float("nan"), device="cuda", dtype=torch.float32)
    status = torch.zeros(2, dtype=torch.int32, device="cuda")
    lib = _lib.load()
    rc = lib.crs_gemm_bf16(_p(A), _p(B), _p(D), M, N, K, N, bn, _p(status),
                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    assert int(status[0]) == 0
    ref = A.double() @ B.double().T
    err = (D.double() - ref).abs().max().item()
    scale = (A.double().abs() @ B.double().abs().T).max().item()
    assert err <= 1e-5 * scale, (err, scale)


def test_gemm_exact_small_integers():
    """Integer-valued operands (the stoichiometric matrix case) are exact."""
    M, N, K = 256, 64, 128
    g = torch.Generator(device="cuda").manual_seed(7)
    A = torch.randint(-3, 4, (M, K), device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randint(-2, 3, (N, K), device="cuda", generator=g).to(torch.bfloat16)
    D = torch.empty((M, N), device="cuda", dtype=torch.float32)
    lib = _lib.load()
    assert lib.crs_gemm_bf16(_p(A), _p(B), _p(D), M, N, K, N, 64, None, None) == 0
    torch.cuda.synchronize()
    assert torch.equal(D, (A.float() @ B.float().T))


def test_gemm_argument_checks():
    lib = _lib.load()
    A = torch.zeros((128, 64), device="cuda", dtype=torch.bfloat16)
    D = torch.zeros((128, 64), device="cuda", dtype=torch.float32)
    assert lib.crs_gemm_bf16(_p(A), _p(A), _p(D), 100, 64, 64, 64, 64, None, None) == 1
    assert lib.crs_gemm_bf16(_p(A), _p(A), _p(D), 128, 64, 60, 64, 64, None, None) == 1
    assert lib.crs_gemm_bf16(_p(A), _p(A), _p(D), 128, 64, 64, 64, 96, None, None) == 1
