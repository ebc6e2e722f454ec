"""Numerics of the contraction kernels of the mixed path against a PyTorch
reference of the same op (complex128 matmul of the same complex64 inputs).
Tolerance: relative Frobenius error <= 3e-6, FP32 level: about sqrt(K) 6e-8 for
the CUDA-core kernel and for the tensor-core kernels (3xTF32 split; the mma.sync
kernel accumulates every k8 step separately and adds it in FP32, the tcgen05
kernel reads every 16-deep K stage out of tensor memory and adds it in FP32)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("tc", [2, 1, 0])
@pytest.mark.parametrize("M,N,K", [(64, 64, 64), (100, 37, 129), (7, 200, 33), (256, 256, 512), (128, 64, 16),
                                   (300, 130, 1000), (129, 65, 17)])
def test_gemm_c64_matches_torch(tc, M, N, K):
    torch = pytest.importorskip("torch")
    from qca_gb300 import _lib
    g = torch.Generator(device="cuda").manual_seed(M * 1000 + N + K)
    A = torch.randn(M, K, dtype=torch.complex64, device="cuda", generator=g)
    B = torch.randn(K, N, dtype=torch.complex64, device="cuda", generator=g)
    C = torch.zeros(M, N, dtype=torch.complex64, device="cuda")
    torch.cuda.synchronize()
    _lib.call("qca_test_gemm_c64", M, N, K, ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
              ctypes.c_void_p(C.data_ptr()), tc, None)
    ref = A.to(torch.complex128) @ B.to(torch.complex128)
    err = (C.to(torch.complex128) - ref).norm() / ref.norm()
    assert err.item() < 3e-6, err.item()
