"""The tcgen05 BF16 GEMM primitive (tensor memory accumulators, shared-memory descriptors,
mbarrier-tracked MMAs) against an FP32 matmul of the same BF16 inputs."""
import ctypes

import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form", [0, 1, 2])
@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 64, 192), (384, 128, 576),
                                   (128, 32, 64), (200, 256, 128), (1000, 128, 1152),
                                   (128, 32, 72), (256, 64, 200), (512, 32, 8), (640, 128, 4096)])
def test_tc_gemm_bf16(native, M, N, K, form):
    L = native.lib()
    g = torch.Generator(device="cuda").manual_seed(M * 7 + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    C = torch.full((M, N), float("nan"), device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = L.lentils_tc_gemm_bf16(ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
                                ctypes.c_void_p(C.data_ptr()), M, N, K, form,
                                ctypes.c_void_p(err.data_ptr()), None)
    torch.cuda.synchronize()
    assert st == 0 and int(err.item()) == 0
    ref = A.double() @ B.double().T
    rel = float(((C.double() - ref).abs().max() / ref.abs().max()).item())
    assert rel < 5e-6


def test_bounded_wait_times_out_and_context_survives(native):
    """A wait that nothing completes gives up after its poll limit: the kernel returns, sets
    the error flag and frees its tensor memory; the next tensor-core GEMM runs normally."""
    L = native.lib()
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    assert L.lentils_tc_timeout_selftest(ctypes.c_void_p(err.data_ptr()), 1000, None) == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 1
    for form in (0, 1, 2):
        test_tc_gemm_bf16(native, 128, 64, 64, form)
