"""The tcgen05 BF16 GEMM (tensor cores, FP32 accumulation in tensor memory) against torch in FP32."""
import ctypes as C

import pytest


@pytest.mark.gpu
@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (128, 32, 16), (300, 100, 70), (1000, 256, 256), (257, 128, 200),
                                   (300, 200, 64), (257, 48, 24), (4000, 256, 520), (129, 256, 1000)])
def test_tc_gemm_matches_torch(gpu, M, N, K):
    import torch
    from unomol_gb300 import native
    L = native.lib()
    L.unomol_tc_gemm_bf16.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    g = torch.Generator(device="cpu").manual_seed(M * 7 + N * 3 + K)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).to(gpu)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).to(gpu)
    Cm = torch.full((M, N), float("nan"), dtype=torch.float32, device=gpu)
    st = torch.zeros(1, dtype=torch.int32, device=gpu)
    assert L.unomol_tc_gemm_bf16(A.data_ptr(), B.data_ptr(), M, N, K, Cm.data_ptr(), st.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = A.float() @ B.float().T
    err = (Cm - ref).abs().max().item()
    assert err <= 1e-4 * ref.abs().max().item() + 1e-5, err
