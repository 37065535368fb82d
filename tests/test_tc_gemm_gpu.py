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


@pytest.mark.gpu
def test_tc_gemm_bounded_wait_gives_up_and_recovers(gpu):
    """Failure detection without a GPU fault: with the pipeline waits told to give up at once
    (unomol_tc_set_wait_polls(-1)), the GEMM drains the copies it issued, releases its tensor memory
    and reports the timeout in its status word; the network's calls return UNOMOL_ETIMEOUT.  With the
    default limit restored the same calls give the results of a clean run: the context stays usable
    and no tensor memory was leaked (a leak would leave the next allocation unable to proceed)."""
    import torch
    from unomol_gb300 import native
    L = native.lib()
    L.unomol_tc_gemm_bf16.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
    M, N, K = 1000, 256, 520
    g = torch.Generator(device="cpu").manual_seed(11)
    A = torch.randn(M, K, generator=g).to(torch.bfloat16).to(gpu)
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).to(gpu)
    Cm = torch.zeros((M, N), dtype=torch.float32, device=gpu)
    st = torch.zeros(1, dtype=torch.int32, device=gpu)
    ref = A.float() @ B.float().T
    assert L.unomol_tc_set_wait_polls(-1) == 0
    try:
        assert L.unomol_tc_gemm_bf16(A.data_ptr(), B.data_ptr(), M, N, K, Cm.data_ptr(), st.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert int(st.item()) == 1  # the wait gave up and said so
    finally:
        L.unomol_tc_set_wait_polls(0)
    st.zero_()
    for _ in range(2):
        Cm.fill_(float("nan"))
        assert L.unomol_tc_gemm_bf16(A.data_ptr(), B.data_ptr(), M, N, K, Cm.data_ptr(), st.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert int(st.item()) == 0
        assert (Cm - ref).abs().max().item() <= 1e-4 * ref.abs().max().item() + 1e-5

    # through the network: forward returns UNOMOL_ETIMEOUT, then the same output as before
    L.unomol_mlp_create.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_ulonglong, C.POINTER(C.c_void_p)]
    L.unomol_mlp_forward.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
    L.unomol_mlp_destroy.argtypes = [C.c_void_p]
    L.unomol_mlp_destroy.restype = None
    h = C.c_void_p()
    assert L.unomol_mlp_create(24, 256, 3, 48, 5, C.byref(h)) == 0
    try:
        x = torch.randn(700, 24, generator=g).to(gpu)
        y0 = torch.zeros(700, 48, device=gpu)
        y1 = torch.full((700, 48), float("nan"), device=gpu)
        assert L.unomol_mlp_forward(h, x.data_ptr(), 700, y0.data_ptr(), None) == 0
        L.unomol_tc_set_wait_polls(-1)
        try:
            assert L.unomol_mlp_forward(h, x.data_ptr(), 700, y1.data_ptr(), None) == -5  # UNOMOL_ETIMEOUT
        finally:
            L.unomol_tc_set_wait_polls(0)
        assert L.unomol_mlp_forward(h, x.data_ptr(), 700, y1.data_ptr(), None) == 0
        torch.cuda.synchronize()
        assert torch.equal(y0, y1)
    finally:
        L.unomol_mlp_destroy(h)
