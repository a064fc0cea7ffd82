"""The tcgen05 contraction with fused per-tile argmax (BF16 x BF16 and FP8-e4m3 x
FP8-e4m3, FP32 accumulation) against an FP32 matmul of the same operands (ragged M and
N exercise the TMA zero fill)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("kind,M,N,K", [("bf16", 128, 256, 64), ("bf16", 300, 1000, 448),
                                        ("bf16", 1000, 3000, 1280), ("e4m3", 128, 256, 128),
                                        ("e4m3", 300, 1000, 512), ("e4m3", 1000, 3000, 1280)])
def test_gemm_argmax_matches_fp32_matmul(built, kind, M, N, K):
    import torch
    from cryoim_gb300._abi import call
    torch.manual_seed(M + N + K)
    dev = torch.device("cuda", 0)
    dt = torch.bfloat16 if kind == "bf16" else torch.float8_e4m3fn
    a = torch.randn(M, K, device=dev).to(dt)
    b = torch.randn(N, K, device=dev).to(dt)
    nt = (N + 255) // 256
    topv = torch.empty(M, nt, device=dev)
    topi = torch.empty(M, nt, dtype=torch.int32, device=dev)
    cfull = torch.zeros(M, N, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream().cuda_stream
    call(f"cryoim_gemm_{kind}_argmax", C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), M, N, K,
         C.c_void_p(topv.data_ptr()), C.c_void_p(topi.data_ptr()), C.c_void_p(cfull.data_ptr()),
         C.c_void_p(err.data_ptr()), C.c_void_p(s))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    ref = a.float() @ b.float().T
    scale = float(ref.abs().max())
    assert float((cfull - ref).abs().max()) < 1e-5 * scale * np.sqrt(K / 64)
    # per-tile max and a column that attains it
    pad = torch.full((M, nt * 256 - N), -3e38, device=dev)
    tiles = torch.cat([ref, pad], 1).view(M, nt, 256)
    want = tiles.max(-1).values
    assert float((topv - want).abs().max()) < 1e-5 * scale * np.sqrt(K / 64)
    got_at = torch.gather(ref, 1, topi.long())
    assert float((got_at - want).abs().max()) < 1e-5 * scale * np.sqrt(K / 64)
    assert bool(((topi // 256) == torch.arange(nt, device=dev)[None, :]).all())


def test_pipeline_wait_that_runs_out_reports_and_frees(built):
    """The failure path of the tcgen05 pipeline: CTA 0's producer leaves one k-stage of
    its first tile unloaded (nothing ever completes that barrier), every wait is limited
    to 10 ms.  The launch returns with the error flag set and no CUDA error; the next
    launches on the same context (TMEM released, barriers re-initialised) give the normal
    result, twice."""
    import time
    import torch
    from cryoim_gb300._abi import call
    torch.manual_seed(5)
    dev = torch.device("cuda", 0)
    M, N, K = 600, 2000, 640
    a = torch.randn(M, K, device=dev).to(torch.bfloat16)
    b = torch.randn(N, K, device=dev).to(torch.bfloat16)
    nt = (N + 255) // 256
    s = torch.cuda.current_stream().cuda_stream

    def normal():
        topv = torch.empty(M, nt, device=dev)
        topi = torch.empty(M, nt, dtype=torch.int32, device=dev)
        err = torch.zeros(1, dtype=torch.int32, device=dev)
        call("cryoim_gemm_bf16_argmax", C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), M, N, K,
             C.c_void_p(topv.data_ptr()), C.c_void_p(topi.data_ptr()), None, C.c_void_p(err.data_ptr()),
             C.c_void_p(s))
        torch.cuda.synchronize()
        return int(err.item()), topv.cpu(), topi.cpu()

    e0, v0, i0 = normal()
    assert e0 == 0
    topv = torch.empty(M, nt, device=dev)
    topi = torch.empty(M, nt, dtype=torch.int32, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    t0 = time.perf_counter()
    call("cryoim_gemm_bf16_argmax_withhold", C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), M, N, K,
         C.c_void_p(topv.data_ptr()), C.c_void_p(topi.data_ptr()), C.c_void_p(err.data_ptr()), 3, 10000,
         C.c_void_p(s))
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    assert int(err.item()) == 1
    assert dt < 5.0, dt
    for _ in range(2):
        e1, v1, i1 = normal()
        assert e1 == 0
        assert torch.equal(v1, v0) and torch.equal(i1, i0)
