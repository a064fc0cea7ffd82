"""The tcgen05 BF16 contraction with fused per-tile argmax against an FP32 matmul of
the same BF16 operands (ragged M and N exercise the TMA zero fill)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K", [(128, 256, 64), (300, 1000, 448), (1000, 3000, 1280)])
def test_gemm_argmax_matches_fp32_matmul(built, M, N, K):
    import torch
    from cryoim_gb300._abi import call
    torch.manual_seed(M + N + K)
    dev = torch.device("cuda", 0)
    a = torch.randn(M, K, device=dev).to(torch.bfloat16)
    b = torch.randn(N, K, device=dev).to(torch.bfloat16)
    nt = (N + 255) // 256
    topv = torch.empty(M, nt, device=dev)
    topi = torch.empty(M, nt, dtype=torch.int32, device=dev)
    cfull = torch.zeros(M, N, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    s = torch.cuda.current_stream().cuda_stream
    call("cryoim_gemm_bf16_argmax", C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), M, N, K,
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
