"""The tcgen05 BF16 GEMM (C = A B^T, FP32 accumulation) against a plain
PyTorch FP32 product of the same BF16 values, for every tile width and
epilogue."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(M, N, K, epi, seed=0):
    import torch
    from channel_flow_gb300 import _lib
    lib = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(seed)
    A = torch.randn(M, K, generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn(N, K, generator=g, device="cuda").to(torch.bfloat16)
    bias = torch.randn(N, generator=g, device="cuda")
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    ref = A.float() @ B.float().t()
    if epi == 0:
        out = torch.full((M, N), float("nan"), device="cuda")
        z = None
    elif epi == 1:
        out = torch.zeros(M, N, dtype=torch.bfloat16, device="cuda")
        z = torch.zeros(M, N, device="cuda")
    else:
        out = torch.zeros(M, N, device="cuda")
        z = None
    s = torch.cuda.current_stream().cuda_stream
    rc = lib.cf_gemm_bf16(s, A.data_ptr(), B.data_ptr(), M, N, K, epi, bias.data_ptr() if epi else None,
                          out.data_ptr(), z.data_ptr() if z is not None else None, N, err.data_ptr())
    torch.cuda.synchronize()
    assert rc == 0
    assert int(err.item()) == 0
    return ref, bias, out, z


@pytest.mark.parametrize("M,N,K", [(128, 16, 64), (256, 128, 320), (384, 320, 128), (128, 256, 512),
                                   (256, 32, 64), (128, 64, 4096)])
def test_gemm_fp32_out(M, N, K, cuda_lib):
    import torch
    ref, _, out, _ = _run(M, N, K, 0)
    rel = float((out - ref).abs().max() / ref.abs().max())
    assert rel <= 1e-5, rel


@pytest.mark.parametrize("M,N,K", [(256, 128, 320), (128, 16, 128)])
def test_gemm_bias_silu_bf16(M, N, K, cuda_lib):
    import torch
    ref, bias, out, z = _run(M, N, K, 1, seed=1)
    zr = ref + bias
    assert float((z - zr).abs().max() / zr.abs().max()) <= 1e-5
    yr = torch.nn.functional.silu(zr)
    assert float((out.float() - yr).abs().max() / yr.abs().max()) <= 1e-2


def test_gemm_bias_f32(cuda_lib):
    import torch
    ref, bias, out, _ = _run(256, 16, 128, 2, seed=2)
    zr = ref + bias
    assert float((out - zr).abs().max() / zr.abs().max()) <= 1e-5


@pytest.mark.parametrize("M,N,K,splits", [(128, 320, 131072, 60), (128, 128, 65536, 300), (128, 16, 8192, 128),
                                          (256, 64, 4096, 7), (128, 320, 640, 10), (128, 64, 512, 1)])
def test_gemm_splitk_fp32_out(M, N, K, splits, cuda_lib):
    """The weight-gradient form: K split over `splits` CTAs per tile (uneven
    slab counts included), partials summed in split order, against the
    FP32 product of the same BF16 values."""
    import torch
    from channel_flow_gb300 import _lib
    lib = _lib.load()
    g = torch.Generator(device="cuda").manual_seed(3)
    A = torch.randn(M, K, generator=g, device="cuda").to(torch.bfloat16)
    B = torch.randn(N, K, generator=g, device="cuda").to(torch.bfloat16)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    partial = torch.full((splits * M * N,), float("nan"), device="cuda")
    out = torch.full((M, N), float("nan"), device="cuda")
    rc = lib.cf_gemm_bf16_splitk(torch.cuda.current_stream().cuda_stream, A.data_ptr(), B.data_ptr(), M, N, K,
                                 splits, partial.data_ptr(), out.data_ptr(), err.data_ptr())
    torch.cuda.synchronize()
    assert rc == 0 and int(err.item()) == 0
    ref = A.float() @ B.float().t()
    rel = float((out - ref).abs().max() / ref.abs().max())
    assert rel <= 1e-5, rel
    # more splits than K-slabs is refused before any launch
    assert lib.cf_gemm_bf16_splitk(None, A.data_ptr(), B.data_ptr(), M, N, K, K // 64 + 1, partial.data_ptr(),
                                   out.data_ptr(), err.data_ptr()) == _lib.CF_ERR_ARG
