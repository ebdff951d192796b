"""The surrogate's BF16 tensor-core GEMM (tcgen05) through the C-ABI against a torch FP32
reference of the same op on the same bf16 inputs."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _gemm(L, M, N, K, A, B, epi, act=0, bias=None, out=None, n_valid=0, accumulate=0, z_out=None, z_in=None):
    p = lambda t: None if t is None else C.c_void_p(t.data_ptr())  # noqa: E731
    import torch
    r = L.sbz_mlp_gemm(M, N, K, p(A), p(B), epi, act, p(bias), p(out), out.shape[1], n_valid, accumulate, p(z_out), p(z_in),
                       C.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert r == 0, L.sbz_last_error()


@pytest.mark.parametrize("M,N,K", [(128, 64, 64), (256, 128, 128), (256, 256, 512), (384, 512, 192), (128, 192, 64)])
def test_gemm_f32_epilogue(M, N, K):
    torch = pytest.importorskip("torch")
    from symboltz import _lib
    L = _lib.lib()
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    out = torch.full((M, N), float("nan"), device="cuda")
    _gemm(L, M, N, K, A, B, 0, out=out)
    ref = A.float() @ B.float().T
    torch.testing.assert_close(out, ref, rtol=1e-4, atol=1e-4 * K ** 0.5)
    _gemm(L, M, N, K, A, B, 0, out=out, accumulate=1)  # accumulate: 2 D
    torch.testing.assert_close(out, 2 * ref, rtol=1e-4, atol=2e-4 * K ** 0.5)


def test_gemm_act_and_dact_epilogues():
    torch = pytest.importorskip("torch")
    from symboltz import _lib
    L = _lib.lib()
    M, N, K = 256, 512, 512
    g = torch.Generator(device="cuda").manual_seed(7)
    A = (0.1 * torch.randn(M, K, device="cuda", generator=g)).to(torch.bfloat16)
    B = (0.1 * torch.randn(N, K, device="cuda", generator=g)).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    y = torch.empty(M, N, device="cuda", dtype=torch.bfloat16)
    z = torch.empty(M, N, device="cuda", dtype=torch.bfloat16)
    _gemm(L, M, N, K, A, B, 1, act=1, bias=bias, out=y, z_out=z)
    zr = A.float() @ B.float().T + bias
    torch.testing.assert_close(z.float(), zr, rtol=1e-2, atol=1e-2)
    torch.testing.assert_close(y.float(), torch.nn.functional.silu(zr), rtol=1e-2, atol=1e-2)
    dy = torch.empty(M, N, device="cuda", dtype=torch.bfloat16)
    _gemm(L, M, N, K, A, B, 2, act=1, out=dy, z_in=z)
    zf = z.float()
    s = torch.sigmoid(zf)
    torch.testing.assert_close(dy.float(), (A.float() @ B.float().T) * s * (1 + zf * (1 - s)), rtol=2e-2, atol=2e-2)


def test_gemm_partial_columns_and_bad_sizes():
    torch = pytest.importorskip("torch")
    from symboltz import _lib
    L = _lib.lib()
    M, N, K = 128, 64, 512
    A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda").to(torch.bfloat16)
    out = torch.zeros(M, 4, device="cuda", dtype=torch.bfloat16)
    _gemm(L, M, N, K, A, B, 1, act=0, out=out, n_valid=4)  # ldo = 4: only the first 4 columns
    torch.testing.assert_close(out.float(), (A.float() @ B.float().T)[:, :4], rtol=1e-2, atol=1e-1)
    bad = L.sbz_mlp_gemm(100, N, K, C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()), 0, 0, None, C.c_void_p(out.data_ptr()), 4, 0, 0,
                         None, None, None)
    assert bad == _lib.SBZ_ERR_ARG
