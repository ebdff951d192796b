"""sbz_cl_integrate_noalloc (static-scratch C_l integration on caller-owned device buffers)
against sbz_cl_integrate, through the C-ABI.

Collected last on purpose: it must give the same answer whether it runs alone in a fresh process
or after every other test has used the library on the same device."""
import ctypes as C
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-11  # the C_l integral tolerance of the parity tests


def _case(seed, nk, nl):
    rng = np.random.default_rng(seed)
    ks = np.sort(rng.uniform(1e-4, 5.0, nk))
    ks = np.unique(ks)
    P0 = rng.uniform(0.5, 2.0, len(ks)) * ks ** -3
    ThA = rng.standard_normal((len(ks), nl)) * 1e-3
    ThB = rng.standard_normal((len(ks), nl)) * 1e-3
    return ks, P0, ThA, ThB


def _reference(L, ks, P0, ThA, ThB):
    dp = lambda a: np.ascontiguousarray(a, dtype=np.float64).ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    nl = ThA.shape[1]
    out = np.zeros(nl)
    r = L.sbz_cl_integrate(len(ks), dp(ks), dp(P0), nl, dp(ThA), dp(ThB), dp(out))
    assert r == 0, L.sbz_last_error()
    return out


def _noalloc(L, torch, ks, P0, ThA, ThB):
    dev = [torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda") for a in (ks, P0, ThA, ThB)]
    nl = ThA.shape[1]
    out = torch.full((nl,), float("nan"), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    r = L.sbz_cl_integrate_noalloc(len(ks), *[C.c_void_p(t.data_ptr()) for t in dev[:2]], nl,
                                   *[C.c_void_p(t.data_ptr()) for t in dev[2:]], C.c_void_p(out.data_ptr()),
                                   C.c_void_p(stream.cuda_stream))
    assert r == 0, L.sbz_last_error()
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_allocating_entry_on_consecutive_calls():
    torch = pytest.importorskip("torch")
    from symboltz import _lib
    L = _lib.lib()
    # two calls in a row with different sizes and data: the second must not see the first's scratch
    # (larger first, then smaller), then a larger one again
    for seed, nk, nl in ((1, 700, 90), (2, 257, 33), (3, 1500, 120)):
        ks, P0, ThA, ThB = _case(seed, nk, nl)
        ref = _reference(L, ks, P0, ThA, ThB)
        got = _noalloc(L, torch, ks, P0, ThA, ThB)
        assert np.all(np.isfinite(got))
        np.testing.assert_allclose(got, ref, rtol=RTOL, atol=1e-12 * np.max(np.abs(ref)))


def test_noalloc_rejects_sizes_beyond_the_scratch():
    torch = pytest.importorskip("torch")
    from symboltz import _lib
    L = _lib.lib()
    cap = 2097152
    nk, nl = 4000, 600  # 2*4032 + 4001*600 doubles > cap
    assert 2 * ((nk + 1 + 31) // 32 * 32) + (nk + 1) * nl > cap
    buf = torch.zeros(8, dtype=torch.float64, device="cuda")
    p = C.c_void_p(buf.data_ptr())
    r = L.sbz_cl_integrate_noalloc(nk, p, p, nl, p, p, p, None)
    assert r == _lib.SBZ_ERR_ARG
    assert b"scratch" in L.sbz_last_error()
    # a size that just fits is accepted
    ks, P0, ThA, ThB = _case(4, 2000, 1040)
    assert 2 * ((len(ks) + 1 + 31) // 32 * 32) + (len(ks) + 1) * 1040 <= cap
    got = _noalloc(L, torch, ks, P0, ThA, ThB)
    np.testing.assert_allclose(got, _reference(L, ks, P0, ThA, ThB), rtol=RTOL, atol=1e-12 * np.max(np.abs(got)))


def test_noalloc_warm_calls_take_no_device_memory():
    """The entry's promise itself: once loaded, repeated calls leave the device's free memory
    unchanged (a cudaMalloc inside it, even one freed again before returning, would show up as a
    changed reading or as a synchronising allocation the caller's pool cannot see)."""
    torch = pytest.importorskip("torch")
    from symboltz import _lib
    L = _lib.lib()
    ks, P0, ThA, ThB = _case(5, 900, 64)
    dev = [torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda") for a in (ks, P0, ThA, ThB)]
    out = torch.zeros(64, dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream()
    args = (len(ks), *[C.c_void_p(t.data_ptr()) for t in dev[:2]], 64, *[C.c_void_p(t.data_ptr()) for t in dev[2:]],
            C.c_void_p(out.data_ptr()), C.c_void_p(stream.cuda_stream))
    assert L.sbz_cl_integrate_noalloc(*args) == 0, L.sbz_last_error()
    torch.cuda.synchronize()
    # objects of earlier tests still waiting for the garbage collector free their device buffers
    # when it runs; let it run now, so the readings below only see this entry
    gc.collect()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    for _ in range(20):
        assert L.sbz_cl_integrate_noalloc(*args) == 0, L.sbz_last_error()
        free_mid, _ = torch.cuda.mem_get_info()
        assert free_mid >= free0, (free_mid, free0)  # an allocation inside the call would lower it
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] >= free0
    assert torch.cuda.memory_reserved() == reserved0
    np.testing.assert_allclose(out.cpu().numpy(), _reference(L, ks, P0, ThA, ThB), rtol=RTOL,
                               atol=1e-12 * float(torch.max(torch.abs(out))))
