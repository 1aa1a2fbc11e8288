"""The emulated GEMM entry point that allocates nothing (GPU).

gbcc_dgemm_emu_noalloc serves callers that cannot let the library allocate
device memory (their own arena already holds the HBM budget, or their hot
loop must stay out of the CUDA allocator, whose latency they do not
control).  It must give the same result as
the allocating emulated GEMM (gbcc_dgemm with GBCC_PREC_EMU), also on a second
call right after the first, when the shared scratch array still holds the
first call's data.  This file is collected last on purpose, so that a failure
here cannot stop the other tests of a run that stops at the first failure.
"""
import numpy as np
import pytest

from sisi4s_gb300 import capi

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch  # device-memory plumbing of the test only
    return torch.tensor(np.asarray(a, dtype=np.float64).T.copy().ravel(),
                        device="cuda")


def _gemm(ctx, fn, ta, tb, A, B, C0, alpha, beta):
    import torch
    M = A.shape[1] if ta else A.shape[0]
    K = A.shape[0] if ta else A.shape[1]
    N = B.shape[0] if tb else B.shape[1]
    dA, dB, dC = _dev(A), _dev(B), _dev(C0)
    torch.cuda.synchronize()
    args = [ctx.h, ta, tb, M, N, K, alpha, dA.data_ptr(), A.shape[0],
            dB.data_ptr(), B.shape[0], beta, dC.data_ptr(), M]
    if fn == "alloc":
        st = ctx.lib.gbcc_dgemm(*args, capi.PREC_EMU)
    else:
        st = ctx.lib.gbcc_dgemm_emu_noalloc(*args)
    torch.cuda.synchronize()
    return st, dC.cpu().numpy().reshape(N, M).T


def test_noalloc_matches_allocating_emulated_gemm(ctx):
    ctx.set_emulation(6, 0.0)
    rng = np.random.default_rng(42)
    # two calls in a row: the second is smaller, so stale panels of the first
    # call remain in the shared array around the region the second one uses
    for (ta, tb, M, N, K) in [(0, 1, 300, 200, 900), (1, 0, 70, 33, 130)]:
        A = rng.normal(size=(K, M) if ta else (M, K))
        B = rng.normal(size=(N, K) if tb else (K, N))
        C0 = rng.normal(size=(M, N))
        st_a, ref = _gemm(ctx, "alloc", ta, tb, A, B, C0, 0.5, -0.25)
        st_n, got = _gemm(ctx, "noalloc", ta, tb, A, B, C0, 0.5, -0.25)
        assert st_a == capi.OK and st_n == capi.OK
        # same kernels and the same arithmetic: identical results
        assert np.array_equal(got, ref)
        exact = 0.5 * ((A.T if ta else A) @ (B.T if tb else B)) - 0.25 * C0
        assert np.abs(got - exact).max() < 1e-10 * np.abs(exact).max()


def test_noalloc_rejects_oversized_gemm(ctx):
    ctx.set_emulation(6, 0.0)
    import torch
    M = N = 4096
    K = 4096
    # full-size operands, so that nothing could read out of bounds even if the
    # size check were missing
    a = torch.zeros(M * K, dtype=torch.float64, device="cuda")
    b = torch.zeros(K * N, dtype=torch.float64, device="cuda")
    c = torch.zeros(M * N, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = ctx.lib.gbcc_dgemm_emu_noalloc(ctx.h, 0, 0, M, N, K, 1.0, a.data_ptr(),
                                        M, b.data_ptr(), K, 0.0, c.data_ptr(), M)
    assert st == capi.BAD_ARG
    assert b"scratch" in ctx.lib.gbcc_last_error(ctx.h)
