"""Emulated-FP64 GEMM on the bf16 tensor cores vs numpy FP64 (GPU)."""
import numpy as np
import pytest

from sisi4s_gb300 import capi

pytestmark = pytest.mark.gpu


def _dev(a):
    import torch  # device-memory plumbing only
    return torch.tensor(np.asarray(a, dtype=np.float64).T.copy().ravel(),
                        device="cuda")


def _run(ctx, ta, tb, A, B, C0, alpha, beta, slices):
    import torch
    M = A.shape[1] if ta else A.shape[0]
    K = A.shape[0] if ta else A.shape[1]
    N = B.shape[0] if tb else B.shape[1]
    dA, dB, dC = _dev(A), _dev(B), _dev(C0)
    torch.cuda.synchronize()
    ctx.set_emulation(slices, 0.0)
    ctx.check(ctx.lib.gbcc_dgemm(ctx.h, ta, tb, M, N, K, alpha, dA.data_ptr(),
                                 A.shape[0], dB.data_ptr(), B.shape[0], beta,
                                 dC.data_ptr(), M, capi.PREC_EMU))
    torch.cuda.synchronize()
    return dC.cpu().numpy().reshape(N, M).T


@pytest.mark.parametrize("slices", [4, 6, 8])
def test_exact_when_digits_suffice(ctx, slices):
    # integers below 2^18 with K <= 512: every digit product is kept and every
    # partial sum is exact, so the emulated result equals the exact product
    rng = np.random.default_rng(1)
    M, N, K = 130, 70, 300
    A = rng.integers(-(2 ** 17), 2 ** 17, size=(M, K)).astype(np.float64)
    B = rng.integers(-(2 ** 17), 2 ** 17, size=(K, N)).astype(np.float64)
    A[:, 0] = 2.0 ** 17  # fix the row scale
    B[0, :] = 2.0 ** 17
    exact = A @ B        # |C| < 2^53: exact in float64
    got = _run(ctx, 0, 0, A, B, np.zeros((M, N)), 1.0, 0.0, slices)
    if slices >= 6:
        assert np.array_equal(got, exact)
    else:
        assert np.abs(got - exact).max() <= 1e-6 * np.abs(exact).max()


@pytest.mark.parametrize("ta,tb,M,N,K", [(0, 0, 128, 64, 512), (1, 0, 300, 130, 1000),
                                         (0, 1, 77, 200, 3000), (1, 1, 129, 65, 33),
                                         (0, 0, 1, 1, 1), (0, 0, 256, 256, 5000)])
def test_random_accuracy(ctx, ta, tb, M, N, K):
    rng = np.random.default_rng(M * N + K)
    A = rng.normal(size=(K, M) if ta else (M, K))
    B = rng.normal(size=(N, K) if tb else (K, N))
    C0 = rng.normal(size=(M, N))
    ref = 0.5 * ((A.T if ta else A) @ (B.T if tb else B)) + 0.25 * C0
    got = _run(ctx, ta, tb, A, B, C0, 0.5, 0.25, 6)
    # error bound of the fixed-point split, relative to the row/column scales:
    # |err_ij| <~ K 2^-40 max|A_i.| max|B_.j|
    amax = np.abs(A.T if ta else A).max(axis=1)[:, None]
    bmax = np.abs(B.T if tb else B).max(axis=0)[None, :]
    bound = K * 2.0 ** -40 * amax * bmax + 1e-15 * np.abs(ref)
    assert np.all(np.abs(got - ref) <= bound)


def test_split_k_is_exact(ctx):
    # few output tiles and a long K: the product is split over K; the split
    # totals are exact integers, so an exactly representable product must
    # still come out exactly
    rng = np.random.default_rng(7)
    M, N, K = 40, 24, 20000
    A = rng.integers(-(2 ** 10), 2 ** 10, size=(M, K)).astype(np.float64)
    B = rng.integers(-(2 ** 10), 2 ** 10, size=(K, N)).astype(np.float64)
    A[:, 0] = 2.0 ** 10
    B[0, :] = 2.0 ** 10
    got = _run(ctx, 0, 0, A, B, np.zeros((M, N)), 1.0, 0.0, 6)
    assert np.array_equal(got, A @ B)


def test_very_long_k_accuracy(ctx):
    # 4096 exact chunks: the fixed-point width adapts so the int64 totals
    # cannot overflow
    rng = np.random.default_rng(8)
    M, N, K = 32, 32, 1 << 21
    A = rng.normal(size=(K, M))
    B = rng.normal(size=(K, N))
    ref = A.T @ B
    got = _run(ctx, 1, 0, A, B, np.zeros((M, N)), 1.0, 0.0, 6)
    bound = K * 2.0 ** -40 * np.abs(A).max(axis=0)[:, None] * np.abs(B).max(axis=0)[None, :]
    assert np.all(np.abs(got - ref) <= bound)


@pytest.mark.parametrize("alpha", [1.0, -2.0, 0.7])
def test_wide_totals_round_to_nearest(ctx, alpha):
    # 21-bit integers are exactly three 7-bit digits, so with 8 slices every
    # digit product is kept and the int64 totals are exact; the exact products
    # need more than 53 significant bits, so the conversion of the totals to
    # double must round to nearest (ties to even) like numpy's int64 -> float64
    rng = np.random.default_rng(11)
    M, N, K = 64, 48, 16384
    A = rng.integers(2 ** 19, 2 ** 20, size=(M, K))
    B = rng.integers(2 ** 19, 2 ** 20, size=(K, N))
    A[:, 0] = 2 ** 20
    B[0, :] = 2 ** 20
    exact = A @ B                      # int64, 2^52 < . < 2^55
    assert (exact > 2 ** 53).mean() > 0.5
    want = exact.astype(np.float64) * alpha
    got = _run(ctx, 0, 0, A.astype(np.float64), B.astype(np.float64),
               np.zeros((M, N)), alpha, 0.0, 8)
    assert np.array_equal(got, want)
