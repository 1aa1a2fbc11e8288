"""Failure paths on the GPU, by fault injection (no GPU fault, trap or hang).

Each injected fault makes one event fail as if it had happened; the call
returns its status code and the context stays usable, as the next correct
call shows.  The device-side case is a bounded wait on a barrier that nothing
completes inside the tensor-core GEMM.
"""
import time

import numpy as np
import pytest

from sisi4s_gb300 import capi
from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu


@pytest.fixture
def clean(ctx):
    yield ctx
    ctx.inject_fault(capi.FAULT_NONE)  # an unconsumed fault must not leak
    ctx.set_emulation(6, 1e7)


def _emu_gemm(ctx, A, B):
    import torch  # device memory plumbing only
    M, K = A.shape
    N = B.shape[1]
    dA = torch.tensor(A.T.copy().ravel(), device="cuda")
    dB = torch.tensor(B.T.copy().ravel(), device="cuda")
    dC = torch.zeros(M * N, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    st = ctx.lib.gbcc_dgemm(ctx.h, 0, 0, M, N, K, 1.0, dA.data_ptr(), M, dB.data_ptr(), K,
                            0.0, dC.data_ptr(), M, capi.PREC_EMU)
    torch.cuda.synchronize()
    return st, dC.cpu().numpy().reshape(N, M).T


def test_device_wait_gives_up_and_context_survives(clean):
    ctx = clean
    rng = np.random.default_rng(3)
    A, B = rng.normal(size=(700, 300)), rng.normal(size=(300, 500))
    ctx.set_emulation(6, 0.0)
    ctx.inject_fault(capi.FAULT_DEVICE_WAIT)
    t0 = time.perf_counter()
    st, _ = _emu_gemm(ctx, A, B)
    assert st == capi.TIMEOUT
    assert time.perf_counter() - t0 < 30.0  # bounded: the kernel gave up and returned
    st, got = _emu_gemm(ctx, A, B)           # same context, no fault
    assert st == capi.OK
    ref = A @ B
    assert np.abs(got - ref).max() < 1e-11 * np.abs(ref).max()


def test_allocation_failure_is_oom_then_recovers(clean):
    ctx = clean
    s = make_system(3, 10, 20, seed=2)
    ctx.inject_fault(capi.FAULT_OOM)
    with pytest.raises(capi.GbccError) as e:
        gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, max_iterations=3)
    assert e.value.status == capi.OOM
    r = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, max_iterations=3)
    assert np.isfinite(r["energy"]) and r["iterations"] == 3


def test_nan_norm_is_diverged(clean):
    ctx = clean
    s = make_system(3, 10, 20, seed=3)
    ctx.inject_fault(capi.FAULT_NAN)
    with pytest.raises(capi.GbccError) as e:
        gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, max_iterations=4)
    assert e.value.status == capi.DIVERGED


def test_singular_diis_is_reported(clean):
    ctx = clean
    s = make_system(3, 10, 20, seed=4)
    ctx.inject_fault(capi.FAULT_DIIS_SINGULAR)
    with pytest.raises(capi.GbccError) as e:
        gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, mixer="DiisMixer", max_iterations=4)
    assert e.value.status == capi.DIIS_SINGULAR
    # the same solve without the fault runs all its iterations
    r = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, mixer="DiisMixer", max_iterations=4)
    assert r["iterations"] == 4


def test_unknown_fault_kind_is_rejected(clean):
    assert clean.lib.gbcc_ctx_inject_fault(clean.h, 99) == capi.BAD_ARG
