"""Failure paths of the complex branch and of the stored formulation, by
fault injection (GPU; no GPU fault, trap or hang).

An injected allocation failure inside these paths returns GBCC_OOM, and the
context stays usable: the same call then gives the bits of a fault-free
call.  This file is collected after the validated GPU tests on purpose, so
that a failure here cannot stop them in a run that stops at the first
failure.
"""
import numpy as np
import pytest

from sisi4s_gb300 import capi
from sisi4s_gb300 import ccsd as gpu
from tests.golden import cases

pytestmark = pytest.mark.gpu

KW = dict(max_iterations=4, energy_convergence=0.0, amplitudes_convergence=0.0)


@pytest.fixture
def clean(ctx):
    yield ctx
    ctx.inject_fault(capi.FAULT_NONE)  # an unconsumed fault must not leak


def _oom_then_recover(ctx, call):
    want = call()
    ctx.inject_fault(capi.FAULT_OOM)
    with pytest.raises(capi.GbccError) as e:
        call()
    assert e.value.status == capi.OOM
    return want, call()


def test_complex_solve_and_triples_recover_from_an_allocation_failure(clean):
    s, g = cases.complex_system(3, 7, 11, seed=4)
    solve = lambda: gpu.ccsd_solve_complex(clean, s.eps_h, s.eps_p, g, slice_size=3, **KW)
    want, got = _oom_then_recover(clean, solve)
    assert np.array_equal(got["history"], want["history"])
    trip = lambda: gpu.triples_complex(clean, s.eps_h, s.eps_p, g, want["T1"], want["T2"])[0]
    want_t, got_t = _oom_then_recover(clean, trip)
    assert got_t == want_t


def test_stored_formulation_recovers_from_an_allocation_failure(clean):
    s = cases.real_system()
    solve = lambda: gpu.ccsd_solve(clean, s.eps_h, s.eps_p, s.gamma, formulation="stored",
                                   mixer="DiisMixer", **KW)
    want, got = _oom_then_recover(clean, solve)
    assert np.array_equal(got["history"], want["history"])


def test_stored_formulation_reports_divergence(clean):
    s = cases.real_system()
    clean.inject_fault(capi.FAULT_NAN)
    with pytest.raises(capi.GbccError) as e:
        gpu.ccsd_solve(clean, s.eps_h, s.eps_p, s.gamma, formulation="stored", **KW)
    assert e.value.status == capi.DIVERGED
