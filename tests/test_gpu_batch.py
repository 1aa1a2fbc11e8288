"""Lockstep solve of several systems of one shape (gbcc_ccsd_solve_batch):
each contraction runs once for all systems, as one batched product, and every
system ends where its own solve ends."""
import numpy as np
import pytest

from sisi4s_gb300 import capi
from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu

OPTS = dict(mixer="DiisMixer", max_residua=5, max_iterations=40,
            energy_convergence=1e-10, amplitudes_convergence=1e-7)


def _alone(ctx, s, **opts):
    return gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, want_amplitudes=True, **opts)


# precision mode with a low tensor-core threshold, so that the batched
# products take the grouped tensor-core launch
@pytest.mark.parametrize("precision,tol,extra", [
    ("fp64", 1e-10, {}),
    ("emu", 1e-9, {"emu_min_flops": 1e4}),
])
def test_batch_matches_each_solve_alone(ctx, precision, tol, extra):
    systems = [make_system(4, 24, 72, seed=s) for s in (1, 2, 3)]
    opts = dict(OPTS, precision=precision, **extra)
    batch = gpu.ccsd_solve_batch(ctx, [(s.eps_h, s.eps_p, s.gamma) for s in systems],
                                 want_amplitudes=True, **opts)
    for s, got in zip(systems, batch):
        ref = _alone(ctx, s, **opts)
        assert got["status"] == ref["status"]
        assert got["iterations"] == ref["iterations"]
        assert abs(got["energy"] - ref["energy"]) <= tol
        np.testing.assert_allclose(got["history"], ref["history"], rtol=0, atol=tol)
        np.testing.assert_allclose(got["T2"], ref["T2"], rtol=0, atol=1e-8)


def test_batch_with_uneven_iteration_counts(ctx):
    """Systems that converge at different iterations: each is frozen where it
    converged while the others go on."""
    systems = [make_system(3, 20, 60, seed=s) for s in (5, 6, 7, 8)]
    opts = dict(OPTS, precision="fp64", max_residua=4)
    batch = gpu.ccsd_solve_batch(ctx, [(s.eps_h, s.eps_p, s.gamma) for s in systems],
                                 **opts)
    refs = [_alone(ctx, s, **opts) for s in systems]
    assert [b["iterations"] for b in batch] == [r["iterations"] for r in refs]
    for got, ref in zip(batch, refs):
        assert abs(got["energy"] - ref["energy"]) <= 1e-10


def test_batch_rejects_systems_of_different_shapes(ctx):
    a, b = make_system(3, 20, 60, seed=1), make_system(3, 22, 66, seed=2)
    with pytest.raises(capi.GbccError) as e:
        gpu.ccsd_solve_batch(ctx, [(a.eps_h, a.eps_p, a.gamma), (b.eps_h, b.eps_p, b.gamma)],
                             **OPTS)
    assert e.value.status == capi.BAD_ARG
    with pytest.raises(capi.GbccError) as e:
        gpu.ccsd_solve_batch(ctx, [(a.eps_h, a.eps_p, a.gamma)] * 2,
                             **dict(OPTS, mixer="LinearMixer"))
    assert e.value.status == capi.BAD_ARG
