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


@pytest.mark.parametrize("precision,tol,extra", [
    ("fp64", 1e-10, {}),
    ("emu", 1e-9, {"emu_min_flops": 1e4}),
])
def test_batch_with_uneven_iteration_counts(ctx, precision, tol, extra):
    """Systems that converge at different iterations: each stops where it
    converged and leaves the stacked inputs (whose cached digit panels are
    then dropped) while the others go on."""
    systems = [make_system(3, 20, 60, seed=s) for s in (5, 6, 7, 8)]
    opts = dict(OPTS, precision=precision, max_residua=4, **extra)
    batch = gpu.ccsd_solve_batch(ctx, [(s.eps_h, s.eps_p, s.gamma) for s in systems],
                                 **opts)
    refs = [_alone(ctx, s, **opts) for s in systems]
    assert [b["iterations"] for b in batch] == [r["iterations"] for r in refs]
    for got, ref in zip(batch, refs):
        assert abs(got["energy"] - ref["energy"]) <= tol


def test_a_failing_system_leaves_the_batch(ctx):
    """A system that stops with an error (a singular DIIS matrix, made on the
    host) reports it and drops out of the stacked inputs; the others go on
    and end as they would alone."""
    systems = [make_system(3, 20, 60, seed=s) for s in (5, 6, 7)]
    opts = dict(OPTS, precision="fp64", max_residua=4)
    ctx.inject_fault(capi.FAULT_DIIS_SINGULAR)
    batch = gpu.ccsd_solve_batch(ctx, [(s.eps_h, s.eps_p, s.gamma) for s in systems],
                                 **opts)
    ctx.inject_fault(capi.FAULT_NONE)
    # the first system to take in an iteration's results takes the fault
    assert batch[0]["status"] == capi.DIIS_SINGULAR and batch[0]["iterations"] == 1
    for s, got in zip(systems[1:], batch[1:]):
        ref = _alone(ctx, s, **opts)
        assert got["status"] == ref["status"] == capi.OK
        assert got["iterations"] == ref["iterations"]
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


def test_server_solves_queued_requests_of_one_shape_together(ctx):
    """A server slot that admits a request takes the queued requests of the
    same shape and options with it and solves them in lockstep; each result
    agrees with the request's solve alone."""
    from sisi4s_gb300 import serve
    opts = dict(OPTS, precision="fp64")
    blocker = make_system(4, 28, 112, seed=9)
    same = [make_system(3, 20, 80, seed=s) for s in (21, 22, 23, 24)]
    srv = serve.Server(slots=1)
    ids = [srv.submit(blocker, **opts)]  # holds the only slot meanwhile
    ids += [srv.submit(s, **opts) for s in same]
    res = [srv.wait(i) for i in ids]
    srv.close()
    assert len({r["t_admit"] for r in res[1:]}) == 1
    assert res[1]["t_admit"] >= res[0]["t_done"]
    for s, r in zip(same, res[1:]):
        ref = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **opts)
        et, _ = gpu.triples(ctx, s.eps_h, s.eps_p, s.gamma, ref["T1"], ref["T2"])
        assert r["status"] == ref["status"]
        assert r["iterations"] == ref["iterations"]
        assert abs(r["e_ccsd"] - ref["energy"]) <= 1e-10
        assert abs(r["e_t"] - et) <= 1e-10
