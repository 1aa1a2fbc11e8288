"""The stepping form of the C ABI (GPU): gbcc_ccsd_setup / step / result,
gbcc_triples_from_solver, gbcc_ccsd_device_amplitudes and gbcc_energy.

The solver keeps its state on the device between calls, so iterating in
chunks must give the bits of one gbcc_ccsd_solve call, and (T) from the
resident amplitudes must equal (T) from the same amplitudes passed from the
host.  This file is collected after the validated GPU tests on purpose, so
that a failure here cannot stop them in a run that stops at the first
failure.
"""
import ctypes as C

import numpy as np
import pytest

from oracle.ccsd import energy as oracle_energy
from oracle.coulomb import coulomb_integrals
from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu

KW = dict(mixer="DiisMixer", max_residua=4, max_iterations=9, energy_convergence=0.0,
          amplitudes_convergence=0.0)


@pytest.mark.parametrize("chunks", [(1, 2, 6), (4, 5), (9,)])
def test_stepping_in_chunks_equals_one_solve(ctx, chunks):
    s = make_system(4, 12, 30, seed=21)
    one = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **KW)
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, **KW)
    try:
        for n in chunks:
            e, _ = sol.step(n)
        r = sol.result()
    finally:
        sol.close()
    assert r["iterations"] == one["iterations"] == sum(chunks)
    assert e == r["energy"] == one["energy"]
    assert np.array_equal(r["T2"], one["T2"]) and np.array_equal(r["T1"], one["T1"])


def test_triples_from_the_resident_amplitudes(ctx):
    s = make_system(3, 10, 24, seed=22)
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, **KW)
    try:
        sol.step(KW["max_iterations"])
        r = sol.result()
        et, etot = sol.triples()
    finally:
        sol.close()
    et_host, etot_host = gpu.triples(ctx, s.eps_h, s.eps_p, s.gamma, r["T1"], r["T2"],
                                     e_ccsd=r["energy"])
    assert abs(et - et_host) <= 1e-14 * abs(et_host)
    assert etot == r["energy"] + et


def test_energy_of_device_amplitudes(ctx):
    """gbcc_energy on the solver's resident amplitudes (device pointers from
    gbcc_ccsd_device_amplitudes) and a device copy of V_abij."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs CUDA device memory for the integrals")
    s = make_system(4, 12, 30, seed=23)
    ints = coulomb_integrals(s.gamma, 4)
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, **KW)
    try:
        sol.step(KW["max_iterations"])
        r = sol.result()
        t1, t2 = C.c_void_p(), C.c_void_p()
        ctx.check(ctx.lib.gbcc_ccsd_device_amplitudes(sol.h, C.byref(t1), C.byref(t2)))
        V = torch.tensor(ints["PPHH"].transpose(3, 2, 1, 0).copy().ravel(), device="cuda")
        torch.cuda.synchronize()
        d, x = C.c_double(), C.c_double()
        ctx.check(ctx.lib.gbcc_energy(ctx.h, 4, 12, t1, t2, C.c_void_p(V.data_ptr()),
                                      C.byref(d), C.byref(x)))
    finally:
        sol.close()
    ref = oracle_energy(r["T1"], r["T2"], ints["PPHH"])
    assert abs(d.value - ref["direct"]) < 1e-12 * abs(ref["direct"])
    assert abs(x.value - ref["exchange"]) < 1e-12 * abs(ref["exchange"])
    assert abs((d.value + x.value) - r["energy"]) < 1e-12 * abs(r["energy"])
