"""The large system (GPU): No=24, Nv=360, NG=1440 (seed 5), where V_abcd would
take 134 GB.  The particle ladder is streamed from the vertex slice by slice
(CcsdEnergyFromCoulombIntegrals.cxx:374-452), so the library's device
allocations must stay far below that size; and the precision form must give
the FP64 path's energies, from the MP2 start with DiisMixer(5) and
levelShift 16, within 1 microhartree over the first three iterations (the
FP64 path takes about 50 s per iteration here).
"""
import pytest

from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu

C5 = {"No": 24, "Nv": 360, "NG": 1440, "seed": 5}
SOLVE = {"mixer": "DiisMixer", "max_residua": 5, "level_shift": 16.0,
         "max_iterations": 12, "energy_convergence": 0.0, "amplitudes_convergence": 0.0}
ITERATIONS = 3


def _energies(ctx, s, precision):
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, precision=precision, **SOLVE)
    try:
        return [sol.step(1)[0] for _ in range(ITERATIONS)]
    finally:
        sol.close()


def test_large_system_streams_the_ladder_and_meets_one_microhartree(ctx):
    s = make_system(**C5)
    vabcd = 8 * C5["Nv"] ** 4
    emu = {}
    # 6 and 5 bf16 digits per operand
    for digits in (6, 5):
        ctx.set_emulation(digits, 1e7)
        ctx.pool_high_water(reset=True)
        try:
            emu[digits] = _energies(ctx, s, "emu")
        finally:
            ctx.set_emulation(6, 1e7)
        peak = ctx.pool_high_water()
        assert 0 < peak < 0.3 * vabcd, (digits, peak, vabcd)
    fp64 = _energies(ctx, s, "fp64")
    for digits, es in emu.items():
        dE = [a - b for a, b in zip(es, fp64)]
        assert max(abs(x) for x in dE) <= 1e-6, (digits, es, fp64)
