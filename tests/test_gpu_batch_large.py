"""Lockstep batch whose particle ladder runs system by system: when one
system's V blocks fill the GPU with output tiles, the batch keeps the fused
ladder (V written by the tensor cores straight into the digit panels of
R = V.X) for each system instead of a batched product.  (Sizes beyond the
host simulation's reach: GPU only.)"""
import pytest

from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu


def test_batch_with_per_system_fused_ladder(ctx):
    # Nv = 96, integralsSliceSize 16: V blocks of 1536 x 1536 are 288 output
    # tiles, above the 152 SMs
    systems = [make_system(3, 96, 288, seed=s) for s in (41, 42)]
    opts = dict(mixer="DiisMixer", max_residua=5, max_iterations=6, energy_convergence=0.0,
                amplitudes_convergence=0.0, precision="emu", emu_min_flops=1e6)
    batch = gpu.ccsd_solve_batch(ctx, [(s.eps_h, s.eps_p, s.gamma) for s in systems], **opts)
    for s, got in zip(systems, batch):
        ref = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, want_amplitudes=False, **opts)
        assert got["iterations"] == ref["iterations"] == 6
        assert abs(got["energy"] - ref["energy"]) <= 1e-9
        assert max(abs(a - b) for a, b in zip(got["history"], ref["history"])) <= 1e-9
