"""Precision gate at the headline size (GPU): No=32, Nv=256, NG=1024, seed 1,
12 iterations from the MP2 start with DiisMixer(5) and levelShift 16, then
(T) on the 12th-iteration amplitudes.

The precision form (every large contraction emulated in FP64 on the bf16
tensor cores: 6 or 5 digits per operand in the CCSD iterations, one more in
(T))
must reproduce the FP64 energies within 1 microhartree:

* every one of the 12 iteration energies against the CPU oracle's trajectory
  (committed in tests/golden/c2_trajectory.json);
* E_(T) and E_CCSD + E_(T) (the reference's CcsdPerturbativeTriplesEnergy,
  CcsdPerturbativeTriples.cxx:241-247) against the FP64 (T) of the FP64
  trajectory, end to end: each side iterates and computes (T) in its own
  arithmetic.

The FP64 GPU path itself is checked against the oracle on the first full
iteration (bound 1e-9 Ha at |E| ~ 300 Ha).  The energies here are of order
1e2-1e4 Ha, so 1 microhartree is a relative accuracy of about 1e-9 to 1e-10.
"""
import json
import os

import pytest

from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system
from tests.golden.cases import C2, C2_FILE, C2_SOLVE

pytestmark = pytest.mark.gpu

BOUND_HA = 1e-6


@pytest.fixture(scope="module")
def c2():
    with open(C2_FILE) as f:
        doc = json.load(f)
    assert doc["system"] == C2 and doc["solve"] == C2_SOLVE
    return make_system(**C2), doc


# (digits per operand in the CCSD iterations, digits in (T))
@pytest.mark.parametrize("ccsd_digits,triples_digits", [(6, 7), (5, 6)])
def test_precision_form_meets_one_microhartree_at_c2(ctx, c2, ccsd_digits, triples_digits):
    s, doc = c2
    ref = [r["energy"] for r in doc["oracle"]["energies"]]
    ctx.set_emulation(ccsd_digits, 1e7)
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, precision="emu", **C2_SOLVE)
    try:
        es = [sol.step(1)[0] for _ in range(C2_SOLVE["max_iterations"])]
        # (T) runs with one digit more than the context's setting
        ctx.set_emulation(triples_digits - 1, 1e7)
        e_t, _ = sol.triples("emu")
    finally:
        ctx.set_emulation(6, 1e7)
        sol.close()
    dE = [a - b for a, b in zip(es, ref)]
    assert len(dE) == 12
    assert max(abs(x) for x in dE) <= BOUND_HA, dE
    g = doc["gpu_fp64"]
    dE_t = e_t - g["e_t"]
    dE_total = (es[-1] + e_t) - (ref[-1] + g["e_t"])
    assert abs(dE_t) <= BOUND_HA, (e_t, g["e_t"])
    assert abs(dE_total) <= BOUND_HA, dE_total


def test_fp64_path_follows_the_oracle_at_c2(ctx, c2):
    s, doc = c2
    ref = [r["energy"] for r in doc["oracle"]["energies"]]
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, precision="fp64", **C2_SOLVE)
    try:
        es = [sol.step(1)[0] for _ in range(2)]
    finally:
        sol.close()
    assert abs(es[0] - ref[0]) <= 1e-9 and abs(es[1] - ref[1]) <= 1e-9, (es, ref[:2])
    # the recorded FP64 trajectory follows the oracle at every iteration
    fp = doc["gpu_fp64"]["energies"]
    assert max(abs(a - b) for a, b in zip(fp, ref)) <= 1e-8
