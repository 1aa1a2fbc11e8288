"""The GPU path against the committed golden fixtures of ``tests/golden/``.

``oracle_cases.json`` records the oracle's energies on the seeded systems of
``tests/golden/cases.py``: CCSD trajectories of both real formulations, the
(T) energy, and a complex trajectory with its complex (T).  The device
solvers, called through the C ABI, must reproduce them.  This file is
collected after the other GPU tests on purpose, so that a failure here cannot
stop them in a run that stops at the first failure.
"""
import numpy as np
import pytest

from sisi4s_gb300 import ccsd as gpu
from tests.golden import cases

pytestmark = pytest.mark.gpu

ETOL = 1e-10  # Ha, per iteration


@pytest.fixture(scope="module")
def fx():
    return cases.load(cases.ORACLE_FILE)


@pytest.mark.parametrize("formulation,key", [("vertex", "vertex"), ("stored", "stored")])
def test_real_trajectory_matches_fixture(ctx, fx, formulation, key):
    f = fx["real"][key]
    s = cases.real_system()
    r = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, formulation=formulation,
                       **cases.REAL_SOLVE)
    assert r["iterations"] == len(f["history"])
    assert np.abs(r["history"] - np.array(f["history"])).max() < ETOL
    assert abs(r["direct"] - f["direct"]) < ETOL
    assert abs(r["exchange"] - f["exchange"]) < ETOL
    assert abs(np.sum(r["T2"] ** 2) - f["t2_sumsq"]) < 1e-9 * f["t2_sumsq"]
    if key == "vertex":
        et, _ = gpu.triples(ctx, s.eps_h, s.eps_p, s.gamma, r["T1"], r["T2"])
        assert abs(et - f["triples"]) < 1e-12


def test_complex_trajectory_matches_fixture(ctx, fx):
    f = fx["complex"]
    s, g = cases.complex_system(**cases.COMPLEX)
    r = gpu.ccsd_solve_complex(ctx, s.eps_h, s.eps_p, g, **cases.COMPLEX_SOLVE)
    want = cases.complex_list(f["history"])
    assert r["iterations"] == want.size
    assert np.abs(r["history"] - want).max() < 1e-12
    et, _ = gpu.triples_complex(ctx, s.eps_h, s.eps_p, g, r["T1"], r["T2"])
    assert abs(et - cases.complex_list([f["triples"]])[0]) < 1e-12
