"""gbcc_ccsd_restart (GPU): a resident solver sent back to its starting state
repeats its trajectory bit for bit, with the integrals, buffers and captured
iteration graphs of the first pass.  Each case runs past the point where the
DIIS ring is full (so graphs are captured and replayed) before restarting;
the linear mixer case restarts after an odd number of iterations, when its
two amplitude buffers have swapped roles.
"""
import numpy as np
import pytest

from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system, mp2_amplitudes

pytestmark = pytest.mark.gpu


def _trajectory(sol, n):
    es = [sol.step(1)[0] for _ in range(n)]
    r = sol.result()
    return es, r


@pytest.mark.parametrize("mixer,n,first", [("DiisMixer", 9, 7), ("DiisMixer", 4, 2),
                                           ("LinearMixer", 5, 3)])
def test_restart_repeats_the_trajectory(ctx, mixer, n, first):
    s = make_system(4, 14, 33, seed=31)
    kw = dict(mixer=mixer, max_residua=3, max_iterations=n, energy_convergence=0.0,
              amplitudes_convergence=0.0, level_shift=0.5, mixing_ratio=0.8)
    fresh = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    try:
        sol.step(first)
        sol.restart()
        assert sol.result(amplitudes=False)["iterations"] == 0
        es, r = _trajectory(sol, n)
        sol.restart()
        es2, r2 = _trajectory(sol, n)
    finally:
        sol.close()
    assert es == list(fresh["history"]) == es2
    assert np.array_equal(r["T2"], fresh["T2"]) and np.array_equal(r2["T2"], fresh["T2"])
    assert np.array_equal(r["T1"], fresh["T1"])
    assert list(r["history"]) == es


def test_restart_returns_to_the_given_amplitudes(ctx):
    s = make_system(3, 11, 27, seed=32)
    init = mp2_amplitudes(s)
    kw = dict(mixer="DiisMixer", max_residua=4, max_iterations=6, energy_convergence=0.0,
              amplitudes_convergence=0.0)
    fresh = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, initial=init, **kw)
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, initial=init, **kw)
    try:
        sol.step(6)
        sol.restart()
        es, r = _trajectory(sol, 6)
    finally:
        sol.close()
    assert es == list(fresh["history"])
    assert np.array_equal(r["T2"], fresh["T2"])
