"""Energy terms of getEnergy beyond the canonical ones (GPU): the
HPFockMatrix noncanonical term and the energy of given amplitudes at
maxIterations 0 (ClusterSinglesDoublesAlgorithm.cxx:113-119, 199-209).

This file is collected after the other GPU tests on purpose, so that a
failure here cannot stop them in a run that stops at the first failure.
"""
import numpy as np
import pytest

from oracle.ccsd import ccsd as oracle_ccsd
from oracle.ccsd import energy as oracle_energy
from oracle.coulomb import coulomb_integrals as oracle_ints
from sisi4s_gb300 import capi
from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu

ETOL = 1e-10


def _rand_amplitudes(Nv, No, seed, scale=0.02):
    rng = np.random.default_rng(seed)
    T1 = rng.normal(0, scale, (Nv, No))
    T2 = rng.normal(0, scale, (Nv, Nv, No, No))
    return T1, 0.5 * (T2 + T2.transpose(1, 0, 3, 2))


@pytest.mark.parametrize("mixer", ["LinearMixer", "DiisMixer"])
def test_noncanonical_fock_term_matches_oracle(ctx, mixer):
    """HPFockMatrix adds spins * T1_ai f_ia to every iteration's energy
    (ClusterSinglesDoublesAlgorithm.cxx:199-209)."""
    s = make_system(4, 13, 30, seed=12)
    ints = oracle_ints(s.gamma, 4)
    fia = np.random.default_rng(4).normal(0, 0.05, (4, 13))
    kw = dict(mixer=mixer, max_residua=3, max_iterations=6,
              energy_convergence=0.0, amplitudes_convergence=0.0)
    ref = oracle_ccsd(s.eps_h, s.eps_p, ints, s.gamma, fock_hp=fia, **kw)
    got = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, fock_hp=fia, **kw)
    plain = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    refh = np.array([h["energy"]["value"] for h in ref["history"]])
    assert got["iterations"] == ref["iterations"] == 6
    assert np.abs(np.array(got["history"]) - refh).max() < ETOL
    # the term is present: after the MP2 start T1 != 0 and the energies move
    assert abs(got["energy"] - plain["energy"]) > 1e-8


def test_zero_iterations_report_the_energy_of_the_given_amplitudes(ctx):
    """maxIterations 0: no iteration runs and the energy of the given
    amplitudes is reported (ClusterSinglesDoublesAlgorithm.cxx:113-119)."""
    s = make_system(4, 12, 30, seed=13)
    ints = oracle_ints(s.gamma, 4)
    T1, T2 = _rand_amplitudes(12, 4, seed=6)
    fia = np.random.default_rng(5).normal(0, 0.05, (4, 12))
    ref = oracle_energy(T1, T2, ints["PPHH"], fock_hp=fia)["value"]
    r = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, initial=(T1, T2),
                       fock_hp=fia, max_iterations=0)
    assert r["status"] == capi.OK and r["iterations"] == 0
    assert abs(r["energy"] - ref) < 1e-12 * abs(ref)
    assert np.array_equal(r["T1"], T1) and np.array_equal(r["T2"], T2)
