"""Options of the real CCSD solver against the oracle (GPU): levelShift,
integralsSliceFactor, PairEnergy, given starting amplitudes and a one-vector
DIIS.

This file is collected after the validated GPU tests on purpose, so that a
failure here cannot stop them in a run that stops at the first failure.
"""
import numpy as np
import pytest

from oracle.ccsd import ccsd as oracle_ccsd
from oracle.ccsd import pair_energy as oracle_pair_energy
from oracle.coulomb import coulomb_integrals
from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu

ETOL = 1e-10  # Ha, per iteration


def _case(No=4, Nv=13, NG=30, seed=12):
    s = make_system(No, Nv, NG, seed=seed)
    return s, coulomb_integrals(s.gamma, No)


def _history(r):
    return np.array([h["energy"]["value"] for h in r["history"]])


@pytest.mark.parametrize("mixer", ["LinearMixer", "DiisMixer"])
def test_level_shift(ctx, mixer):
    """levelShift s: T = -(R - s T) / (D + s) (CcsdEnergyFromCoulombIntegrals.cxx:302-331)."""
    s, ints = _case()
    kw = dict(mixer=mixer, max_residua=4, level_shift=0.4, max_iterations=10,
              energy_convergence=0.0, amplitudes_convergence=0.0)
    ref = oracle_ccsd(s.eps_h, s.eps_p, ints, s.gamma, **kw)
    got = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    assert np.abs(got["history"] - _history(ref)).max() < ETOL


@pytest.mark.parametrize("factor", [0.25, 0.5, 1.0])
def test_slice_factor(ctx, factor):
    """integralsSliceFactor: slices of Nv * factor; the energies do not depend
    on the slicing."""
    s, ints = _case()
    kw = dict(max_iterations=5, energy_convergence=0.0, amplitudes_convergence=0.0)
    ref = oracle_ccsd(s.eps_h, s.eps_p, ints, s.gamma, slice_factor=factor, **kw)
    got = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, slice_factor=factor, **kw)
    assert np.abs(got["history"] - _history(ref)).max() < ETOL


def test_pair_energies(ctx):
    """PairEnergy[i,j] (ClusterSinglesDoublesAlgorithm.cxx:218-234) of the final
    amplitudes; the pair energies add up to the correlation energy."""
    s, ints = _case()
    r = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, pair_energy=True, max_iterations=6,
                       energy_convergence=0.0, amplitudes_convergence=0.0)
    ref = oracle_pair_energy(r["T1"], r["T2"], ints["PPHH"])
    assert np.abs(r["pair_energy"] - ref).max() < 1e-12 * np.abs(ref).max()
    assert abs(r["pair_energy"].sum() - r["energy"]) < 1e-12 * abs(r["energy"])


def test_given_starting_amplitudes(ctx):
    """initialSinglesAmplitudes / initialDoublesAmplitudes: the first iteration
    is a full one from the given amplitudes (no MP2 start)."""
    s, ints = _case()
    rng = np.random.default_rng(3)
    T1 = 0.01 * rng.normal(size=(s.Nv, s.No))
    T2 = 0.01 * rng.normal(size=(s.Nv, s.Nv, s.No, s.No))
    T2 = 0.5 * (T2 + T2.transpose(1, 0, 3, 2))
    kw = dict(mixer="DiisMixer", max_residua=3, max_iterations=8, energy_convergence=0.0,
              amplitudes_convergence=0.0)
    ref = oracle_ccsd(s.eps_h, s.eps_p, ints, s.gamma, initial=(T1, T2), **kw)
    got = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, initial=(T1, T2), **kw)
    assert np.abs(got["history"] - _history(ref)).max() < ETOL
    assert np.abs(got["T2"] - ref["T2"]).max() < 1e-9 * np.abs(ref["T2"]).max()


def test_diis_with_one_vector(ctx):
    """maxResidua 1: the DIIS solve of a 2x2 bordered system, i.e. the plain
    Jacobi update."""
    s, ints = _case()
    kw = dict(mixer="DiisMixer", max_residua=1, max_iterations=6, energy_convergence=0.0,
              amplitudes_convergence=0.0)
    ref = oracle_ccsd(s.eps_h, s.eps_p, ints, s.gamma, **kw)
    got = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    assert np.abs(got["history"] - _history(ref)).max() < ETOL
    lin = oracle_ccsd(s.eps_h, s.eps_p, ints, s.gamma, mixer="LinearMixer",
                      **{k: v for k, v in kw.items() if k not in ("mixer", "max_residua")})
    assert np.abs(_history(ref) - _history(lin)).max() < 1e-13
