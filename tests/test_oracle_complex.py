"""Pins of the complex (k-point) CCSD(T) oracle (no GPU).

The complex branch of the reference (complex integrals, complex residual,
complex (T)) is checked four ways:
- on a real vertex it must equal the real path;
- mixing the vertex rows by a unitary leaves every integral unchanged, so the
  residual must not move;
- a phase change of the orbitals must change the residual covariantly and
  leave the energies unchanged;
- on the plane-wave vertex of the reference's UEG integration test, made
  genuinely complex by random orbital phases, it must reproduce that test's
  golden MP2, CCSD and (T) energies.
"""
import numpy as np
import pytest

from oracle.ccsd import energy, residual
from oracle.ccsd_complex import (ComplexDiisUnsupported, ccsd_complex,
                                 coulomb_integrals_complex, energy_complex,
                                 residual_complex, triples_complex_loop)
from oracle.coulomb import coulomb_integrals
from oracle.triples import triples_loop
from oracle.ueg import UEG_GOLDEN, ueg_planewave
from sisi4s_gb300.inputs import make_system

No, Nv, NG = 3, 9, 14


@pytest.fixture(scope="module")
def case():
    s = make_system(No, Nv, NG, seed=4)
    rng = np.random.default_rng(3)
    T1 = rng.normal(0, 0.05, (Nv, No))
    T2 = rng.normal(0, 0.05, (Nv, Nv, No, No))
    T2 = 0.5 * (T2 + T2.transpose(1, 0, 3, 2))
    ints = coulomb_integrals(s.gamma, No, keys=("PPHH", "PHPH", "HHHH", "HHHP"))
    cints = coulomb_integrals_complex(s.gamma.astype(complex), No)
    return s, T1, T2, ints, cints


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


def test_complex_integrals_of_a_real_vertex_are_the_real_integrals(case):
    s, _, _, ints, ci = case
    for k in ("PPHH", "PHPH", "HHHH", "HHHP"):
        assert np.array_equal(ci[k], ints[k])
    assert np.array_equal(ci["HHPP"], ints["PPHH"].transpose(2, 3, 0, 1))
    # the real path builds PHHP and PHHH by permutation
    # (CoulombIntegralsFromVertex.cxx:516, :539)
    assert np.array_equal(ci["PHHP"], np.einsum("abji->aijb", ints["PPHH"]))
    assert np.array_equal(ci["PHHH"], np.einsum("kjia->aijk", ints["HHHP"]))


@pytest.mark.parametrize("dist,ppl,slice_size", [(0, 1, -1), (1, 1, 2), (0, 0, -1), (0, 1, 4)])
def test_complex_residual_equals_real_residual_on_real_input(case, dist, ppl, slice_size):
    s, T1, T2, ints, ci = case
    r1, r2 = residual(1, T1, T2, ints, s.gamma, distinguishable=dist, ppl=ppl,
                      slice_size=slice_size)
    c1, c2 = residual_complex(1, T1, T2, ci, s.gamma.astype(complex),
                              distinguishable=dist, ppl=ppl, slice_size=slice_size)
    assert _rel(c1, r1) < 1e-14 and _rel(c2, r2) < 1e-14


def test_vertex_row_mixing_leaves_the_residual_unchanged(case):
    s, T1, T2, ints, _ = case
    rng = np.random.default_rng(5)
    W, _ = np.linalg.qr(rng.normal(size=(NG, NG)) + 1j * rng.normal(size=(NG, NG)))
    gm = np.einsum("GH,Hpq->Gpq", W, s.gamma)
    cm = coulomb_integrals_complex(gm, No)
    c1, c2 = residual_complex(1, T1, T2, cm, gm, slice_size=2)
    r1, r2 = residual(1, T1, T2, ints, s.gamma, slice_size=2)
    assert _rel(c1, r1) < 1e-13 and _rel(c2, r2) < 1e-13


def _phased(case, seed=7):
    """Orbital phases phi_p -> e^{i t_p} phi_p: Gamma_Gpq -> e^{-i t_p}
    Gamma_Gpq e^{i t_q}, T_ai -> e^{-i t_a} T_ai e^{i t_i} (likewise T2)."""
    s, T1, T2, _, _ = case
    ph = np.exp(1j * np.random.default_rng(seed).uniform(0, 2 * np.pi, No + Nv))
    g = np.conj(ph)[None, :, None] * s.gamma * ph[None, None, :]
    pa, pi = ph[No:], ph[:No]
    f1 = np.conj(pa)[:, None] * pi[None, :]
    f2 = (np.conj(pa)[:, None, None, None] * np.conj(pa)[None, :, None, None]
          * pi[None, None, :, None] * pi[None, None, None, :])
    return g, f1, f2


def test_orbital_phases_act_covariantly(case):
    s, T1, T2, ints, _ = case
    g, f1, f2 = _phased(case)
    cp = coulomb_integrals_complex(g, No)
    c1, c2 = residual_complex(1, T1 * f1, T2 * f2, cp, g, slice_size=2)
    r1, r2 = residual(1, T1, T2, ints, s.gamma, slice_size=2)
    assert _rel(c1, r1 * f1) < 1e-13 and _rel(c2, r2 * f2) < 1e-13
    e = energy_complex(T1 * f1, T2 * f2, cp["HHPP"])["value"]
    ref = energy(T1, T2, ints["PPHH"])["value"]
    assert abs(e - ref) < 1e-15 and abs(e.imag) < 1e-16


def test_complex_triples_agrees_with_the_real_triples(case):
    s, T1, T2, ints, ci = case
    ref = triples_loop(s.eps_h, s.eps_p, T1, T2, ints["PPHH"], ints["HHHP"], s.gamma)
    et = triples_complex_loop(s.eps_h, s.eps_p, T1.astype(complex), T2.astype(complex),
                              ci["PPHH"], ci["PHHH"], s.gamma.astype(complex))
    g, f1, f2 = _phased(case)
    cp = coulomb_integrals_complex(g, No)
    etp = triples_complex_loop(s.eps_h, s.eps_p, T1 * f1, T2 * f2, cp["PPHH"],
                               cp["PHHH"], g)
    for e in (et, etp):
        assert abs(e.real - ref) < 1e-14 * abs(ref) and abs(e.imag) < 1e-16


def test_complex_path_reproduces_the_ueg_golden_energies():
    """The reference's UEG test (No=7, Nv=26, rs=1) run through the complex
    branch on its own plane-wave vertex, made complex by random orbital
    phases.  The reference has no complex DIIS, so the linear mixer is used;
    the golden CCSD energy was converged to 1e-8 (relative) with DIIS."""
    g = UEG_GOLDEN
    _, eps, gam, _ = ueg_planewave(g["No"], g["Nv"], g["rs"])
    ph = np.exp(1j * np.random.default_rng(11).uniform(0, 2 * np.pi, gam.shape[1]))
    gam = np.conj(ph)[None, :, None] * gam * ph[None, None, :]
    n = g["No"]
    ci = coulomb_integrals_complex(gam, n)
    r = ccsd_complex(eps[:n], eps[n:], ci, gam, max_iterations=60,
                     energy_convergence=1e-11, amplitudes_convergence=1e-9)
    assert r["converged"]
    assert abs(r["history"][0]["energy"]["value"] - g["mp2"]) < 1e-14
    assert abs(r["energy"] - g["ccsd"]) < 1e-8 * abs(g["ccsd"])
    assert abs(r["energy_complex"].imag) < 1e-15
    et = triples_complex_loop(eps[:n], eps[n:], r["T1"], r["T2"], ci["PPHH"],
                              ci["PHHH"], gam)
    assert abs(et.real - g["triples"]) < 1e-10 and abs(et.imag) < 1e-15


def test_complex_diis_is_refused_as_in_the_reference(case):
    s, _, _, _, ci = case
    with pytest.raises(ComplexDiisUnsupported):
        ccsd_complex(s.eps_h, s.eps_p, ci, s.gamma.astype(complex), mixer="DiisMixer")
