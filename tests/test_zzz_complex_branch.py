"""Complex (k-point) CCSD through the C ABI against the complex oracle (GPU).

The statement sequence is shared with the host-backend check of
``tests/test_complex_program.py``; these tests run it on the device.  This
file is collected after the other GPU tests on purpose, so that a failure
here cannot stop them in a run that stops at the first failure.
"""
import ctypes as C

import numpy as np
import pytest

from oracle.ccsd_complex import (ccsd_complex, coulomb_integrals_complex, pair_energy_complex,
                                 residual_complex, triples_complex_loop)
from oracle.ueg import UEG_GOLDEN, ueg_planewave
from sisi4s_gb300 import capi
from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu


def _system(No, Nv, NG, seed):
    s = make_system(No, Nv, NG, seed=seed)
    rng = np.random.default_rng(seed + 100)
    W, _ = np.linalg.qr(rng.normal(size=(NG, NG)) + 1j * rng.normal(size=(NG, NG)))
    ph = np.exp(1j * rng.uniform(0, 2 * np.pi, No + Nv))
    g = np.einsum("GH,Hpq->Gpq", W, np.conj(ph)[None, :, None] * s.gamma * ph[None, None, :])
    T1 = rng.normal(0, 0.05, (Nv, No)) + 1j * rng.normal(0, 0.05, (Nv, No))
    T2 = rng.normal(0, 0.05, (Nv, Nv, No, No)) + 1j * rng.normal(0, 0.05, (Nv, Nv, No, No))
    return s, g, T1, 0.5 * (T2 + T2.transpose(1, 0, 3, 2))


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("No,Nv,NG,dist,ppl,slice_size", [
    (3, 7, 11, 0, 1, -1), (3, 9, 14, 1, 1, 2), (2, 10, 12, 0, 0, -1), (4, 11, 20, 0, 1, 4)])
def test_complex_residual_matches_oracle(ctx, No, Nv, NG, dist, ppl, slice_size):
    s, g, T1, T2 = _system(No, Nv, NG, seed=No + Nv)
    ci = coulomb_integrals_complex(g, No)
    r1, r2 = gpu.ccsd_residual_complex(ctx, 1, T1, T2, s.eps_h, s.eps_p, g,
                                       initial_doubles=True, distinguishable=dist,
                                       ppl=ppl, slice_size=slice_size)
    o1, o2 = residual_complex(1, T1, T2, ci, g, distinguishable=dist, ppl=ppl,
                              slice_size=slice_size, initial_doubles=True)
    assert _rel(r1, o1) < 1e-12 and _rel(r2, o2) < 1e-12


def test_complex_residual_emulated_matches_oracle(ctx):
    No, Nv, NG = 4, 40, 64
    s, g, T1, T2 = _system(No, Nv, NG, seed=9)
    ci = coulomb_integrals_complex(g, No)
    ctx.set_emulation(6, 0.0)  # every GEMM emulated
    try:
        r1, r2 = gpu.ccsd_residual_complex(ctx, 1, T1, T2, s.eps_h, s.eps_p, g,
                                           initial_doubles=True, precision="emu",
                                           slice_size=16)
    finally:
        ctx.set_emulation(6, 1e7)
    o1, o2 = residual_complex(1, T1, T2, ci, g, slice_size=16, initial_doubles=True)
    assert _rel(r1, o1) < 1e-10 and _rel(r2, o2) < 1e-10


@pytest.mark.parametrize("ratio", [1.0, 0.7])
def test_complex_iterations_match_oracle(ctx, ratio):
    No, Nv, NG = 3, 9, 14
    s, g, _, _ = _system(No, Nv, NG, seed=6)
    ci = coulomb_integrals_complex(g, No)
    kw = dict(mixing_ratio=ratio, max_iterations=40, energy_convergence=1e-10,
              amplitudes_convergence=1e-8, slice_size=2)
    ref = ccsd_complex(s.eps_h, s.eps_p, ci, g, **kw)
    got = gpu.ccsd_solve_complex(ctx, s.eps_h, s.eps_p, g, **kw)
    rh = np.array([h["energy"]["value"] for h in ref["history"]])
    assert got["iterations"] == ref["iterations"] and got["converged"] == ref["converged"]
    assert np.abs(got["history"] - rh).max() < 1e-12
    assert _rel(got["T2"], ref["T2"]) < 1e-9


@pytest.mark.parametrize("No,Nv,NG,slice_size", [(1, 2, 1, 1), (1, 3, 2, -1), (2, 1, 3, -1)])
def test_complex_minimal_sizes(ctx, No, Nv, NG, slice_size):
    """One hole or one particle, one vertex row: single-element ladder slices,
    and (T) where all six images of a triple coincide (one hole) or all
    particle indices are equal (one particle).  There the spin/Fermi factors
    sum to zero (8 - 3*4 + 2*2), so E_(T) vanishes up to round-off."""
    s, g, _, _ = _system(No, Nv, NG, seed=3)
    ci = coulomb_integrals_complex(g, No)
    kw = dict(max_iterations=5, energy_convergence=0.0, amplitudes_convergence=0.0,
              slice_size=slice_size)
    ref = ccsd_complex(s.eps_h, s.eps_p, ci, g, **kw)
    got = gpu.ccsd_solve_complex(ctx, s.eps_h, s.eps_p, g, **kw)
    rh = np.array([h["energy"]["value"] for h in ref["history"]])
    assert got["iterations"] == rh.size
    assert np.abs(got["history"] - rh).max() < 1e-12 * np.abs(rh).max()
    et, _ = gpu.triples_complex(ctx, s.eps_h, s.eps_p, g, got["T1"], got["T2"])
    ref_t = triples_complex_loop(s.eps_h, s.eps_p, ref["T1"], ref["T2"], ci["PPHH"],
                                 ci["PHHH"], g)
    scale = abs(ref["energy_complex"])
    assert abs(ref_t) < 1e-14 * scale and abs(et) < 1e-14 * scale


def test_real_vertex_through_the_complex_branch_equals_the_real_branch(ctx):
    s = make_system(4, 12, 30, seed=5)
    kw = dict(max_iterations=6, energy_convergence=0.0, amplitudes_convergence=0.0)
    real = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    cplx = gpu.ccsd_solve_complex(ctx, s.eps_h, s.eps_p, s.gamma.astype(complex), **kw)
    assert np.abs(cplx["history"].real - np.array(real["history"])).max() < 1e-12
    assert np.abs(cplx["history"].imag).max() < 1e-15


def test_ueg_golden_through_the_complex_branch(ctx):
    """The reference's UEG test on its own plane-wave vertex, made complex by
    random orbital phases, with the linear mixer (no complex DIIS exists)."""
    gd = UEG_GOLDEN
    _, eps, gam, _ = ueg_planewave(gd["No"], gd["Nv"], gd["rs"])
    ph = np.exp(1j * np.random.default_rng(11).uniform(0, 2 * np.pi, gam.shape[1]))
    gam = np.conj(ph)[None, :, None] * gam * ph[None, None, :]
    n = gd["No"]
    r = gpu.ccsd_solve_complex(ctx, eps[:n], eps[n:], gam, max_iterations=60,
                               energy_convergence=1e-11, amplitudes_convergence=1e-9)
    assert r["converged"]
    assert abs(r["history"][0].real - gd["mp2"]) < 1e-12
    assert abs(r["energy"].real - gd["ccsd"]) < 1e-8 * abs(gd["ccsd"])
    assert abs(r["energy"].imag) < 1e-14
    et, etot = gpu.triples_complex(ctx, eps[:n], eps[n:], gam, r["T1"], r["T2"],
                                   e_ccsd=r["energy"].real)
    assert abs(et.real - gd["triples"]) < 1e-10 and abs(et.imag) < 1e-14
    assert etot == r["energy"].real + et.real


def test_complex_diis_is_refused(ctx):
    s, g, _, _ = _system(2, 5, 7, seed=1)
    inp = gpu.ComplexInput(s.eps_h, s.eps_p, g)
    o = gpu.make_opts(mixer="DiisMixer")
    out = capi.ComplexOut()
    st = ctx.lib.gbcc_ccsd_solve_complex(ctx.h, C.byref(inp.s), C.byref(o), C.byref(out))
    assert st == capi.BAD_ARG


@pytest.mark.parametrize("No,Nv,NG,precision", [(3, 6, 9, "fp64"), (2, 7, 10, "fp64"),
                                                (3, 12, 20, "emu")])
def test_complex_triples_matches_oracle(ctx, No, Nv, NG, precision):
    s, g, T1, T2 = _system(No, Nv, NG, seed=No + Nv)
    ci = coulomb_integrals_complex(g, No)
    ref = triples_complex_loop(s.eps_h, s.eps_p, T1, T2, ci["PPHH"], ci["PHHH"], g)
    if precision == "emu":
        ctx.set_emulation(6, 0.0)  # every GEMM emulated
    try:
        et, _ = gpu.triples_complex(ctx, s.eps_h, s.eps_p, g, T1, T2, precision=precision)
    finally:
        ctx.set_emulation(6, 1e7)
    tol = 1e-12 if precision == "fp64" else 1e-10
    assert abs(et - ref) < tol * abs(ref)


def test_complex_integrals_match_oracle(ctx):
    s, g, _, _ = _system(3, 7, 11, seed=2)
    ref = coulomb_integrals_complex(g, 3)
    got = gpu.coulomb_integrals_complex(ctx, g, 3)
    for k in ("PPHH", "PHHP", "HHPP", "PHPH", "HHHH", "HHHP", "PHHH"):
        assert _rel(got[k], ref[k]) < 1e-13, k


def test_complex_noncanonical_fock_term(ctx):
    No, Nv, NG = 3, 8, 12
    s, g, _, _ = _system(No, Nv, NG, seed=4)
    ci = coulomb_integrals_complex(g, No)
    rng = np.random.default_rng(12)
    f = rng.normal(0, 0.05, (No, Nv)) + 1j * rng.normal(0, 0.05, (No, Nv))
    kw = dict(max_iterations=6, energy_convergence=0.0, amplitudes_convergence=0.0,
              slice_size=3)
    ref = ccsd_complex(s.eps_h, s.eps_p, ci, g, fock_hp=f, **kw)
    got = gpu.ccsd_solve_complex(ctx, s.eps_h, s.eps_p, g, fock_hp=f, **kw)
    rh = np.array([h["energy"]["value"] for h in ref["history"]])
    assert np.abs(got["history"] - rh).max() < 1e-12


def test_complex_pair_energies(ctx):
    No, Nv, NG = 3, 8, 12
    s, g, _, _ = _system(No, Nv, NG, seed=5)
    ci = coulomb_integrals_complex(g, No)
    r = gpu.ccsd_solve_complex(ctx, s.eps_h, s.eps_p, g, pair_energy=True, max_iterations=4,
                               energy_convergence=0.0, amplitudes_convergence=0.0)
    ref = pair_energy_complex(r["T1"], r["T2"], ci["HHPP"])
    assert np.abs(r["pair_energy"] - ref).max() < 1e-12 * np.abs(ref).max()
    # the pair energies sum to the correlation energy (:189, :227-232)
    assert abs(r["pair_energy"].sum() - r["energy"]) < 1e-12 * abs(r["energy"])


COMPLEX_STEPS = """
- name: DefineHolesAndParticles
  in: { fileName: "EigenEnergies.yaml" }
  out: { HoleEigenEnergies: $Eh, ParticleEigenEnergies: $Ep }
- name: Read
  in: { fileName: "CoulombVertex.yaml" }
  out: { destination: $G }
- name: CoulombIntegralsFromVertex
  in: { CoulombVertex: $G, HoleEigenEnergies: $Eh, ParticleEigenEnergies: $Ep, complex: 1 }
  out:
    PPHHCoulombIntegrals: $PPHH
    PHPHCoulombIntegrals: $PHPH
    HHHHCoulombIntegrals: $HHHH
    HHHPCoulombIntegrals: $HHHP
    PHHHCoulombIntegrals: $PHHH
- name: CcsdEnergyFromCoulombIntegrals
  in:
    maxIterations: 60
    energyConvergence: 1e-11
    amplitudesConvergence: 1e-9
    HoleEigenEnergies: $Eh
    ParticleEigenEnergies: $Ep
    CoulombVertex: $G
    PPHHCoulombIntegrals: $PPHH
    PHPHCoulombIntegrals: $PHPH
    HHHHCoulombIntegrals: $HHHH
    HHHPCoulombIntegrals: $HHHP
  out:
    CcsdEnergy: $E
    CcsdSinglesAmplitudes: $T1
    CcsdDoublesAmplitudes: $T2
- name: CcsdPerturbativeTriplesComplex
  in:
    HoleEigenEnergies: $Eh
    ParticleEigenEnergies: $Ep
    CoulombVertex: $G
    PPHHCoulombIntegrals: $PPHH
    CcsdEnergy: $E
    CcsdSinglesAmplitudes: $T1
    CcsdDoublesAmplitudes: $T2
  out:
    CcsdPerturbativeTriplesComplexEnergy: $Etot
"""


def test_ueg_golden_through_the_complex_pipeline_in_the_runner(tmp_path):
    """The step runner end to end on the complex branch: the reference's UEG
    plane-wave vertex with random orbital phases, written as a Complex64 cc4s
    file, through CoulombIntegralsFromVertex (complex: 1), the complex CCSD
    and CcsdPerturbativeTriplesComplex; the golden energies come out."""
    import json
    import os
    import subprocess

    from sisi4s_gb300 import build
    build.build()
    runner = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                          "sisi4s_gb300", "_lib", "sisi4s-gb300")
    gd = UEG_GOLDEN
    _, eps, gam, _ = ueg_planewave(gd["No"], gd["Nv"], gd["rs"])
    ph = np.exp(1j * np.random.default_rng(11).uniform(0, 2 * np.pi, gam.shape[1]))
    gam = np.conj(ph)[None, :, None] * gam * ph[None, None, :]
    n = gd["No"]
    fermi = 0.5 * (eps[:n].max() + eps[n:].min())
    (tmp_path / "EigenEnergies.yaml").write_text(
        "metaData:\n  fermiEnergy: %.17g\n  energies: [%s]\n"
        % (fermi, ", ".join("%.17g" % e for e in eps)))
    NG, Np, _ = gam.shape
    (tmp_path / "CoulombVertex.yaml").write_text(
        "version: 100\ntype: Tensor\ndimensions:\n"
        "  - length: %d\n    type: AuxiliaryField\n"
        "  - length: %d\n    type: State\n  - length: %d\n    type: State\n"
        "scalarType: Complex64\nelements:\n  type: IeeeBinaryFile\nunit: 1.0\n" % (NG, Np, Np))
    z = np.ascontiguousarray(gam.transpose(2, 1, 0)).ravel()
    z.view(np.float64).tofile(tmp_path / "CoulombVertex.elements")
    (tmp_path / "in.yaml").write_text(COMPLEX_STEPS)
    r = subprocess.run([runner, "-i", "in.yaml", "-o", "out.yaml"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads((tmp_path / "out.yaml").read_text())
    steps = {s["name"]: s for s in out["steps"]}
    cc = steps["CcsdEnergyFromCoulombIntegrals"]
    assert cc["convergenceReached"] == 1
    assert abs(cc["iterations"][0]["energy"]["value"] - gd["mp2"]) < 1e-12
    assert abs(cc["energy"]["value"] - gd["ccsd"]) < 1e-8 * abs(gd["ccsd"])
    assert abs(cc["energy"]["imaginary"]) < 1e-14
    t = steps["CcsdPerturbativeTriplesComplex"]["energy"]
    assert abs(t["triples"] - gd["triples"]) < 1e-10 and abs(t["triplesImaginary"]) < 1e-14
    assert t["value"] == cc["energy"]["value"] + t["triples"]
