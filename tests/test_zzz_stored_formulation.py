"""CcsdEnergyFromCoulombIntegralsReference -- the stored-V_abcd formulation
of the same CCSD -- through the C ABI against the oracle (GPU).

Its statement program is shared with the host check in
``tests/test_complex_program.py``.  This file is collected after the other
GPU tests on purpose, so that a failure here cannot stop them in a run that
stops at the first failure.
"""
import numpy as np
import pytest

from oracle.ccsd import ccsd as oracle_ccsd
from oracle.ccsd import residual_reference
from oracle.coulomb import coulomb_integrals
from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu

KEYS = ("PPHH", "PHPH", "HHHH", "HHHP", "PPPP", "PPPH")


def _amplitudes(Nv, No, seed):
    rng = np.random.default_rng(seed)
    T1 = rng.normal(0, 0.02, (Nv, No))
    T2 = rng.normal(0, 0.02, (Nv, Nv, No, No))
    return T1, 0.5 * (T2 + T2.transpose(1, 0, 3, 2))


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("No,Nv,NG", [(3, 9, 20), (4, 14, 30), (1, 5, 8)])
def test_stored_residual_matches_oracle(ctx, No, Nv, NG):
    s = make_system(No, Nv, NG, seed=No + Nv)
    ints = coulomb_integrals(s.gamma, No, keys=KEYS)
    T1, T2 = _amplitudes(Nv, No, seed=3)
    r1, r2 = residual_reference(1, T1, T2, ints)
    g1, g2 = gpu.ccsd_residual(ctx, 1, T1, T2, s.eps_h, s.eps_p, s.gamma, formulation="stored")
    assert _rel(g1, r1) < 1e-12 and _rel(g2, r2) < 1e-12
    # the same with every integral given and no vertex
    h1, h2 = gpu.ccsd_residual(ctx, 1, T1, T2, s.eps_h, s.eps_p, None,
                               ints={k: ints[k] for k in KEYS}, formulation="stored")
    assert _rel(h1, r1) < 1e-12 and _rel(h2, r2) < 1e-12


def test_only_ppl_matches_oracle(ctx):
    s = make_system(3, 10, 20, seed=2)
    ints = coulomb_integrals(s.gamma, 3, keys=KEYS)
    T1, T2 = _amplitudes(10, 3, seed=4)
    _, r2 = residual_reference(0, T1, T2, ints, only_ppl=True)
    g1, g2 = gpu.ccsd_residual(ctx, 0, T1, T2, s.eps_h, s.eps_p, s.gamma,
                               formulation="stored", only_ppl=1)
    assert not g1.any() and _rel(g2, r2) < 1e-12


def test_stored_residual_emulated(ctx):
    s = make_system(4, 40, 64, seed=6)
    ints = coulomb_integrals(s.gamma, 4, keys=KEYS)
    T1, T2 = _amplitudes(40, 4, seed=5)
    r1, r2 = residual_reference(1, T1, T2, ints)
    ctx.set_emulation(6, 0.0)  # every GEMM emulated
    try:
        g1, g2 = gpu.ccsd_residual(ctx, 1, T1, T2, s.eps_h, s.eps_p, s.gamma,
                                   formulation="stored", precision="emu")
    finally:
        ctx.set_emulation(6, 1e7)
    assert _rel(g1, r1) < 1e-10 and _rel(g2, r2) < 1e-10


@pytest.mark.parametrize("mixer", ["LinearMixer", "DiisMixer"])
def test_stored_iterations_match_oracle_and_vertex_formulation(ctx, mixer):
    s = make_system(4, 14, 36, seed=8)
    ints = coulomb_integrals(s.gamma, 4, keys=KEYS)
    kw = dict(mixer=mixer, max_residua=3, max_iterations=10, energy_convergence=1e-12,
              amplitudes_convergence=1e-9)
    ref = oracle_ccsd(s.eps_h, s.eps_p, ints, s.gamma, formulation="reference", **kw)
    stored = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, formulation="stored", **kw)
    vertex = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    refh = np.array([h["energy"]["value"] for h in ref["history"]])
    assert stored["iterations"] == ref["iterations"]
    assert np.abs(np.array(stored["history"]) - refh).max() < 1e-10
    assert np.abs(np.array(stored["history"]) - np.array(vertex["history"])).max() < 1e-10


def test_particle_integrals_match_oracle(ctx):
    s = make_system(3, 8, 15, seed=9)
    ref = coulomb_integrals(s.gamma, 3, keys=("PPPP", "PPPH"))
    got = gpu.coulomb_integrals_pp(ctx, s.gamma, 3)
    for k in ("PPPP", "PPPH"):
        assert _rel(got[k], ref[k]) < 1e-13


REFERENCE_STEPS = """
- name: DefineHolesAndParticles
  in: { fileName: "EigenEnergies.yaml" }
  out: { HoleEigenEnergies: $HoleEigenEnergies, ParticleEigenEnergies: $ParticleEigenEnergies }
- name: Read
  in: { fileName: "CoulombVertex.yaml" }
  out: { destination: $CoulombVertex }
- name: CoulombIntegralsFromVertex
  in:
    CoulombVertex: $CoulombVertex
    HoleEigenEnergies: $HoleEigenEnergies
    ParticleEigenEnergies: $ParticleEigenEnergies
  out:
    PPHHCoulombIntegrals: $PPHHCoulombIntegrals
    PHPHCoulombIntegrals: $PHPHCoulombIntegrals
    HHHHCoulombIntegrals: $HHHHCoulombIntegrals
    HHHPCoulombIntegrals: $HHHPCoulombIntegrals
    PPPPCoulombIntegrals: $PPPPCoulombIntegrals
    PPPHCoulombIntegrals: $PPPHCoulombIntegrals
- name: CcsdEnergyFromCoulombIntegralsReference
  in:
    mixer: DiisMixer
    maxResidua: 4
    maxIterations: 20
    energyConvergence: 1e-8
    amplitudesConvergence: 1e-8
    HoleEigenEnergies: $HoleEigenEnergies
    ParticleEigenEnergies: $ParticleEigenEnergies
    PPHHCoulombIntegrals: $PPHHCoulombIntegrals
    PHPHCoulombIntegrals: $PHPHCoulombIntegrals
    HHHHCoulombIntegrals: $HHHHCoulombIntegrals
    HHHPCoulombIntegrals: $HHHPCoulombIntegrals
    PPPPCoulombIntegrals: $PPPPCoulombIntegrals
    PPPHCoulombIntegrals: $PPPHCoulombIntegrals
  out:
    CcsdEnergy: $CcsdEnergyReference
"""


def test_ueg_golden_through_the_stored_formulation_in_the_runner(tmp_path):
    """The reference's UEG input runs CcsdEnergyFromCoulombIntegralsReference
    on the integrals alone (no vertex); its CCSD energy is the golden one."""
    import json
    import os
    import subprocess

    from oracle.ueg import UEG_GOLDEN, ueg_real_vertex
    from sisi4s_gb300 import build
    build.build()
    runner = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                          "sisi4s_gb300", "_lib", "sisi4s-gb300")
    g = UEG_GOLDEN
    gamma, eh, ep = ueg_real_vertex(g["No"], g["Nv"], g["rs"])
    fermi = 0.5 * (eh.max() + ep.min())
    (tmp_path / "EigenEnergies.yaml").write_text(
        "metaData:\n  fermiEnergy: %.17g\n  energies: [%s]\n"
        % (fermi, ", ".join("%.17g" % e for e in np.concatenate([eh, ep]))))
    NG, Np, _ = gamma.shape
    (tmp_path / "CoulombVertex.yaml").write_text(
        "version: 100\ntype: Tensor\ndimensions:\n"
        "  - length: %d\n    type: AuxiliaryField\n"
        "  - length: %d\n    type: State\n  - length: %d\n    type: State\n"
        "scalarType: Real64\nelements:\n  type: IeeeBinaryFile\nunit: 1.0\n" % (NG, Np, Np))
    gamma.transpose(2, 1, 0).copy().tofile(tmp_path / "CoulombVertex.elements")
    (tmp_path / "in.yaml").write_text(REFERENCE_STEPS)
    r = subprocess.run([runner, "-i", "in.yaml", "-o", "out.yaml"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads((tmp_path / "out.yaml").read_text())
    step = [s for s in out["steps"] if s["name"] == "CcsdEnergyFromCoulombIntegralsReference"][0]
    assert step["convergenceReached"] == 1
    assert abs(step["energy"]["value"] - g["ccsd"]) < 2e-9
