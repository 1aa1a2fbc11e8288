"""The YAML step runner end to end on the GPU: the reference's UEG integration
test pipeline (DefineHolesAndParticles, Read, CoulombIntegralsFromVertex,
CcsdEnergyFromCoulombIntegrals, CcsdPerturbativeTriples, TensorWriter) must
reproduce the golden CCSD and (T) energies."""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle.ueg import UEG_GOLDEN, ueg_real_vertex

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RUNNER = os.path.join(ROOT, "sisi4s_gb300", "_lib", "sisi4s-gb300")

STEPS = """
- name: Nop
  energyConvergence: &energyConvergence 1e-8
  amplitudesConvergence: &amplitudesConvergence 1e-8
  maxIterations: &maxIterations 20
  mixer: &mixer DiisMixer
  maxResidua: &maxResidua 4

- name: DefineHolesAndParticles
  in:
    fileName: "EigenEnergies.yaml"
  out:
    HoleEigenEnergies: $HoleEigenEnergies
    ParticleEigenEnergies: $ParticleEigenEnergies

- name: Read
  in:
    fileName: "CoulombVertex.yaml"
  out:
    destination: $CoulombVertex

- name: CoulombIntegralsFromVertex
  in:
    CoulombVertex: $CoulombVertex
    HoleEigenEnergies: $HoleEigenEnergies
    ParticleEigenEnergies: $ParticleEigenEnergies
    complex: 0
  out:
    PPHHCoulombIntegrals: $PPHHCoulombIntegrals
    PHPHCoulombIntegrals: $PHPHCoulombIntegrals
    HHHPCoulombIntegrals: $HHHPCoulombIntegrals
    HHHHCoulombIntegrals: $HHHHCoulombIntegrals

- name: CcsdEnergyFromCoulombIntegrals
  in:
    mixer: *mixer
    maxResidua: *maxResidua
    maxIterations: *maxIterations
    energyConvergence: *energyConvergence
    amplitudesConvergence: *amplitudesConvergence
    HoleEigenEnergies: $HoleEigenEnergies
    ParticleEigenEnergies: $ParticleEigenEnergies
    CoulombVertex: $CoulombVertex
    PPHHCoulombIntegrals: $PPHHCoulombIntegrals
    PHPHCoulombIntegrals: $PHPHCoulombIntegrals
    HHHHCoulombIntegrals: $HHHHCoulombIntegrals
    HHHPCoulombIntegrals: $HHHPCoulombIntegrals
  out:
    CcsdEnergy: $CcsdEnergy
    CcsdSinglesAmplitudes: $CcsdSinglesAmplitudes
    CcsdDoublesAmplitudes: $CcsdDoublesAmplitudes
    PairEnergy: $CcsdPairEnergy

- name: CcsdPerturbativeTriples
  in:
    CoulombVertex: $CoulombVertex
    PPHHCoulombIntegrals: $PPHHCoulombIntegrals
    HHHPCoulombIntegrals: $HHHPCoulombIntegrals
    ParticleEigenEnergies: $ParticleEigenEnergies
    HoleEigenEnergies: $HoleEigenEnergies
    CcsdEnergy: $CcsdEnergy
    CcsdSinglesAmplitudes: $CcsdSinglesAmplitudes
    CcsdDoublesAmplitudes: $CcsdDoublesAmplitudes
  out:
    CcsdPerturbativeTriplesEnergy: $CcsdPerturbativeTriplesEnergy

- name: TensorWriter
  in:
    Data: $CcsdPerturbativeTriplesEnergy
  out:
    {}
"""


def test_ueg_pipeline_through_runner(tmp_path):
    from sisi4s_gb300 import build
    build.build()
    g = UEG_GOLDEN
    gamma, eh, ep = ueg_real_vertex(g["No"], g["Nv"], g["rs"])
    energies = np.concatenate([eh, ep])
    fermi = 0.5 * (eh.max() + ep.min())
    (tmp_path / "EigenEnergies.yaml").write_text(
        "metaData:\n  fermiEnergy: %.17g\n  energies: [%s]\n"
        % (fermi, ", ".join("%.17g" % e for e in energies)))
    NG, Np, _ = gamma.shape
    (tmp_path / "CoulombVertex.yaml").write_text(
        "version: 100\ntype: Tensor\ndimensions:\n"
        "  - length: %d\n    type: AuxiliaryField\n"
        "  - length: %d\n    type: State\n  - length: %d\n    type: State\n"
        "scalarType: Real64\nelements:\n  type: IeeeBinaryFile\nunit: 1.0\n"
        % (NG, Np, Np))
    gamma.transpose(2, 1, 0).copy().tofile(tmp_path / "CoulombVertex.elements")
    (tmp_path / "in.yaml").write_text(STEPS)
    r = subprocess.run([RUNNER, "-i", "in.yaml", "-o", "out.yaml"], cwd=tmp_path,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    out = json.loads((tmp_path / "out.yaml").read_text())
    ccsd = [s for s in out["steps"] if s["name"] == "CcsdEnergyFromCoulombIntegrals"][0]
    t = [s for s in out["steps"] if s["name"] == "CcsdPerturbativeTriples"][0]
    assert ccsd["convergenceReached"] == 1
    e_ccsd = ccsd["energy"]["value"]
    assert abs(e_ccsd - g["ccsd"]) < 2e-9
    assert abs(t["energy"]["triples"] - g["triples"]) < 1e-10
    assert abs(t["energy"]["value"] - (e_ccsd + t["energy"]["triples"])) < 1e-14
    # TensorWriter's text format (src/util/TensorIo.cxx:158-226): a name/order
    # line, an index-order line, then the value with 16 significant digits
    lines = open(tmp_path / "CcsdPerturbativeTriplesEnergy.dat").read().split("\n")
    assert lines[0] == "CcsdPerturbativeTriplesEnergy 0"
    written = float(lines[2])
    assert abs(written - t["energy"]["value"]) <= 1e-15 * abs(t["energy"]["value"])
