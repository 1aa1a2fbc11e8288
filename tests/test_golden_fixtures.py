"""The committed golden fixtures of ``tests/golden/`` (CPU).

``ueg_rs1.0-7occ-26virt.json`` holds the energies that the reference's UEG
integration test expects, read by ``tests/golden/make_golden.py`` from that
test's record (``cc4s.correct.out.yaml``).  The oracle's pinned constants must
be exactly those values.  ``oracle_cases.json`` holds the oracle's energies on
the seeded systems of ``tests/golden/cases.py``; the oracle must still
reproduce them, to round-off, since BLAS summation order may differ between
machines.
"""
import numpy as np
import pytest

from oracle.ccsd import ccsd, mp2_energy
from oracle.ccsd_complex import ccsd_complex, coulomb_integrals_complex, triples_complex_loop
from oracle.coulomb import coulomb_integrals
from oracle.triples import triples_loop
from oracle.ueg import UEG_GOLDEN
from tests.golden import cases
from tests.golden.make_golden import parse_yaml_maps


@pytest.fixture(scope="module")
def ueg():
    return cases.load(cases.UEG_FILE)


@pytest.fixture(scope="module")
def fx():
    return cases.load(cases.ORACLE_FILE)


def test_ueg_fixture_is_the_oracle_pin(ueg):
    assert (ueg["No"], ueg["Nv"], ueg["rs"]) == (UEG_GOLDEN["No"], UEG_GOLDEN["Nv"],
                                                  UEG_GOLDEN["rs"])
    assert float(ueg["ccsd"]["secondOrder"]["value"]) == UEG_GOLDEN["mp2"]
    assert float(ueg["ccsd"]["correlation"]["value"]) == UEG_GOLDEN["ccsd"]
    assert float(ueg["triples"]["correlation"]["value"]) == UEG_GOLDEN["triples"]
    st, mine = ueg["ccsd_settings"], UEG_GOLDEN["ccsd_settings"]
    assert st["mixer"]["value"] == mine["mixer"]
    assert int(st["maxResidua"]["value"]) == mine["max_residua"]
    assert float(st["energyConvergence"]["value"]) == mine["energy_convergence"]
    assert float(st["amplitudesConvergence"]["value"]) == mine["amplitudes_convergence"]
    assert int(st["maxIterations"]["value"]) == mine["max_iterations"]
    assert st["convergenceReached"]["value"] == "1"
    # direct + exchange = correlation in the record itself
    d = float(ueg["ccsd"]["direct"]["value"])
    x = float(ueg["ccsd"]["exchange"]["value"])
    assert abs(d + x - UEG_GOLDEN["ccsd"]) < 1e-15


def test_record_parser():
    doc = parse_yaml_maps("steps:\n  6:\n    in:\n      mixer:\n        maxResidua: 4\n"
                          "    name: CoupledCluster\n    out:\n      energy:\n"
                          "        correlation: -0.5\n  7:\n    name: X\nversion: v\n")
    assert doc["steps"]["6"]["in"]["mixer"]["maxResidua"] == ("4", 5)
    assert doc["steps"]["6"]["name"] == ("CoupledCluster", 6)
    assert doc["steps"]["6"]["out"]["energy"]["correlation"] == ("-0.5", 9)
    assert doc["steps"]["7"]["name"] == ("X", 11)
    assert doc["version"] == ("v", 12)
    with pytest.raises(ValueError):
        parse_yaml_maps("a:\n  - 1\n")


def _close(a, b, rel):
    a, b = np.asarray(a), np.asarray(b)
    return np.abs(a - b).max() <= rel * np.abs(b).max()


def test_oracle_reproduces_the_real_cases(fx):
    f = fx["real"]
    assert f["system"] == cases.REAL and f["solve"] == cases.REAL_SOLVE
    s = cases.real_system()
    ints = coulomb_integrals(s.gamma, s.No, keys=("PPHH", "PHPH", "HHHH", "HHHP",
                                                  "PPPP", "PPPH"))
    assert _close(mp2_energy(s.eps_h, s.eps_p, ints["PPHH"]), f["mp2"], 1e-13)
    for form, key in (("vertex", "vertex"), ("reference", "stored")):
        r = ccsd(s.eps_h, s.eps_p, ints, s.gamma, formulation=form, **cases.REAL_SOLVE)
        g = f[key]
        assert r["iterations"] == len(g["history"]) == cases.REAL_SOLVE["max_iterations"]
        assert _close([h["energy"]["value"] for h in r["history"]], g["history"], 1e-12)
        last = r["history"][-1]["energy"]
        assert _close(last["direct"], g["direct"], 1e-12)
        assert _close(last["exchange"], g["exchange"], 1e-12)
        assert _close(np.sum(r["T2"] ** 2), g["t2_sumsq"], 1e-11)
        if key == "vertex":
            et = triples_loop(s.eps_h, s.eps_p, r["T1"], r["T2"], ints["PPHH"],
                              ints["HHHP"], s.gamma)
            assert _close(et, g["triples"], 1e-11)


def test_the_two_recorded_formulations_agree(fx):
    """Gamma-ladder and stored-Vabcd residuals give the same trajectory."""
    v, st = fx["real"]["vertex"], fx["real"]["stored"]
    assert _close(v["history"], st["history"], 1e-13)
    assert _close(v["t2_sumsq"], st["t2_sumsq"], 1e-12)


def test_oracle_reproduces_the_complex_case(fx):
    f = fx["complex"]
    assert f["system"] == cases.COMPLEX and f["solve"] == cases.COMPLEX_SOLVE
    s, g = cases.complex_system(**cases.COMPLEX)
    ci = coulomb_integrals_complex(g, s.No)
    r = ccsd_complex(s.eps_h, s.eps_p, ci, g, **cases.COMPLEX_SOLVE)
    h = np.array([x["energy"]["value"] for x in r["history"]])
    assert _close(h, cases.complex_list(f["history"]), 1e-12)
    et = triples_complex_loop(s.eps_h, s.eps_p, r["T1"], r["T2"], ci["PPHH"], ci["PHHH"], g)
    assert _close(et, cases.complex_list([f["triples"]])[0], 1e-11)
    # the vertex is a unitary rotation of a real one: the energies are real
    assert np.abs(cases.complex_list(f["history"]).imag).max() < 1e-15


def test_c2_fixture_first_iteration_from_the_oracle():
    """The headline workload's fixture (c2_trajectory.json): its first
    energy is the MP2-start iteration with the level shift, T2 = -V/(D + s)
    (update_amplitudes with T = 0; a one-vector DIIS returns the estimate),
    recomputed here from the generator in a few seconds; and its FP64 GPU
    trajectory follows the oracle's."""
    from oracle.ccsd import energy, excitation_denominators
    from sisi4s_gb300.inputs import make_system
    doc = cases.load(cases.C2_FILE)
    assert doc["system"] == cases.C2 and doc["solve"] == cases.C2_SOLVE
    s = make_system(**cases.C2)
    gai = np.ascontiguousarray(s.gamma[:, s.No:, :s.No])
    NG, Nv, No = gai.shape
    g2 = gai.reshape(NG, Nv * No)
    V = (g2.T @ g2).reshape(Nv, No, Nv, No).transpose(0, 2, 1, 3)
    _, d2 = excitation_denominators(s.eps_h, s.eps_p)
    T2 = -V / (d2 + cases.C2_SOLVE["level_shift"])
    e = energy(np.zeros((Nv, No)), T2, V)["value"]
    ref = doc["oracle"]["energies"]
    assert len(ref) == cases.C2_SOLVE["max_iterations"]
    assert abs(e - ref[0]["energy"]) < 1e-8
    fp = doc["gpu_fp64"]["energies"]
    assert max(abs(a - b["energy"]) for a, b in zip(fp, ref)) <= 1e-8
