"""Writes the golden fixtures of this folder.

* ``ueg_rs1.0-7occ-26virt.json``: the energies that the reference's UEG
  integration test expects, read as text from
  ``integration-tests/tests/cc4s/ueg/rs1.0-7occ-26virt/cc4s.correct.out.yaml``
  of a sisi4s source tree, each with the line it came from, plus the solver
  settings of that run.  The test's input tensors are downloads that the
  source tree does not hold; ``oracle/ueg.py`` restates the reference's UEG
  vertex generator to rebuild them.
* ``oracle_cases.json``: the oracle's energies on the seeded systems of
  ``cases.py``.

    python tests/golden/make_golden.py --reference SISI4S_TREE [--oracle-only]
"""
import argparse
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

UEG_TEST = "integration-tests/tests/cc4s/ueg/rs1.0-7occ-26virt"


def parse_yaml_maps(text):
    """Nested dicts of a YAML file made of ``key: value`` maps only (the
    shape of the reference's ``*.out.yaml`` records).  Leaves are
    (raw string, line number)."""
    root = {}
    stack = [(-1, root)]
    for n, raw in enumerate(text.splitlines(), 1):
        body = raw.strip()
        if not body or body.startswith("#"):
            continue
        if body.startswith("- "):
            raise ValueError("line %d: lists are not expected here" % n)
        indent = len(raw) - len(raw.lstrip(" "))
        key, sep, val = body.partition(":")
        if not sep:
            raise ValueError("line %d: not a key: value line" % n)
        while stack[-1][0] >= indent:
            stack.pop()
        parent = stack[-1][1]
        val = val.strip()
        if val:
            parent[key.strip()] = (val, n)
        else:
            child = {}
            parent[key.strip()] = child
            stack.append((indent, child))
    return root


def _leaf(v):
    raw, line = v
    return {"value": raw, "line": line}


def ueg_fixture(reference):
    rel = UEG_TEST + "/cc4s.correct.out.yaml"
    with open(os.path.join(reference, rel)) as f:
        doc = parse_yaml_maps(f.read())
    m = re.match(r"rs([0-9.]+)-([0-9]+)occ-([0-9]+)virt$", os.path.basename(UEG_TEST))
    out = {"source": rel, "rs": float(m.group(1)), "No": int(m.group(2)),
           "Nv": int(m.group(3))}
    for step in doc["steps"].values():
        name = step["name"][0]
        if name == "CoupledCluster" and step["in"]["method"][0] == "Ccsd":
            e = step["out"]["energy"]
            out["ccsd"] = {k: _leaf(e[k]) for k in ("correlation", "direct", "exchange",
                                                    "secondOrder")}
            i = step["in"]
            out["ccsd_settings"] = {
                "mixer": _leaf(i["mixer"]["type"]),
                "maxResidua": _leaf(i["mixer"]["maxResidua"]),
                "energyConvergence": _leaf(i["energyConvergence"]),
                "amplitudesConvergence": _leaf(i["amplitudesConvergence"]),
                "maxIterations": _leaf(i["maxIterations"]),
                "convergenceReached": _leaf(step["out"]["convergenceReached"])}
        elif name == "PerturbativeTriplesReference":
            out["triples"] = {"correlation": _leaf(step["out"]["energy"]["correlation"])}
    for k in ("ccsd", "triples"):
        if k not in out:
            raise ValueError("%s: no %s step found" % (rel, k))
    return out


def _pairs(z):
    import numpy as np
    z = np.asarray(z, dtype=np.complex128).ravel()
    return [[float(v.real), float(v.imag)] for v in z]


def oracle_fixture():
    import numpy as np

    from oracle.ccsd import ccsd, mp2_energy
    from oracle.ccsd_complex import ccsd_complex, coulomb_integrals_complex, triples_complex_loop
    from oracle.coulomb import coulomb_integrals
    from oracle.triples import triples_loop
    from tests.golden import cases

    s = cases.real_system()
    ints = coulomb_integrals(s.gamma, s.No, keys=("PPHH", "PHPH", "HHHH", "HHHP",
                                                  "PPPP", "PPPH"))
    real = {"system": cases.REAL, "solve": cases.REAL_SOLVE,
            "mp2": float(mp2_energy(s.eps_h, s.eps_p, ints["PPHH"]))}
    for form, key in (("vertex", "vertex"), ("reference", "stored")):
        r = ccsd(s.eps_h, s.eps_p, ints, s.gamma, formulation=form, **cases.REAL_SOLVE)
        last = r["history"][-1]["energy"]
        rec = {"history": [float(h["energy"]["value"]) for h in r["history"]],
               "direct": float(last["direct"]), "exchange": float(last["exchange"]),
               "t1_sumsq": float(np.sum(r["T1"] ** 2)), "t2_sumsq": float(np.sum(r["T2"] ** 2))}
        if form == "vertex":
            rec["triples"] = float(triples_loop(s.eps_h, s.eps_p, r["T1"], r["T2"],
                                                ints["PPHH"], ints["HHHP"], s.gamma))
        real[key] = rec

    sc, g = cases.complex_system(**cases.COMPLEX)
    ci = coulomb_integrals_complex(g, sc.No)
    r = ccsd_complex(sc.eps_h, sc.eps_p, ci, g, **cases.COMPLEX_SOLVE)
    et = triples_complex_loop(sc.eps_h, sc.eps_p, r["T1"], r["T2"], ci["PPHH"], ci["PHHH"], g)
    cplx = {"system": cases.COMPLEX, "solve": cases.COMPLEX_SOLVE,
            "history": _pairs([h["energy"]["value"] for h in r["history"]]),
            "t2_sumsq": float(np.sum(np.abs(r["T2"]) ** 2)),
            "triples": _pairs([et])[0]}
    return {"generator": "tests/golden/make_golden.py", "real": real, "complex": cplx}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("SISI4S_SOURCE"),
                    help="sisi4s source tree holding the integration tests "
                         "(default: $SISI4S_SOURCE); not needed with --oracle-only")
    ap.add_argument("--oracle-only", action="store_true")
    args = ap.parse_args()
    from tests.golden import cases
    if not args.oracle_only:
        if not args.reference:
            ap.error("--reference (or SISI4S_SOURCE) is required unless --oracle-only")
        with open(cases.UEG_FILE, "w") as f:
            json.dump(ueg_fixture(args.reference), f, indent=1)
            f.write("\n")
    with open(cases.ORACLE_FILE, "w") as f:
        json.dump(oracle_fixture(), f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
