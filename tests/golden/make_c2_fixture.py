"""Writes ``c2_trajectory.json``: FP64 reference energies of the headline
workload (No=32, Nv=256, NG=1024, seed 1; MP2 start, DiisMixer with 5
vectors, levelShift 16, 12 iterations), against which the precision form is
gated and the bench states its energy error.

Two parts, each merged into the same file:

``--oracle``   the CPU oracle (numpy restatement of the reference's CTF
               statements) runs the 12 iterations on the host: every
               iteration's energy, direct and exchange terms.  About half an
               hour on 8 cores.
``--gpu-fp64`` the library's FP64 path on a GPU runs the same 12 iterations
               (the check that it follows the oracle at this size) and the
               FP64 (T) on its final amplitudes.  The oracle's literal (T)
               loop is hours at this size on the CPU; the FP64 (T) path it
               is checked against at smaller sizes and on the reference's UEG
               golden energies stands in for it, and the file says so.

    python tests/golden/make_c2_fixture.py --oracle [--out FILE]
    python tests/golden/make_c2_fixture.py --gpu-fp64 [--out FILE]
"""
import argparse
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from tests.golden.cases import C2, C2_SOLVE, C2_FILE  # noqa: E402


def _load(path):
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def _save(path, doc):
    with open(path, "w") as f:
        json.dump(doc, f, indent=1)
        f.write("\n")


def oracle_part():
    from oracle.ccsd import ccsd
    from oracle.coulomb import coulomb_integrals
    from sisi4s_gb300.inputs import make_system

    s = make_system(**C2)
    t0 = time.time()
    ints = coulomb_integrals(s.gamma, s.No)
    hist = []

    def cb(it, amp, en):
        hist.append({"iteration": it + 1, "energy": float(en["value"]),
                     "direct": float(en["direct"]), "exchange": float(en["exchange"]),
                     "seconds": time.time() - t0})
        print(json.dumps(hist[-1]), flush=True)

    r = ccsd(s.eps_h, s.eps_p, ints, s.gamma, callback=cb, **C2_SOLVE)
    return {"what": "CPU oracle (numpy restatement), FP64", "energies": hist,
            "energy": float(r["energy"]), "iterations": int(r["iterations"]),
            "seconds": time.time() - t0}


def gpu_fp64_part():
    from sisi4s_gb300 import capi
    from sisi4s_gb300 import ccsd as gpu
    from sisi4s_gb300.inputs import make_system

    s = make_system(**C2)
    ctx = capi.Context(0)
    t0 = time.time()
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, precision="fp64", **C2_SOLVE)
    es = []
    for _ in range(C2_SOLVE["max_iterations"]):
        e, _ = sol.step(1)
        es.append(e)
    t_ccsd = time.time() - t0
    t0 = time.time()
    e_t, _ = sol.triples("fp64")
    t_t = time.time() - t0
    sol.close()
    ctx.close()
    return {"what": "library FP64 path on a GB300 (CCSD iterations and (T))",
            "energies": es, "e_t": e_t, "e_ccsd_t": es[-1] + e_t,
            "seconds_ccsd": t_ccsd, "seconds_triples": t_t}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--oracle", action="store_true")
    ap.add_argument("--gpu-fp64", action="store_true")
    ap.add_argument("--out", default=C2_FILE)
    args = ap.parse_args()
    doc = _load(args.out)
    doc.update(generator="tests/golden/make_c2_fixture.py", system=C2, solve=C2_SOLVE)
    if args.oracle:
        doc["oracle"] = oracle_part()
        _save(args.out, doc)
    if args.gpu_fp64:
        doc["gpu_fp64"] = gpu_fp64_part()
        _save(args.out, doc)


if __name__ == "__main__":
    main()
