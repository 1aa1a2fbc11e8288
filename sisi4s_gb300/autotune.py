"""Autotuner of the serving layer's execution settings.

A served CCSD(T) request of a given shape runs many small contractions.
Which of them are worth emulating on the tensor cores, and how the FP64 and
emulated GEMMs split K to fill the GPU, depends on the shape.  This module
measures that on the GPU and keeps the answer in a table:

* shapes are bucketed by No (holes) and Nv (particles), three ranges each,
  covering the serving stream's No in 4..16 and Nv in 20..160;
* for each bucket, a seeded system of the bucket's representative shape
  (geometric middle of its ranges, NG = 4 Nv) is iterated with every
  candidate setting (for precision mode: the tensor-core threshold
  emu_min_flops, the FP64 K-split target and the emulated GEMM's K-split
  cap; for FP64 mode: the FP64 K-split target);
* a setting's cost is the time of 40 iterations (the median of timed
  steady-state iterations, after the DIIS ring is full and the iteration
  graphs are captured) plus one (T);
* the cheapest setting of each bucket is kept.

The table lives in ``tuning/gb300_serving.json`` of this package; the server
applies the entry of a request's bucket through the request's options
(``gbcc_ccsd_opts`` execution fields).  Energies do not depend on the choice
beyond rounding.

    python -m sisi4s_gb300.autotune [--out FILE] [--iterations N]
"""
import argparse
import itertools
import json
import math
import os
import time

HERE = os.path.dirname(os.path.abspath(__file__))
TABLE = os.path.join(HERE, "tuning", "gb300_serving.json")

NO_RANGES = [(4, 7), (8, 11), (12, 16)]
NV_RANGES = [(20, 39), (40, 79), (80, 160)]
SOLVE = dict(mixer="DiisMixer", max_residua=5, energy_convergence=0.0,
             amplitudes_convergence=0.0)
ITERATIONS_PER_SOLVE = 40


def candidates(precision):
    """Settings tried for one bucket."""
    if precision == "fp64":
        return [{"f64_split_blocks": b} for b in (0, 1, 2, 3, 6)]
    return [{"emu_min_flops": f, "f64_split_blocks": b, "emu_max_ksplit": k}
            for f, b, k in itertools.product((1e5, 1e6, 1e7, 1e8, 1e10), (0, 1, 3),
                                             (1, 64))]


def representative(lo, hi):
    return int(round(math.sqrt(lo * hi)))


def bucket_of(No, Nv):
    """(i, j) of the No and Nv ranges holding a shape; shapes outside the
    tuned ranges take the nearest one."""
    def idx(x, ranges):
        for k, (lo, hi) in enumerate(ranges):
            if lo <= x <= hi:
                return k
        return 0 if x < ranges[0][0] else len(ranges) - 1
    return idx(No, NO_RANGES), idx(Nv, NV_RANGES)


def lookup(table, precision, No, Nv):
    """The tuned setting for a request (a dict of gbcc_ccsd_opts execution
    fields), or {} when the table has no entry."""
    if not table:
        return {}
    i, j = bucket_of(No, Nv)
    for e in table.get(precision, []):
        if e["bucket"] == [i, j]:
            return dict(e["setting"])
    return {}


def load(path=TABLE):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def measure(ctx, system, precision, setting, warm=6, timed=6):
    """(ms per steady-state iteration, ms of (T)) for one setting."""
    from . import ccsd as gpu
    sol = gpu.Solver(ctx, system.eps_h, system.eps_p, system.gamma, precision=precision,
                     max_iterations=warm + timed, **SOLVE, **setting)
    try:
        sol.step(warm)
        ts = []
        for _ in range(timed):
            t0 = time.perf_counter()
            sol.step(1)  # returns after the host has read the iteration's energy
            ts.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        sol.triples(precision)
        t_t = time.perf_counter() - t0
    finally:
        sol.close()
    ts.sort()
    return 1e3 * ts[len(ts) // 2], 1e3 * t_t


def tune(precisions=("emu", "fp64"), timed=6, log=print):
    from . import capi
    from .inputs import make_system
    ctx = capi.Context(0)
    out = {"how": "per bucket, median steady-state iteration time x %d + one (T), "
                  "cheapest setting kept" % ITERATIONS_PER_SOLVE,
           "no_ranges": NO_RANGES, "nv_ranges": NV_RANGES}
    try:
        for prec in precisions:
            rows = []
            for i, (nlo, nhi) in enumerate(NO_RANGES):
                for j, (vlo, vhi) in enumerate(NV_RANGES):
                    No, Nv = representative(nlo, nhi), representative(vlo, vhi)
                    s = make_system(No, Nv, 4 * Nv, seed=1000 + 10 * i + j)
                    best = None
                    tried = []
                    for setting in candidates(prec):
                        it_ms, t_ms = measure(ctx, s, prec, setting, timed=timed)
                        cost = ITERATIONS_PER_SOLVE * it_ms + t_ms
                        tried.append({"setting": setting, "iteration_ms": it_ms,
                                      "triples_ms": t_ms, "cost_ms": cost})
                        if best is None or cost < best["cost_ms"]:
                            best = tried[-1]
                    default = tried[0]["cost_ms"]
                    for t in tried:
                        if t["setting"] == {"f64_split_blocks": 3} or t["setting"] == {
                                "emu_min_flops": 1e7, "f64_split_blocks": 3,
                                "emu_max_ksplit": 64}:
                            default = t["cost_ms"]
                    rows.append({"bucket": [i, j], "No": No, "Nv": Nv,
                                 "setting": best["setting"],
                                 "cost_ms": best["cost_ms"],
                                 "default_cost_ms": default,
                                 "tried": tried})
                    log(json.dumps({"precision": prec, "No": No, "Nv": Nv,
                                    "best": best["setting"], "cost_ms": best["cost_ms"],
                                    "default_cost_ms": default}))
            out[prec] = rows
    finally:
        ctx.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=TABLE)
    ap.add_argument("--iterations", type=int, default=6,
                    help="timed steady-state iterations per setting")
    args = ap.parse_args()
    table = tune(timed=args.iterations)
    os.makedirs(os.path.dirname(os.path.abspath(args.out)), exist_ok=True)
    with open(args.out, "w") as f:
        json.dump(table, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
