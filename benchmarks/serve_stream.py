"""The serving stream: CCSD(T) requests of uneven size with Poisson arrivals.

    python -m benchmarks.serve_stream [--requests N] [--precision emu|fp64]
        [--lam L | --load X] [--slots S] [--capacity-sample M] [--no-tuning]

Requests r = 0, 1, ... (No ~ U{4..16}, Nv log-uniform in [20, 160], NG = 4 Nv,
request r seeded with r; sisi4s_gb300/serve.py), each a full RCCSD + (T) with
DIIS(5), energyConvergence 3e-11, amplitudesConvergence 1e-7 and
maxIterations 100.  The arrival rate is either given (--lam) or set to
--load times the one-at-a-time FP64 capacity, which is measured first on the
first M requests (one slot, all submitted at once).  The served requests use
the committed autotuner table unless --no-tuning.  Prints one JSON line:
solves/s and arrival-to-result p50/p99, overall and for the converged
solves, with the split of final statuses.
"""
import argparse
import json

SOLVE = dict(mixer="DiisMixer", max_residua=5, max_iterations=100,
             energy_convergence=3e-11, amplitudes_convergence=1e-7)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=512)
    ap.add_argument("--precision", default="emu", choices=["emu", "fp64"])
    ap.add_argument("--lam", type=float, default=0.0)
    ap.add_argument("--load", type=float, default=1.5)
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--capacity-sample", type=int, default=16)
    ap.add_argument("--no-tuning", action="store_true")
    args = ap.parse_args()
    from sisi4s_gb300 import autotune, serve

    table = None if args.no_tuning else autotune.load()
    out = {"requests": args.requests, "precision": args.precision, "slots": args.slots,
           "tuning": "none" if table is None else "autotuner table",
           "solve": "RCCSD + (T), DIIS(5), energyConvergence 3e-11, "
                    "amplitudesConvergence 1e-7, maxIterations 100"}
    lam = args.lam
    if lam <= 0:
        reqs = serve.make_requests(args.capacity_sample)
        srv = serve.Server(slots=1)
        recs, wall = serve.run_stream(srv, reqs, lam=None, precision="fp64",
                                      tuning=table, **SOLVE)
        srv.close()
        cap = serve.latency_stats(recs, wall)["solves_per_s"]
        lam = args.load * cap
        out["fp64_one_at_a_time"] = {"requests": args.capacity_sample,
                                     "solves_per_s": cap}
        out["offered_load"] = "%g x one-at-a-time FP64 capacity" % args.load
    out["lam_per_s"] = lam
    reqs = serve.make_requests(args.requests)
    srv = serve.Server(slots=args.slots)
    recs, wall = serve.run_stream(srv, reqs, lam=lam, precision=args.precision,
                                  tuning=table, **SOLVE)
    srv.close()
    st = serve.latency_stats(recs, wall)
    st["arrivals"] = "Poisson, rate %g /s (seed 0)" % lam
    out["stream"] = st
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
