"""Serving requests that share one shape: lockstep batches against solves
that only run side by side.

    python -m benchmarks.serve_same_shape [--shape No,Nv] [--requests N]
        [--precision emu|fp64] [--slots S] [--max-batch B] [--no-triples]

N requests of one shape (NG = 4 Nv), request r a system of the serving
stream's generator seeded with 2000 + r, all submitted at once (saturation),
each a full RCCSD (+ (T)) with DIIS(5), energyConvergence 3e-11,
amplitudesConvergence 1e-7, maxIterations 100.  Runs the same requests
three times:
- one at a time (one slot, no batching);
- side by side (S slots, each request on its own stream);
- in lockstep batches (S slots, a slot taking up to B queued requests of
  the shape at once).
Prints one JSON line: solves/s and p50/p99 latency of each, and the largest
energy difference between the batched and the one-at-a-time results.
"""
import argparse
import json

SOLVE = dict(mixer="DiisMixer", max_residua=5, max_iterations=100,
             energy_convergence=3e-11, amplitudes_convergence=1e-7)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--shape", default="6,40")
    ap.add_argument("--requests", type=int, default=64)
    ap.add_argument("--precision", default="emu", choices=["emu", "fp64"])
    ap.add_argument("--slots", type=int, default=8)
    ap.add_argument("--max-batch", type=int, default=8)
    ap.add_argument("--no-triples", action="store_true")
    args = ap.parse_args()
    from sisi4s_gb300 import serve
    from sisi4s_gb300.inputs import make_system

    No, Nv = (int(x) for x in args.shape.split(","))
    systems = [make_system(No, Nv, 4 * Nv, seed=2000 + r) for r in range(args.requests)]
    triples = not args.no_triples
    out = {"shape": {"No": No, "Nv": Nv, "NG": 4 * Nv}, "requests": args.requests,
           "precision": args.precision, "triples": triples,
           "arrivals": "all at t = 0",
           "solve": "RCCSD%s, DIIS(5), energyConvergence 3e-11, amplitudesConvergence 1e-7, "
                    "maxIterations 100" % (" + (T)" if triples else "")}
    runs = {}
    for name, slots, mb in (("one_at_a_time", 1, 1), ("side_by_side", args.slots, 1),
                            ("lockstep_batches", args.slots, args.max_batch)):
        # warm-up on two requests (module loading, graph instantiation paths)
        srv = serve.Server(slots=slots, max_batch=mb)
        serve.run_stream(srv, systems[:2], lam=None, triples=triples,
                         precision=args.precision, **SOLVE)
        srv.close()
        srv = serve.Server(slots=slots, max_batch=mb)
        recs, wall = serve.run_stream(srv, systems, lam=None, triples=triples,
                                      precision=args.precision, **SOLVE)
        srv.close()
        st = serve.latency_stats(recs, wall)
        st["slots"], st["max_batch"] = slots, mb
        runs[name] = (st, recs)
        out[name] = st
    # records come in submission order
    de = 0.0
    for r, b in zip(runs["lockstep_batches"][1], runs["one_at_a_time"][1]):
        if r["status"] == b["status"] == 0:
            de = max(de, abs(r["e_total"] - b["e_total"]))
    out["max_abs_dE_total_batched_vs_alone_ha"] = de
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
