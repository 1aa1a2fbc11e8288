"""Times one (T) evaluation on a seeded synthetic system.

    python -m benchmarks.triples_bench No Nv NG [--prec emu|fp64] [--reps R]
        [--batch-images B]

The amplitudes are the MP2 amplitudes of the system (T1 = 0) plus a small
seeded T1, so that every term of the (T) energy is exercised.  Prints one JSON
line with the wall time of each repetition and E_(T).
"""
import argparse
import json
import time

import numpy as np


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("No", type=int)
    ap.add_argument("Nv", type=int)
    ap.add_argument("NG", type=int)
    ap.add_argument("--prec", default="emu", choices=["emu", "fp64"])
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--profile", action="store_true",
                    help="CUDA events around every tensor-core launch of the last "
                         "repetition: time of the W products by kind, the rest is "
                         "the epilogue and set-up")
    ap.add_argument("--batch-images", type=int, default=0,
                    help="bound on the triple images per (T) batch (0: automatic)")
    args = ap.parse_args()

    import torch  # device synchronisation only

    from sisi4s_gb300 import capi
    from sisi4s_gb300 import ccsd as gpu
    from sisi4s_gb300.inputs import make_system, mp2_amplitudes

    s = make_system(args.No, args.Nv, args.NG, args.seed)
    T1, T2 = mp2_amplitudes(s)
    T1 = T1 + 1e-3 * np.random.default_rng(args.seed + 1).normal(size=T1.shape)
    ctx = capi.Context(0)
    ctx.set_triples_batch(args.batch_images)
    times, e_t = [], None
    for rep in range(args.reps):
        if args.profile and rep == args.reps - 1:
            ctx.profile(True)
            ctx.gemm_records()  # drop older records
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e_t, _ = gpu.triples(ctx, s.eps_h, s.eps_p, s.gamma, T1, T2,
                             precision=args.prec)
        times.append(time.perf_counter() - t0)
    out = {"No": args.No, "Nv": args.Nv, "NG": args.NG,
           "precision": args.prec, "seconds": times, "e_t": e_t,
           "hole_triples": args.No * (args.No + 1) * (args.No + 2) // 6}
    if args.profile:
        ctx.profile(False)
        recs = ctx.gemm_records()
        Nv = args.Nv
        hole = lambda r: r[0] == Nv * Nv and r[1] == Nv
        part = lambda r: r[0] == Nv and r[1] == Nv * Nv
        kinds = {"hole (M = Nv^2, N = Nv, K = No)": hole,
                 "particle (M = Nv, N = Nv^2, K = Nv)": part,
                 "other (Wvv and integral builds)": lambda r: not hole(r) and not part(r)}
        for name, sel in kinds.items():
            rr = [r for r in recs if sel(r)]
            out["gemm_" + name] = {"launches": len(rr), "ms": sum(r[3] for r in rr)}
        out["gemm_ms_total"] = sum(r[3] for r in recs)
        out["rest_ms"] = 1e3 * times[-1] - out["gemm_ms_total"]
    print(json.dumps(out))
    ctx.close()


if __name__ == "__main__":
    main()
