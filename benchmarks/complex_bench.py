"""Complex (k-point) CCSD(T) on one seeded synthetic complex system.

    python -m benchmarks.complex_bench No Nv NG [--iterations N] [--no-triples]

The vertex is the seeded real synthetic one with its rows mixed by a random
unitary and random orbital phases, so every quantity is genuinely complex.
Runs N linear-mixer iterations (the reference has no complex DIIS) in
precision mode and in FP64, then the complex (T) on each run's amplitudes,
and prints one JSON line: seconds per iteration (from the difference of an
N- and a 1-iteration solve, so that setup cancels), the energies and their
differences.
"""
import argparse
import json
import time

import numpy as np


def complex_system(No, Nv, NG, seed):
    from sisi4s_gb300.inputs import make_system
    s = make_system(No, Nv, NG, seed)
    rng = np.random.default_rng(seed + 1000)
    W, _ = np.linalg.qr(rng.normal(size=(NG, NG)) + 1j * rng.normal(size=(NG, NG)))
    ph = np.exp(1j * rng.uniform(0, 2 * np.pi, No + Nv))
    g = np.einsum("GH,Hpq->Gpq", W, np.conj(ph)[None, :, None] * s.gamma * ph[None, None, :])
    return s.eps_h, s.eps_p, g


def run(ctx, eh, ep, g, precision, iterations, triples):
    from sisi4s_gb300 import ccsd as gpu
    kw = dict(max_iterations=iterations, energy_convergence=0.0, amplitudes_convergence=0.0,
              precision=precision)
    t0 = time.perf_counter()
    gpu.ccsd_solve_complex(ctx, eh, ep, g, **dict(kw, max_iterations=1))
    t1 = time.perf_counter()
    r = gpu.ccsd_solve_complex(ctx, eh, ep, g, **kw)
    t2 = time.perf_counter()
    out = {"energy": [r["energy"].real, r["energy"].imag],
           "seconds_per_iteration": ((t2 - t1) - (t1 - t0)) / max(iterations - 1, 1)}
    if triples:
        t0 = time.perf_counter()
        et, _ = gpu.triples_complex(ctx, eh, ep, g, r["T1"], r["T2"], precision=precision)
        out.update(e_t=[et.real, et.imag], triples_seconds=time.perf_counter() - t0)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("No", type=int)
    ap.add_argument("Nv", type=int)
    ap.add_argument("NG", type=int)
    ap.add_argument("--iterations", type=int, default=4)
    ap.add_argument("--no-triples", action="store_true")
    ap.add_argument("--seed", type=int, default=1)
    args = ap.parse_args()

    from sisi4s_gb300 import capi

    eh, ep, g = complex_system(args.No, args.Nv, args.NG, args.seed)
    ctx = capi.Context(0)
    trip = not args.no_triples
    emu = run(ctx, eh, ep, g, "emu", args.iterations, trip)
    f64 = run(ctx, eh, ep, g, "fp64", args.iterations, trip)
    line = {"No": args.No, "Nv": args.Nv, "NG": args.NG, "seed": args.seed,
            "iterations": args.iterations, "mixer": "LinearMixer, MP2 start",
            "emu": emu, "fp64": f64,
            "dE_ccsd_ha": emu["energy"][0] - f64["energy"][0],
            "speedup_iteration": f64["seconds_per_iteration"] / emu["seconds_per_iteration"]}
    if trip:
        line["dE_t_ha"] = emu["e_t"][0] - f64["e_t"][0]
    print(json.dumps(line), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
