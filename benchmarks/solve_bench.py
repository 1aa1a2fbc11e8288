"""Mixed vs FP64 CCSD(T) on one seeded synthetic system.

    python -m benchmarks.solve_bench No Nv NG [--iterations N] [--no-triples]
        [--formulation vertex|stored]

Runs N CCSD iterations (DIIS with 5 vectors, MP2 start) in precision mode and
in FP64 on the GPU, then the (T) correction on each run's final amplitudes in
the same precision, and prints one JSON line: seconds per iteration, the
energies and their differences (Ha), and the (T) times.  The two solvers run
one after the other, so the device holds one system at a time.
"""
import argparse
import json
import time


def run(ctx, s, precision, iterations, triples, triples_fp64=False, formulation="vertex"):
    from sisi4s_gb300 import ccsd as gpu

    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, mixer="DiisMixer", max_residua=5,
                     max_iterations=iterations + 1, energy_convergence=0.0,
                     amplitudes_convergence=0.0, precision=precision,
                     formulation=formulation)
    # step() returns after the host has read the iteration's energy, i.e.
    # after the device finished the iteration
    sol.step(1)  # first iteration (setup, graph capture)
    t0 = time.perf_counter()
    e, _ = sol.step(iterations - 1)
    t_it = (time.perf_counter() - t0) / max(iterations - 1, 1)
    out = {"energy": e, "seconds_per_iteration": t_it}
    if triples:
        t0 = time.perf_counter()
        e_t, _ = sol.triples(precision)
        out.update(e_t=e_t, triples_seconds=time.perf_counter() - t0)
    if triples_fp64:
        # FP64 (T) on these same amplitudes: isolates the error of the (T)
        # emulation from the propagation of CCSD amplitude differences
        t0 = time.perf_counter()
        e_t64, _ = sol.triples("fp64")
        out.update(e_t_fp64_same_amplitudes=e_t64,
                   dE_t_same_amplitudes_ha=out["e_t"] - e_t64,
                   triples_fp64_seconds=time.perf_counter() - t0)
    sol.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("No", type=int)
    ap.add_argument("Nv", type=int)
    ap.add_argument("NG", type=int)
    ap.add_argument("--iterations", type=int, default=3)
    ap.add_argument("--no-triples", action="store_true")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--slices", type=int, default=6,
                    help="bf16 digits per operand in precision mode")
    ap.add_argument("--emu-only", action="store_true",
                    help="skip the FP64 run (compare against a recorded one)")
    ap.add_argument("--triples-fp64-on-emu", action="store_true",
                    help="also run the FP64 (T) on the precision-mode amplitudes")
    ap.add_argument("--formulation", default="vertex", choices=["vertex", "stored"],
                    help="vertex: CcsdEnergyFromCoulombIntegrals; stored: "
                         "CcsdEnergyFromCoulombIntegralsReference (resident Vabcd)")
    args = ap.parse_args()

    from sisi4s_gb300 import capi
    from sisi4s_gb300.inputs import make_system

    s = make_system(args.No, args.Nv, args.NG, args.seed)
    ctx = capi.Context(0)
    ctx.set_emulation(args.slices, 1e7)
    trip = not args.no_triples
    emu = run(ctx, s, "emu", args.iterations, trip, trip and args.triples_fp64_on_emu,
              args.formulation)
    line = {"No": args.No, "Nv": args.Nv, "NG": args.NG, "seed": args.seed,
            "iterations": args.iterations, "mixer": "DiisMixer(5), MP2 start",
            "slices": args.slices, "formulation": args.formulation, "emu": emu}
    if args.emu_only:
        print(json.dumps(line), flush=True)
        ctx.close()
        return
    f64 = run(ctx, s, "fp64", args.iterations, trip, formulation=args.formulation)
    line.update(fp64=f64, dE_ccsd_ha=emu["energy"] - f64["energy"],
                speedup_iteration=f64["seconds_per_iteration"] / emu["seconds_per_iteration"])
    if trip:
        line["dE_t_ha"] = emu["e_t"] - f64["e_t"]
        line["dE_ccsd_t_ha"] = line["dE_ccsd_ha"] + line["dE_t_ha"]
        line["speedup_triples"] = f64["triples_seconds"] / emu["triples_seconds"]
    print(json.dumps(line), flush=True)
    ctx.close()


if __name__ == "__main__":
    main()
