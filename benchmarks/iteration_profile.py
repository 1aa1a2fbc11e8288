"""One steady-state CCSD iteration inside a profiler range, for kernel captures.

    python -m benchmarks.iteration_profile No Nv NG [--prec emu|fp64]
        [--warmup W] [--slices S] [--graphs 0|1]

Builds a resident solver (MP2 start, DiisMixer(5), levelShift 16), runs W
iterations (the DIIS ring fills after 5), then runs one more iteration
between cudaProfilerStart and cudaProfilerStop, so that
``ncu --profile-from-start off`` captures only that iteration's launches.
Prints one JSON line with the iteration's device time (CUDA events on the
library stream) and the algorithmic bytes of its bandwidth kernels
(update + DIIS + energy, 8 Nv^2 No^2 (3m + 7) with m = 5).
"""
import argparse
import json


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("No", type=int)
    ap.add_argument("Nv", type=int)
    ap.add_argument("NG", type=int)
    ap.add_argument("--prec", default="emu", choices=["emu", "fp64"])
    ap.add_argument("--warmup", type=int, default=6)
    ap.add_argument("--slices", type=int, default=6)
    ap.add_argument("--graphs", type=int, default=1)
    args = ap.parse_args()
    import torch
    from sisi4s_gb300 import capi
    from sisi4s_gb300 import ccsd as gpu
    from sisi4s_gb300.inputs import make_system

    s = make_system(args.No, args.Nv, args.NG, seed=1)
    ctx = capi.Context(0)
    ctx.set_emulation(args.slices, 1e7)
    ctx.set_graphs(bool(args.graphs))
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, precision=args.prec,
                     mixer="DiisMixer", max_residua=5, level_shift=16.0,
                     max_iterations=args.warmup + 1, energy_convergence=0.0,
                     amplitudes_convergence=0.0)
    sol.step(args.warmup)
    stream = torch.cuda.ExternalStream(ctx.stream)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    l0 = ctx.launches
    torch.cuda.profiler.start()
    e0.record(stream)
    e, _ = sol.step(1)
    e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.profiler.stop()
    ms = e0.elapsed_time(e1)
    n2 = args.Nv ** 2 * args.No ** 2
    print(json.dumps({"No": args.No, "Nv": args.Nv, "NG": args.NG, "prec": args.prec,
                      "iteration_ms": ms, "energy": e, "launches": ctx.launches - l0,
                      "bandwidth_kernel_bytes": 8 * n2 * (3 * 5 + 7),
                      "t2_bytes": 8 * n2}), flush=True)
    sol.close()
    ctx.close()


if __name__ == "__main__":
    main()
