#!/usr/bin/env python
"""RCCSD iteration throughput on GB300 (closed-shell CCSD of sisi4s).

Workload: No=32, Nv=256, NG=1024 (seeded synthetic vertex, see
sisi4s_gb300/inputs.py), MP2 start, DIIS with 5 vectors.  A step is one CCSD
iteration (residual, Jacobi update, DIIS, energy).

  value      mixed-precision iterations/s (contractions emulated in FP64 on
             the bf16 tensor cores; update, DIIS, energies in FP64), inputs
             resident in HBM
  fp64       the same iterations all in FP64 on the GPU, and dE between the
             two energies after the same number of iterations
  e2e        gbcc_ccsd_solve from host buffers (uploads, integral build,
             iterations, amplitude download) in iterations/s
  roofline   the dominant kernel (the tensor-core GEMM) timed live with CUDA
             events on the library stream
  cpu_baseline  the CPU oracle (numpy restatement of the reference) on the
             host cores, one full iteration of the same workload

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun each rank runs an independent replica on its own GPU.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {"workload": "rccsd_no32_nv256_ng1024", "No": 32, "Nv": 256,
            "NG": 1024, "seed": 1, "mixer": "DiisMixer", "maxResidua": 5}
METRIC = "RCCSD iter/s mixed vs FP64 at |dE|<=1uHa; batched solves/s, p50/p99 latency"
UNIT = "iter/s"
REF_MAX_STEPS = 3


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0,
                "bf16_tflops_sustained": 1700.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.rows = []
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.p = None
        return self

    def _read(self):
        for line in self.p.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        import statistics
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        reasons = []
        for k, n in enumerate(names):
            if any(len(r) >= 9 and r[5 + k].lower().startswith("active") for r in self.rows):
                reasons.append(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo")
        pg = dist
    return ws, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class CpuIterations:
    """CCSD iterations of the CPU oracle on one system (residual, update,
    DIIS, energy): the integrals and the MP2-start iteration are built once,
    untimed; every step() times the next full iteration."""

    def __init__(self, sys_, threads):
        os.environ["OMP_NUM_THREADS"] = str(threads)
        from oracle.ccsd import excitation_denominators, residual, update_amplitudes
        from oracle.coulomb import coulomb_integrals
        from oracle.mixers import DiisMixer
        import numpy as np
        self.sys = sys_
        self.ints = coulomb_integrals(sys_.gamma, sys_.No)
        self.d1, self.d2 = excitation_denominators(sys_.eps_h, sys_.eps_p)
        T1 = np.zeros((sys_.Nv, sys_.No))
        T2 = np.zeros((sys_.Nv, sys_.Nv, sys_.No, sys_.No))
        self.mix = DiisMixer(5)
        R1, R2 = residual(0, T1, T2, self.ints, sys_.gamma)
        N1, N2 = update_amplitudes(R1, R2, T1, T2, self.d1, self.d2)
        self.mix.append((N1, N2), (N1 - T1, N2 - T2))
        self.T1, self.T2 = self.mix.get()
        self.it = 1

    def step(self):
        from oracle.ccsd import energy, residual, update_amplitudes
        t0 = time.perf_counter()
        T1, T2 = self.T1, self.T2
        R1, R2 = residual(self.it, T1, T2, self.ints, self.sys.gamma)
        N1, N2 = update_amplitudes(R1, R2, T1, T2, self.d1, self.d2)
        self.mix.append((N1, N2), (N1 - T1, N2 - T2))
        self.T1, self.T2 = self.mix.get()
        energy(self.T1, self.T2, self.ints["PPHH"])
        self.it += 1
        return time.perf_counter() - t0


def pinned_copy(a):
    """(copy of ``a`` in page-locked host memory with the same shape and
    memory order, True), or (``a``, False) where pinning is unavailable."""
    import numpy as np
    try:
        import torch
        buf = torch.empty(a.size, dtype=torch.float64, pin_memory=True).numpy()
    except Exception:
        return a, False
    v = buf.reshape(a.shape[::-1]).T if a.flags.f_contiguous else buf.reshape(a.shape)
    np.copyto(v, a)
    return v, True


def cpu_iteration_time(sys_, threads):
    """One C2 iteration of the CPU oracle (residual, update, DIIS, energy)."""
    return CpuIterations(sys_, threads).step()


SERVE_OPTS = dict(mixer="DiisMixer", max_residua=5, max_iterations=100,
                  energy_convergence=3e-11, amplitudes_convergence=1e-7)


def serve_measure(args):
    """CCSD(T) serving on samples of the request stream (No ~ U{4..16},
    Nv log-uniform in [20, 160], NG = 4 Nv, request r seeded with r, the C1
    convergence settings): one-at-a-time FP64 and mixed on the first
    `serve_single` requests, and batched mixed with `serve_slots` concurrent
    solves on the first `serve_requests`, all submitted at t = 0 (saturated)."""
    from sisi4s_gb300 import serve
    reqs = serve.make_requests(max(args.serve_requests, args.serve_single))
    out = {"requests": args.serve_requests, "slots": args.serve_slots,
           "solve": "RCCSD + (T), DIIS(5), energyConvergence 3e-11, "
                    "amplitudesConvergence 1e-7, maxIterations 100"}
    for prec in ("fp64", "emu"):
        srv = serve.Server(slots=1)
        recs, wall = serve.run_stream(srv, reqs[:args.serve_single], lam=None,
                                      precision=prec, **SERVE_OPTS)
        srv.close()
        st = serve.latency_stats(recs, wall)
        out["one_at_a_time_" + prec] = {"requests": args.serve_single,
                                        "solves_per_s": st["solves_per_s"]}
    lam = args.serve_lambda if args.serve_lambda > 0 else None
    srv = serve.Server(slots=args.serve_slots)
    recs, wall = serve.run_stream(srv, reqs[:args.serve_requests], lam=lam,
                                  precision=args.serve_precision, **SERVE_OPTS)
    srv.close()
    st = serve.latency_stats(recs, wall)
    st["arrivals"] = ("Poisson, rate %g /s (seed 0)" % lam) if lam else "all at t = 0"
    out["batched_" + args.serve_precision] = st
    out["status_counts"] = {str(k): sum(1 for r in recs if r["status"] == k)
                            for k in sorted(set(r["status"] for r in recs))}
    out["batched_over_fp64_one_at_a_time"] = (
        st["solves_per_s"] / out["one_at_a_time_fp64"]["solves_per_s"])
    out["batched_precision"] = args.serve_precision
    return out


def run_reference(args, ws, rank, pg):
    """The reference's math on the host cores: the oracle restatement (the
    reference's CTF build cannot be built here), one C2 iteration per step."""
    if rank != 0:
        return
    from sisi4s_gb300.inputs import make_system
    threads = os.cpu_count() or 1
    s = make_system(WORKLOAD["No"], WORKLOAD["Nv"], WORKLOAD["NG"], WORKLOAD["seed"])
    # the integrals and the MP2-start iteration are built once, untimed (this
    # also warms the BLAS thread pool); each step times the next full CCSD
    # iteration, so the run stays within a few minutes for small K
    # at most REF_MAX_STEPS iterations are timed (about a minute each on 16
    # Grace cores), so that the arm ends within a few minutes for any K
    its = CpuIterations(s, threads)
    n = max(1, min(args.steps, REF_MAX_STEPS))
    times = [its.step() for _ in range(n)]
    t = sum(times)
    v = n / t
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": UNIT,
            "n_gpus": ws, "steps": n, "steps_requested": args.steps,
            "warmup": args.warmup,
            "ms_per_step": 1e3 * t / n, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": dict(WORKLOAD, parallelism="replicas"),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads,
                             "kind": "port",
                             "sample": "per step, the next full CCSD iteration "
                                       "(residual, update, DIIS, energy) of the numpy "
                                       "restatement; integrals and the MP2-start "
                                       "iteration built once, untimed; at most %d "
                                       "steps timed" % REF_MAX_STEPS},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gbcc", choices=["gbcc", "reference"])
    ap.add_argument("--slices", type=int, default=6)
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--serve-requests", type=int, default=32)
    ap.add_argument("--serve-single", type=int, default=4)
    ap.add_argument("--serve-slots", type=int, default=8)
    ap.add_argument("--serve-lambda", type=float, default=0.0,
                    help="Poisson arrival rate of the batched serving run "
                         "(0: all requests at t = 0)")
    ap.add_argument("--serve-precision", default="emu", choices=["emu", "fp64"],
                    help="precision of the batched serving run")
    ap.add_argument("--serve-only", action="store_true",
                    help="run only the serving measurement (one JSON line)")
    ap.add_argument("--no-triples", action="store_true",
                    help="skip the (T) correction on the final amplitudes")
    ap.add_argument("--triples-fp64", action="store_true",
                    help="also run the FP64 (T) for dE_(T) (minutes at the default size)")
    args = ap.parse_args()
    ws, rank, local, pg = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank, pg)
        return

    import numpy as np
    import torch
    from sisi4s_gb300 import capi
    from sisi4s_gb300 import ccsd as gpu
    from sisi4s_gb300.inputs import make_system

    torch.cuda.set_device(local)
    if args.serve_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "serving": serve_measure(args)}), flush=True)
        return
    W = WORKLOAD
    s = make_system(W["No"], W["Nv"], W["NG"], W["seed"])
    ctx = capi.Context(local)
    ctx.set_emulation(args.slices, 1e7)
    stream = torch.cuda.ExternalStream(ctx.stream)
    total_it = args.warmup + args.steps
    kw = dict(mixer=W["mixer"], max_residua=W["maxResidua"],
              max_iterations=total_it + 1, energy_convergence=0.0,
              amplitudes_convergence=0.0)

    # ---- mixed precision, inputs resident (steady-state iterations replay
    # captured CUDA graphs)
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, precision="emu",
                     **dict(kw, max_iterations=total_it + 2))
    sol.step(args.warmup)
    barrier(pg)
    torch.cuda.synchronize()
    l0 = ctx.launches
    f0 = ctx.flops
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        e_mixed, _ = sol.step(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    barrier(pg)
    ms = max_over_ranks(pg, ms)
    launches = ctx.launches - l0
    fl = ctx.flops - f0
    # roofline of the dominant kernel: two more (untimed) steps with CUDA
    # events around every tensor-core GEMM launch (graphs off while profiling)
    ctx.profile(True)
    p0 = torch.cuda.Event(enable_timing=True)
    p1 = torch.cuda.Event(enable_timing=True)
    p0.record(stream)
    sol.step(2)
    p1.record(stream)
    torch.cuda.synchronize()
    ctx.profile(False)
    prof_ms = p0.elapsed_time(p1)
    gs = ctx.gemm_stats()

    # ---- (T) on the final amplitudes: precision mode, optionally FP64
    triples = None
    if not args.no_triples:
        No = W["No"]
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e_t, _ = sol.triples("emu")
        t_emu = time.perf_counter() - t0
        triples = {"seconds": t_emu, "e_t": e_t,
                   "hole_triples": No * (No + 1) * (No + 2) // 6,
                   "precision": "emulated fp64 GEMMs (%d bf16 digits), float-float "
                                "epilogue" % min(8, args.slices + 1),
                   "amplitudes": "after %d iterations" % (total_it + 2)}
        if args.triples_fp64:
            t0 = time.perf_counter()
            e_t64, _ = sol.triples("fp64")
            t64 = time.perf_counter() - t0
            triples.update(fp64_seconds=t64, e_t_fp64=e_t64, dE_t_ha=e_t - e_t64,
                           speedup=t64 / t_emu)
    sol.close()
    value = ws * args.steps / (ms / 1e3)

    # ---- FP64 on the GPU, same iterations (for dE and the speed-up)
    fp64 = None
    if not args.no_fp64:
        solf = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, precision="fp64", **kw)
        solf.step(args.warmup + args.steps - 1)
        torch.cuda.synchronize()
        f0e = torch.cuda.Event(enable_timing=True)
        f1e = torch.cuda.Event(enable_timing=True)
        f0e.record(stream)
        e_fp64, _ = solf.step(1)
        f1e.record(stream)
        torch.cuda.synchronize()
        solf.close()
        fms = f0e.elapsed_time(f1e)
        fp64 = {"iter_per_s": 1e3 / fms, "energy": e_fp64,
                "energy_mixed": e_mixed, "dE_ha": e_mixed - e_fp64,
                "dE_rel": (e_mixed - e_fp64) / abs(e_fp64) if e_fp64 else None,
                "mixed_over_fp64": (1e3 / (ms / args.steps)) / (1e3 / fms),
                "iterations_compared": total_it}

    # ---- end to end through the C ABI from host buffers
    # start from given amplitudes (the MP2 amplitudes) so that every timed
    # iteration is a full CCSD iteration, as in the resident measurement
    from sisi4s_gb300.inputs import mp2_amplitudes
    t1_0, t2_0 = mp2_amplitudes(s)
    # the large inputs (vertex, starting doubles) are staged in page-locked
    # host memory before the clock starts; the column-major views pass
    # through the Python API without a copy
    g_host, g_pin = pinned_copy(s.gamma)
    t2_host, t2_pin = pinned_copy(t2_0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, g_host, precision="emu",
                       initial=(t1_0, t2_host), **dict(kw, max_iterations=args.steps))
    e2e_s = time.perf_counter() - t0
    del g_host, t2_host  # hand the page-locked staging back
    Np = W["No"] + W["Nv"]
    n2 = W["Nv"] ** 2 * W["No"] ** 2
    h2d = 8 * (W["NG"] * Np * Np + W["No"] + W["Nv"] + W["Nv"] * W["No"] + n2)
    d2h = 8 * (W["Nv"] * W["No"] + n2) + 8 * 4
    e2e = {"value": ws * r["iterations"] / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": h2d // args.steps,
           "d2h_bytes_per_step": d2h // args.steps,
           "host_inputs": "pinned" if (g_pin and t2_pin) else "pageable",
           "note": "one gbcc_ccsd_solve of %d full iterations from host "
                   "buffers (vertex, eigenvalues and starting amplitudes "
                   "uploaded, integrals built, amplitudes downloaded inside); "
                   "bytes per iteration" % args.steps}

    peaks, pk = _peaks()
    achieved = gs["tc_flops"] / (gs["ms"] / 1e3) / 1e12 if gs["ms"] > 0 else None
    peak = peaks.get("bf16_tflops")
    roof = {"kernel": "emu_gemm_kernel<%d> (tcgen05 kind::f16)" % args.slices,
            "bound": "tensor", "achieved": achieved, "peak": peak,
            "unit": "TFLOP/s", "frac": achieved / peak if achieved else None,
            "peak_source": pk + " bf16 burst (MEASURED_PEAKS.json)",
            "launches": gs["launches"],
            "avg_launch_ms": gs["ms"] / max(gs["launches"], 1),
            "fp64_equiv_tflops": gs["fp64_flops"] / (gs["ms"] / 1e3) / 1e12 if gs["ms"] else None,
            "gemm_share_of_step": gs["ms"] / prof_ms if prof_ms else None}
    # DRAM traffic per launch: the ncu capture of the same kernel at M=N=K=4096
    # (profiles/emu_gemm_4096.md: dram read + write = 1.942 + 0.153 GB for
    # 21 * 2 * 4096^3 bf16 flop), scaled to this run's average launch by its
    # algorithmic work (the panel re-reads grow with M*N*K for fixed tiles)
    if gs["launches"]:
        per_flop = (1.942e9 + 0.153e9) / (21 * 2.0 * 4096 ** 3)
        roof["traffic"] = per_flop * gs["tc_flops"] / gs["launches"]
        roof["traffic_unit"] = "bytes per launch"
        roof["traffic_source"] = ("ncu dram__bytes_read.sum + dram__bytes_write.sum at "
                                  "4096^3, scaled by work per launch")
    else:
        roof["traffic"] = None

    serving = None
    if not args.no_serve:
        serving = serve_measure(args)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        ct = cpu_iteration_time(s, threads)
        cpu = {"value": 1.0 / ct, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "one full CCSD iteration (residual, update, DIIS, "
                         "energy) of the numpy restatement on this workload"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": dict(W, parallelism="replicas" if ws > 1 else "single",
                               precision="emulated fp64, %d bf16 digits" % args.slices,
                               l2="inputs larger than L2 (T2, V, Gamma >= 0.5 GB)"),
                "fp64": fp64, "e2e": e2e, "roofline": roof, "cpu_baseline": cpu,
                "serving": serving, "triples": triples,
                "gpu_launches": launches,
                "fp64_equiv_tflops_per_step": fl / args.steps / (ms / args.steps / 1e3) / 1e12,
                "clocks": clk.summary()}
        print(json.dumps(line), flush=True)
    ctx.close()
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
