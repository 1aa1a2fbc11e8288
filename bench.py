#!/usr/bin/env python
"""RCCSD(T) on one GB300: the closed-shell CCSD iteration and (T) of sisi4s.

Workload (the headline system): No=32, Nv=256, NG=1024 from the seeded
synthetic generator (sisi4s_gb300/inputs.py, seed 1), 12 iterations from the
MP2 start with DiisMixer(5) and levelShift 16, then (T) on the amplitudes of
the 12th iteration.  A step is one full CCSD iteration (residual, Jacobi
update, DIIS, energy); the MP2-start iteration of each 12-iteration
trajectory is part of its untimed set-up, so a trajectory holds 11 steps.
K steps walk consecutive trajectories: when one ends the solver returns to
the MP2 start (gbcc_ccsd_restart, untimed, keeping the resident integrals
and captured graphs) and the next begins.  Each run of steps inside one
trajectory is bracketed by a barrier and a device synchronisation, timed
with CUDA events on the library stream, and the segment times are summed.

  value         precision-mode iterations/s (contractions emulated in FP64 on
                the bf16 tensor cores; update, DIIS, energies in FP64),
                inputs resident in HBM
  energies      every reported energy states its error against the FP64
                reference energies of this workload (the CPU oracle's 12
                iterations and the FP64 (T), committed fixture)
  fp64          the FP64 GPU path timed on the first full iteration of the
                same trajectory, and its energy against the oracle's
  e2e           gbcc_ccsd_solve from host buffers, as the reference's step
                runs (upload, integrals, MP2 start + 11 iterations, amplitude
                download), iterations/s over the same K steps
  roofline      the dominant kernel (the tensor-core GEMM) timed live with
                CUDA events on the library stream
  cpu_baseline  the CPU oracle (numpy restatement of the reference) on the
                host cores, one full iteration of the same workload

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
Under torchrun each rank runs an independent replica on its own GPU.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SOLVE = {"mixer": "DiisMixer", "max_residua": 5, "level_shift": 16.0,
         "max_iterations": 12, "energy_convergence": 0.0,
         "amplitudes_convergence": 0.0}
TRAJ = SOLVE["max_iterations"]          # iterations per trajectory (incl. MP2 start)
# the headline system (default) and the large one (--workload c5: V_abcd
# would be 134 GB; the ladder is streamed from the vertex)
SYSTEMS = {"c2": {"No": 32, "Nv": 256, "NG": 1024, "seed": 1},
           "c5": {"No": 24, "Nv": 360, "NG": 1440, "seed": 5}}
SYSTEM = SYSTEMS["c2"]
WORKLOAD = None


def select_workload(name):
    global SYSTEM, WORKLOAD
    SYSTEM = SYSTEMS[name]
    WORKLOAD = {"workload": "rccsd_t_no%d_nv%d_ng%d" % (SYSTEM["No"], SYSTEM["Nv"],
                                                         SYSTEM["NG"]),
                **SYSTEM, "mixer": "DiisMixer", "maxResidua": 5, "levelShift": 16.0,
                "maxIterations": TRAJ, "start": "MP2",
                "steps_per_trajectory": TRAJ - 1}


select_workload("c2")
METRIC = "RCCSD iter/s mixed vs FP64 at |dE|<=1uHa; batched solves/s, p50/p99 latency"
UNIT = "iter/s"
REF_MAX_STEPS = 3
FIXTURE = os.path.join(ROOT, "tests", "golden", "c2_trajectory.json")
# DRAM bytes (read + write) per bf16 tensor flop of the emulated GEMM, by
# digits per operand, from one-pass ncu captures of the same kernel on this
# workload (dram__bytes_read.sum + dram__bytes_write.sum of consecutive
# ladder launches, V = G.G at 8192 x 8192 x 1024 and R = V.X at
# 1024 x 1024 x 65536, S(S+1)/2 * 2 * 8192^2 * 1024 bf16 flop each):
# 6 digits, 12 launches, 17.458e9 + 5.292e9 bytes; 5 digits, 24 launches,
# 27.653e9 + 8.671e9 bytes
EMU_GEMM_DRAM_PER_FLOP = {6: (17.458e9 + 5.292e9) / (12 * 21 * 2.0 * 8192 ** 2 * 1024),
                          5: (27.653e9 + 8.671e9) / (24 * 15 * 2.0 * 8192 ** 2 * 1024)}


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


def load_fixture():
    """FP64 reference energies of this workload, or None when the committed
    fixture is missing or describes another workload."""
    try:
        with open(FIXTURE) as f:
            doc = json.load(f)
    except Exception:
        return None
    if doc.get("system") != SYSTEM or doc.get("solve") != SOLVE:
        return None
    return doc


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
        self.shift = SOLVE["level_shift"]
        self.ints = coulomb_integrals(sys_.gamma, sys_.No)
        self.d1, self.d2 = excitation_denominators(sys_.eps_h, sys_.eps_p)
        T1 = np.zeros((sys_.Nv, sys_.No))
        T2 = np.zeros((sys_.Nv, sys_.Nv, sys_.No, sys_.No))
        self.mix = DiisMixer(SOLVE["max_residua"])
        R1, R2 = residual(0, T1, T2, self.ints, sys_.gamma)
        N1, N2 = update_amplitudes(R1, R2, T1, T2, self.d1, self.d2, self.shift)
        self.mix.append((N1, N2), (N1 - T1, N2 - T2))
        self.T1, self.T2 = self.mix.get()
        self.it = 1

    def step(self):
        from oracle.ccsd import energy, residual, update_amplitudes
        t0 = time.perf_counter()
        T1, T2 = self.T1, self.T2
        R1, R2 = residual(self.it, T1, T2, self.ints, self.sys.gamma)
        N1, N2 = update_amplitudes(R1, R2, T1, T2, self.d1, self.d2, self.shift)
        self.mix.append((N1, N2), (N1 - T1, N2 - T2))
        self.T1, self.T2 = self.mix.get()
        e = energy(self.T1, self.T2, self.ints["PPHH"])["value"]
        self.it += 1
        return time.perf_counter() - t0, e


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


class Walker:
    """Walks consecutive 12-iteration trajectories of one resident solver.
    `done` counts iterations of the current trajectory (the MP2 start
    included); a finished trajectory restarts from the MP2 start untimed."""

    def __init__(self, sol, stream, pg):
        self.sol, self.stream, self.pg = sol, stream, pg
        self.done = 0
        self.segments = 0
        self.last_energy = None

    def _begin(self):
        self.sol.restart()
        self.sol.step(1)          # MP2 start: set-up of the trajectory
        self.done = 1

    def walk(self, n, timed):
        import torch
        ms = 0.0
        left = n
        while left > 0:
            if self.done in (0, TRAJ):
                self._begin()
            m = min(left, TRAJ - self.done)
            if timed:
                barrier(self.pg)
                torch.cuda.synchronize()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(self.stream)
                self.last_energy, _ = self.sol.step(m)
                e1.record(self.stream)
                torch.cuda.synchronize()
                barrier(self.pg)
                ms += e0.elapsed_time(e1)
                self.segments += 1
            else:
                self.last_energy, _ = self.sol.step(m)
            self.done += m
            left -= m
        return ms

    def finish(self):
        """Completes the current trajectory (untimed); returns its per-
        iteration energies."""
        if self.done == 0:
            self._begin()
        if self.done < TRAJ:
            self.sol.step(TRAJ - self.done)
            self.done = TRAJ
        return list(self.sol.result(amplitudes=False)["history"])


def _err(ex):
    return "%s: %s" % (type(ex).__name__, ex)


SERVE_OPTS = dict(mixer="DiisMixer", max_residua=5, max_iterations=100,
                  energy_convergence=3e-11, amplitudes_convergence=1e-7)


def serve_measure(args):
    """CCSD(T) serving on samples of the request stream (No ~ U{4..16},
    Nv log-uniform in [20, 160], NG = 4 Nv, request r seeded with r, the C1
    convergence settings): one-at-a-time FP64 and mixed on the first
    `serve_single` requests, and batched with `serve_slots` concurrent
    solves on the first `serve_requests`."""
    from sisi4s_gb300 import autotune, serve
    table = autotune.load()
    reqs = serve.make_requests(max(args.serve_requests, args.serve_single))
    out = {"requests": args.serve_requests, "slots": args.serve_slots,
           "tuning": "none" if table is None else "autotuner table (per shape bucket)",
           "solve": "RCCSD + (T), DIIS(5), energyConvergence 3e-11, "
                    "amplitudesConvergence 1e-7, maxIterations 100"}
    for prec in ("fp64", "emu"):
        srv = serve.Server(slots=1)
        recs, wall = serve.run_stream(srv, reqs[:args.serve_single], lam=None,
                                      precision=prec, tuning=table, **SERVE_OPTS)
        srv.close()
        st = serve.latency_stats(recs, wall)
        out["one_at_a_time_" + prec] = {"requests": args.serve_single,
                                        "solves_per_s": st["solves_per_s"],
                                        "ok_solves_per_s": st["ok_solves_per_s"]}
    lam = args.serve_lambda if args.serve_lambda > 0 else None
    srv = serve.Server(slots=args.serve_slots)
    recs, wall = serve.run_stream(srv, reqs[:args.serve_requests], lam=lam,
                                  precision=args.serve_precision, tuning=table,
                                  **SERVE_OPTS)
    srv.close()
    st = serve.latency_stats(recs, wall)
    st["arrivals"] = ("Poisson, rate %g /s (seed 0)" % lam) if lam else "all at t = 0"
    out["batched_" + args.serve_precision] = st
    out["batched_over_fp64_one_at_a_time"] = (
        st["solves_per_s"] / out["one_at_a_time_fp64"]["solves_per_s"])
    out["batched_precision"] = args.serve_precision
    return out


def run_reference(args, ws, rank, pg):
    """The reference's math on the host cores: the oracle restatement (the
    reference's CTF build cannot be built here), one full iteration of the
    same workload per step."""
    if rank != 0:
        return
    from sisi4s_gb300.inputs import make_system
    threads = os.cpu_count() or 1
    s = make_system(**SYSTEM)
    # the integrals and the MP2-start iteration are built once, untimed (this
    # also warms the BLAS thread pool); at most REF_MAX_STEPS iterations are
    # timed (about a minute each on 16 Grace cores), so that the arm ends
    # within a few minutes for any K
    its = CpuIterations(s, threads)
    n = max(1, min(args.steps, REF_MAX_STEPS))
    times = [its.step()[0] for _ in range(n)]
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
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gbcc", choices=["gbcc", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(SYSTEMS),
                    help="c2: No=32 Nv=256 NG=1024 (default); c5: No=24 Nv=360 NG=1440")
    ap.add_argument("--slices", type=int, default=5,
                    help="bf16 digits per operand in the CCSD iterations (4-8)")
    ap.add_argument("--triples-slices", type=int, default=0,
                    help="bf16 digits per operand in (T) (5-8; 0: one more than --slices)")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-serve", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
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
                    help="skip the (T) correction on the 12th-iteration amplitudes")
    args = ap.parse_args()
    if args.triples_slices <= 0:
        args.triples_slices = min(8, args.slices + 1)
    select_workload(args.workload)
    ws, rank, local, pg = dist_init()
    if args.impl == "reference":
        run_reference(args, ws, rank, pg)
        return

    import torch
    from sisi4s_gb300 import capi
    from sisi4s_gb300 import ccsd as gpu
    from sisi4s_gb300.inputs import make_system

    torch.cuda.set_device(local)
    if args.serve_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "serving": serve_measure(args)}), flush=True)
        return
    s = make_system(**SYSTEM)
    fx = load_fixture()
    ctx = capi.Context(local)
    ctx.set_emulation(args.slices, 1e7)
    stream = torch.cuda.ExternalStream(ctx.stream)
    errors = {}

    # ---- precision mode, inputs resident.  One untimed trajectory captures
    # the steady-state iteration graphs (one per DIIS ring position).
    ctx.pool_high_water(reset=True)
    sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, precision="emu", **SOLVE)
    sol.step(TRAJ)
    Nv = SYSTEM["Nv"]
    memory = {"device_pool_peak_bytes": ctx.pool_high_water(),
              "vabcd_bytes_if_stored": 8 * Nv ** 4,
              "note": "peak of the library's device allocations over setup and one "
                      "12-iteration trajectory; V_abcd is never formed"}
    walker = Walker(sol, stream, pg)
    walker.walk(args.warmup, timed=False)
    l0 = ctx.launches
    f0 = ctx.flops
    with ClockSampler(local) as clk:
        ms = walker.walk(args.steps, timed=True)
    ms = max_over_ranks(pg, ms)
    launches = ctx.launches - l0
    fl = ctx.flops - f0
    value = ws * args.steps / (ms / 1e3)

    # ---- energies of one full trajectory and (T) on its 12th amplitudes,
    # each stated against the FP64 reference energies of this workload
    energies = {"reference": None}
    triples = None
    hist = walker.finish()
    e12 = hist[-1]
    energies["e_ccsd"] = e12
    energies["iterations"] = len(hist)
    if fx is not None and "oracle" in fx:
        ref = [r["energy"] for r in fx["oracle"]["energies"]]
        d = [a - b for a, b in zip(hist, ref)]
        energies.update(reference="CPU oracle (numpy restatement), FP64, 12 iterations",
                        e_ccsd_fp64=ref[-1], dE_ccsd_ha=d[-1],
                        max_abs_dE_ccsd_ha_over_iterations=max(abs(x) for x in d))
    if not args.no_triples:
        try:
            torch.cuda.synchronize()
            t0 = torch.cuda.Event(enable_timing=True)
            t1 = torch.cuda.Event(enable_timing=True)
            # (T) runs with one digit more than the context's setting
            ctx.set_emulation(args.triples_slices - 1, 1e7)
            t0.record(stream)
            e_t, _ = sol.triples("emu")
            t1.record(stream)
            torch.cuda.synchronize()
            ctx.set_emulation(args.slices, 1e7)
            No, Nv, NG = SYSTEM["No"], SYSTEM["Nv"], SYSTEM["NG"]
            f_t = 2.0 * No ** 3 * Nv ** 4 + 2.0 * No ** 4 * Nv ** 3 + 2.0 * NG * No * Nv ** 3
            sec = t0.elapsed_time(t1) / 1e3
            triples = {"seconds": sec, "e_t": e_t, "e_ccsd_t": e12 + e_t,
                       "hole_triples": No * (No + 1) * (No + 2) // 6,
                       "fp64_equiv_tflops": f_t / sec / 1e12,
                       "precision": "emulated fp64 GEMMs (%d bf16 digits), float-float "
                                    "epilogue" % args.triples_slices,
                       "amplitudes": "after the 12th iteration"}
            if fx is not None and "gpu_fp64" in fx:
                g = fx["gpu_fp64"]
                triples.update(e_t_fp64=g["e_t"], dE_t_ha=e_t - g["e_t"],
                               fp64_seconds=g.get("seconds_triples"))
                if energies.get("e_ccsd_fp64") is not None:
                    energies["dE_ccsd_t_ha"] = (e12 + e_t) - (energies["e_ccsd_fp64"] + g["e_t"])
        except Exception as ex:  # noqa: BLE001
            errors["triples"] = _err(ex)

    # ---- roofline of the dominant kernel: two more iterations of a fresh
    # trajectory (eager, profiling on) with CUDA events around every
    # tensor-core GEMM launch
    gs, prof_ms = None, None
    try:
        sol.restart()
        sol.step(1)
        ctx.profile(True)
        p0 = torch.cuda.Event(enable_timing=True)
        p1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        p0.record(stream)
        sol.step(2)
        p1.record(stream)
        torch.cuda.synchronize()
        ctx.profile(False)
        prof_ms = p0.elapsed_time(p1)
        gs = ctx.gemm_stats()
    except Exception as ex:  # noqa: BLE001
        errors["profile"] = _err(ex)
        ctx.profile(False)
    sol.close()

    # ---- FP64 on the GPU: the first full iteration of the same trajectory
    fp64 = None
    if not args.no_fp64:
        try:
            solf = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, precision="fp64", **SOLVE)
            solf.step(1)
            torch.cuda.synchronize()
            f0e = torch.cuda.Event(enable_timing=True)
            f1e = torch.cuda.Event(enable_timing=True)
            f0e.record(stream)
            e_fp64, _ = solf.step(1)
            f1e.record(stream)
            torch.cuda.synchronize()
            solf.close()
            fms = f0e.elapsed_time(f1e)
            fp64 = {"iter_per_s": 1e3 / fms, "iterations_timed": 1,
                    "energy_iteration_2": e_fp64,
                    "mixed_over_fp64": value / ws / (1e3 / fms)}
            if len(hist) >= 2:
                fp64["dE_mixed_vs_fp64_iteration_2_ha"] = hist[1] - e_fp64
            if fx is not None and "oracle" in fx:
                fp64["dE_fp64_vs_oracle_iteration_2_ha"] = (
                    e_fp64 - fx["oracle"]["energies"][1]["energy"])
            if fx is not None and "gpu_fp64" in fx:
                g = fx["gpu_fp64"]
                fp64["trajectory_12_iterations_recorded"] = {
                    "e_ccsd": g["energies"][-1], "e_t": g["e_t"],
                    "seconds_ccsd": g.get("seconds_ccsd"),
                    "seconds_triples": g.get("seconds_triples")}
        except Exception as ex:  # noqa: BLE001
            errors["fp64"] = _err(ex)

    # ---- end to end through the C ABI from host buffers: the reference's
    # step (MP2 start + 11 iterations per solve), as many solves as it takes
    # to cover the K steps; the vertex is staged in page-locked memory first
    e2e = None
    if not args.no_e2e:
        try:
            g_host, g_pin = pinned_copy(s.gamma)
            n_solves = math.ceil(args.steps / (TRAJ - 1))
            wall = 0.0
            done = 0
            h2d = d2h = 0
            No, Nv, NG = SYSTEM["No"], SYSTEM["Nv"], SYSTEM["NG"]
            Np = No + Nv
            for k in range(n_solves):
                n = min(TRAJ - 1, args.steps - done)
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                r = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, g_host, precision="emu",
                                   **dict(SOLVE, max_iterations=n + 1))
                wall += time.perf_counter() - t0
                done += r["iterations"] - 1
                h2d += 8 * (NG * Np * Np + No + Nv)
                d2h += 8 * (Nv * No + Nv * Nv * No * No) + 8 * (n + 1)
            del g_host
            e2e = {"value": ws * done / wall, "unit": UNIT,
                   "h2d_bytes_per_step": h2d // max(done, 1),
                   "d2h_bytes_per_step": d2h // max(done, 1),
                   "host_inputs": "pinned" if g_pin else "pageable",
                   "solves": n_solves,
                   "note": "gbcc_ccsd_solve from host buffers per solve (vertex and "
                           "eigenvalues uploaded, integrals built, MP2 start + "
                           "iterations, amplitudes downloaded), %d full iterations "
                           "in %d solves; bytes per full iteration" % (done, n_solves)}
        except Exception as ex:  # noqa: BLE001
            errors["e2e"] = _err(ex)

    peaks, pk = _peaks()
    roof = None
    if gs is not None and gs["ms"] > 0:
        achieved = gs["tc_flops"] / (gs["ms"] / 1e3) / 1e12
        peak = peaks.get("bf16_tflops")
        roof = {"kernel": "emu_gemm_kernel<%d> (tcgen05 kind::f16)" % args.slices,
                "bound": "tensor", "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": achieved / peak,
                "peak_source": pk + " bf16 burst (MEASURED_PEAKS.json)",
                "launches": gs["launches"],
                "avg_launch_ms": gs["ms"] / max(gs["launches"], 1),
                "fp64_equiv_tflops": gs["fp64_flops"] / (gs["ms"] / 1e3) / 1e12,
                "gemm_share_of_step": gs["ms"] / prof_ms if prof_ms else None,
                "traffic": (EMU_GEMM_DRAM_PER_FLOP[args.slices] * gs["tc_flops"] / gs["launches"]
                            if args.slices in EMU_GEMM_DRAM_PER_FLOP else None),
                "traffic_unit": "bytes per launch",
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of "
                                  "the ladder's launches on this workload, per bf16 flop, "
                                  "scaled to the average launch's work"}

    serving = None
    if not args.no_serve:
        try:
            serving = serve_measure(args)
        except Exception as ex:  # noqa: BLE001
            errors["serving"] = _err(ex)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        try:
            threads = os.cpu_count() or 1
            ct, ce = CpuIterations(s, threads).step()
            cpu = {"value": 1.0 / ct, "unit": UNIT, "cores": threads, "kind": "port",
                   "sample": "one full CCSD iteration (residual, update, DIIS, "
                             "energy) of the numpy restatement on this workload: the "
                             "first after the MP2 start",
                   "energy": ce}
        except Exception as ex:  # noqa: BLE001
            errors["cpu_baseline"] = _err(ex)

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic",
                "config": dict(WORKLOAD, parallelism="replicas" if ws > 1 else "single",
                               precision="emulated fp64, %d bf16 digits (%d in (T))"
                                         % (args.slices, args.triples_slices),
                               l2="inputs larger than L2 (T2, V, Gamma >= 0.5 GB)",
                               timed_segments=walker.segments),
                "energies": energies, "memory": memory, "fp64": fp64, "e2e": e2e,
                "roofline": roof,
                "cpu_baseline": cpu, "serving": serving, "triples": triples,
                "gpu_launches": launches,
                "fp64_equiv_tflops_per_step": fl / (ms / 1e3) / 1e12,
                "clocks": clk.summary()}
        if errors:
            line["errors"] = errors
        print(json.dumps(line), flush=True)
    ctx.close()
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
