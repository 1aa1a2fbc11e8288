"""Serving: many CCSD(T) solves of uneven size on one GPU (gbcc_server_* ABI).

Request stream: for request id r, No ~ U{4..16}, Nv = round(exp(U[ln 20,
ln 160])), NG = 4 Nv, drawn from ``numpy.random.default_rng(r)``; the system
itself is ``make_system(No, Nv, NG, seed=r)``.  Arrivals are a Poisson process
of rate ``lam`` (exponential gaps from ``default_rng(seed)``).
"""
import ctypes as C
import threading
import time

import numpy as np

from . import capi
from .ccsd import CcsdInput, make_opts
from .inputs import make_system

__all__ = ["Server", "request_shape", "make_requests", "run_stream",
           "latency_stats"]


class ServerOpts(C.Structure):
    _fields_ = [("device", C.c_int), ("slots", C.c_int),
                ("hbm_budget_bytes", C.c_int64), ("max_batch", C.c_int)]


class Result(C.Structure):
    _fields_ = [("id", C.c_int64), ("status", C.c_int), ("e_ccsd", C.c_double),
                ("e_t", C.c_double), ("e_total", C.c_double),
                ("iterations", C.c_int), ("converged", C.c_int),
                ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_start", C.c_double), ("t_done", C.c_double)]


_SIGS = {
    "gbcc_server_opts_default": (None, [C.POINTER(ServerOpts)]),
    "gbcc_server_create": (C.c_int, [C.POINTER(ServerOpts), C.POINTER(C.c_void_p)]),
    "gbcc_server_submit": (C.c_int, [C.c_void_p, C.POINTER(capi.CcsdIn),
                                     C.POINTER(capi.CcsdOpts), C.c_int,
                                     C.POINTER(C.c_int64)]),
    "gbcc_server_poll": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(Result),
                                   C.POINTER(C.c_int)]),
    "gbcc_server_wait": (C.c_int, [C.c_void_p, C.c_int64, C.POINTER(Result)]),
    "gbcc_server_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_int),
                                    C.POINTER(C.c_int), C.POINTER(C.c_int64)]),
    "gbcc_server_destroy": (None, [C.c_void_p]),
}


def _lib():
    lib = capi.load()
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def _result_dict(r):
    return {k: getattr(r, k) for k, _ in Result._fields_}


class Server:
    def __init__(self, slots=8, budget_bytes=0, device=0, max_batch=None):
        """``max_batch``: most queued requests of one shape that a slot
        solves together in lockstep (None: the library default, 8; 1: every
        request on its own)."""
        self.lib = _lib()
        o = ServerOpts()
        self.lib.gbcc_server_opts_default(C.byref(o))
        o.device, o.slots, o.hbm_budget_bytes = device, slots, int(budget_bytes)
        if max_batch is not None:
            o.max_batch = int(max_batch)
        h = C.c_void_p()
        st = self.lib.gbcc_server_create(C.byref(o), C.byref(h))
        if st != capi.OK:
            raise capi.GbccError(st, "server creation failed")
        self.h = h

    def submit(self, system, triples=True, tuning=None, **opts):
        """Queues a CCSD(T) solve.  With an autotuner table (``tuning``, see
        ``autotune.load``), the execution settings of the request's shape
        bucket are applied unless ``opts`` sets them."""
        if tuning:
            from .autotune import lookup
            prec = opts.get("precision", "fp64")
            for k, v in lookup(tuning, prec, system.No, system.Nv).items():
                opts.setdefault(k, v)
        inp = CcsdInput(system.eps_h, system.eps_p, system.gamma)
        o = make_opts(**opts)
        rid = C.c_int64()
        st = self.lib.gbcc_server_submit(self.h, C.byref(inp.s), C.byref(o),
                                         1 if triples else 0, C.byref(rid))
        if st != capi.OK:
            raise capi.GbccError(st, "submit failed")
        return rid.value

    def wait(self, rid):
        r = Result()
        st = self.lib.gbcc_server_wait(self.h, rid, C.byref(r))
        if st != capi.OK:
            raise capi.GbccError(st, "wait failed")
        return _result_dict(r)

    def poll(self, rid):
        r = Result()
        done = C.c_int()
        self.lib.gbcc_server_poll(self.h, rid, C.byref(r), C.byref(done))
        return _result_dict(r) if done.value else None

    def stats(self):
        p, r, b = C.c_int(), C.c_int(), C.c_int64()
        self.lib.gbcc_server_stats(self.h, C.byref(p), C.byref(r), C.byref(b))
        return {"pending": p.value, "running": r.value, "bytes_in_use": b.value}

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbcc_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def request_shape(r):
    rng = np.random.default_rng(r)
    No = int(rng.integers(4, 17))
    Nv = int(round(float(np.exp(rng.uniform(np.log(20.0), np.log(160.0))))))
    return No, Nv, 4 * Nv


def make_requests(n, first=0):
    out = []
    for r in range(first, first + n):
        No, Nv, NG = request_shape(r)
        out.append(make_system(No, Nv, NG, seed=r))
    return out


def run_stream(server, systems, lam=None, seed=0, triples=True, tuning=None, **opts):
    """Submit ``systems`` with Poisson arrivals of rate ``lam`` (all at once if
    lam is None), wait for every result, return per-request records.
    ``tuning``: an autotuner table applied to every request."""
    n = len(systems)
    if lam is None:
        gaps = np.zeros(n)
    else:
        gaps = np.random.default_rng(seed).exponential(1.0 / lam, size=n)
    arrivals = np.cumsum(gaps)
    ids = [None] * n
    t_arrive = [0.0] * n
    start = time.perf_counter()

    def submitter():
        for k in range(n):
            delay = start + arrivals[k] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            t_arrive[k] = time.perf_counter()
            ids[k] = server.submit(systems[k], triples=triples, tuning=tuning, **dict(opts))

    th = threading.Thread(target=submitter)
    th.start()
    th.join()
    recs = []
    for k in range(n):
        res = server.wait(ids[k])
        res["latency"] = res["t_done"] - res["t_submit"]
        recs.append(res)
    wall = max(r["t_done"] for r in recs) - min(r["t_submit"] for r in recs)
    return recs, wall


def latency_stats(recs, wall):
    """Throughput and arrival-to-result latency of a stream.  Requests that
    ended with an error status (a singular DIIS matrix, divergence) or
    without converging are served requests too, so ``solves_per_s`` counts
    every one; ``ok_*`` count and time the converged solves (status 0)
    alone, and ``status_counts`` gives the split."""
    lat = np.array([r["latency"] for r in recs])
    ok = np.array([r["latency"] for r in recs if r["status"] == capi.OK])
    counts = {}
    for r in recs:
        counts[capi.status_string(r["status"])] = counts.get(
            capi.status_string(r["status"]), 0) + 1
    out = {"solves": len(recs), "solves_per_s": len(recs) / wall,
           "p50_s": float(np.percentile(lat, 50)),
           "p99_s": float(np.percentile(lat, 99)),
           "mean_s": float(lat.mean()), "wall_s": wall,
           "status_counts": counts, "ok_solves": int(ok.size),
           "ok_solves_per_s": ok.size / wall}
    if ok.size:
        out.update(ok_p50_s=float(np.percentile(ok, 50)),
                   ok_p99_s=float(np.percentile(ok, 99)))
    return out
