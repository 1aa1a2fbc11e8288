"""Serving layer on the GPU: continuous admission, overlap, and results that
are the same alone and in a mix."""
import numpy as np
import pytest

from sisi4s_gb300 import serve
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu

OPTS = dict(mixer="DiisMixer", max_residua=5, max_iterations=30,
            energy_convergence=3e-11, amplitudes_convergence=1e-7)


@pytest.mark.parametrize("precision", ["fp64", "emu"])
def test_alone_equals_in_mix(precision):
    target = make_system(6, 30, 120, seed=11)
    alone = serve.Server(slots=1)
    rid = alone.submit(target, precision=precision, **OPTS)
    ref = alone.wait(rid)
    alone.close()
    assert ref["status"] in (0, 1)
    mix = serve.Server(slots=6)
    others = serve.make_requests(10, first=100)
    ids = [mix.submit(s, precision=precision, **OPTS) for s in others[:5]]
    tid = mix.submit(target, precision=precision, **OPTS)
    ids += [mix.submit(s, precision=precision, **OPTS) for s in others[5:]]
    got = mix.wait(tid)
    rest = [mix.wait(i) for i in ids]
    mix.close()
    # deterministic kernels: bit-identical energies alone and in the mix
    assert got["e_ccsd"] == ref["e_ccsd"]
    assert got["e_t"] == ref["e_t"]
    assert got["iterations"] == ref["iterations"]
    assert all(r["status"] in (0, 1) for r in rest)


def test_requests_overlap_and_admission_respects_budget():
    systems = serve.make_requests(12, first=0)
    srv = serve.Server(slots=4, budget_bytes=8 << 30)
    recs, wall = serve.run_stream(srv, systems, lam=None, triples=False,
                                  precision="emu", **OPTS)
    srv.close()
    assert len(recs) == 12 and all(r["status"] in (0, 1) for r in recs)
    # with four slots some solves must have run at the same time
    spans = sorted((r["t_start"], r["t_done"]) for r in recs)
    overlap = any(spans[k + 1][0] < spans[k][1] for k in range(len(spans) - 1))
    assert overlap
    st = serve.latency_stats(recs, wall)
    assert st["solves_per_s"] > 0 and st["p99_s"] >= st["p50_s"]


def test_serving_result_matches_direct_solve(ctx):
    from sisi4s_gb300 import ccsd as gpu
    s = make_system(5, 24, 96, seed=3)
    direct = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **OPTS)
    et, _ = gpu.triples(ctx, s.eps_h, s.eps_p, s.gamma, direct["T1"], direct["T2"])
    srv = serve.Server(slots=2)
    r = srv.wait(srv.submit(s, **OPTS))
    srv.close()
    assert r["e_ccsd"] == direct["energy"]
    assert abs(r["e_t"] - et) < 1e-12 * max(1.0, abs(et))
    assert np.isfinite(r["e_total"])
