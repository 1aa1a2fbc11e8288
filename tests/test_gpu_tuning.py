"""Execution settings carried by the solve options (GPU), and the serving
autotuner's table applied to served requests.

The settings choose where contractions run (tensor-core emulation or FP64)
and how GEMMs split K; energies must not depend on them beyond rounding, and
a tuned request must give the same bits alone and in a mix.
"""
import numpy as np
import pytest

from sisi4s_gb300 import autotune, serve
from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu

KW = dict(mixer="DiisMixer", max_residua=5, max_iterations=8, energy_convergence=0.0,
          amplitudes_convergence=0.0)


def test_threshold_in_the_options_reaches_the_context(ctx):
    # precision mode with every contraction below the threshold is the FP64 path
    s = make_system(5, 30, 80, seed=51)
    try:
        emu = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, precision="emu",
                             emu_min_flops=1e18, **KW)
        f64 = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, precision="fp64", **KW)
    finally:
        ctx.set_emulation(6, 1e7)
    assert np.array_equal(emu["history"], f64["history"])
    assert np.array_equal(emu["T2"], f64["T2"])


@pytest.mark.parametrize("precision", ["fp64", "emu"])
def test_split_settings_change_rounding_only(ctx, precision):
    s = make_system(6, 40, 120, seed=52)
    out = []
    try:
        for blocks, ks in ((0, 1), (1, 64), (6, 64)):
            out.append(gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, precision=precision,
                                      emu_min_flops=1e5, f64_split_blocks=blocks,
                                      emu_max_ksplit=ks, **KW))
    finally:
        ctx.set_emulation(6, 1e7)
        ctx.set_splits(3, 64)
    for r in out[1:]:
        assert np.abs(np.asarray(r["history"]) - out[0]["history"]).max() < 1e-10


@pytest.mark.parametrize("precision", ["fp64", "emu"])
def test_tuned_request_alone_equals_in_mix(precision):
    table = autotune.load()
    assert table and precision in table, "the committed autotuner table is missing"
    opts = dict(KW, max_iterations=20)
    target = make_system(9, 50, 200, seed=53)
    alone = serve.Server(slots=1)
    ref = alone.wait(alone.submit(target, precision=precision, tuning=table, **opts))
    alone.close()
    mix = serve.Server(slots=6)
    others = serve.make_requests(8, first=200)
    ids = [mix.submit(s, precision=precision, tuning=table, **opts) for s in others[:4]]
    tid = mix.submit(target, precision=precision, tuning=table, **opts)
    ids += [mix.submit(s, precision=precision, tuning=table, **opts) for s in others[4:]]
    got = mix.wait(tid)
    for i in ids:
        mix.wait(i)
    mix.close()
    assert got["e_ccsd"] == ref["e_ccsd"] and got["e_t"] == ref["e_t"]
