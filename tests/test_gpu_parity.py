"""CUDA path vs the oracle, through the C ABI (GPU)."""
import ctypes as C

import numpy as np
import pytest

from oracle.ccsd import ccsd as oracle_ccsd
from oracle.ccsd import energy as oracle_energy
from oracle.ccsd import residual as oracle_residual
from oracle.coulomb import coulomb_integrals as oracle_ints
from oracle.triples import triples_dense
from oracle.ueg import UEG_GOLDEN, ueg_real_vertex
from sisi4s_gb300 import capi
from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

pytestmark = pytest.mark.gpu

# FP64 tolerances.  Contractions are summed in a different order than numpy,
# so results agree to round-off: relative 1e-12 on residual elements and
# 1e-10 Ha on energies (the parity gate of the FP64 path).
RTOL_RES = 1e-12
ETOL = 1e-10


def _rand_amplitudes(Nv, No, seed, scale=0.02):
    rng = np.random.default_rng(seed)
    T1 = rng.normal(0, scale, (Nv, No))
    T2 = rng.normal(0, scale, (Nv, Nv, No, No))
    return T1, 0.5 * (T2 + T2.transpose(1, 0, 3, 2))


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)


def test_dgemm_all_transposes(ctx):
    import torch  # device memory plumbing only
    rng = np.random.default_rng(0)
    for (ta, tb, M, N, K) in [(0, 0, 70, 33, 19), (1, 0, 64, 64, 64),
                              (0, 1, 5, 130, 7), (1, 1, 129, 1, 300),
                              (0, 0, 1, 1, 1000)]:
        A = rng.normal(size=(K, M) if ta else (M, K))
        B = rng.normal(size=(N, K) if tb else (K, N))
        Cm = rng.normal(size=(M, N))
        ref = 0.7 * ((A.T if ta else A) @ (B.T if tb else B)) - 0.3 * Cm
        dA = torch.tensor(A.T.copy().ravel(), device="cuda")  # column-major
        dB = torch.tensor(B.T.copy().ravel(), device="cuda")
        dC = torch.tensor(Cm.T.copy().ravel(), device="cuda")
        torch.cuda.synchronize()
        lda = A.shape[0]
        ldb = B.shape[0]
        ctx.check(ctx.lib.gbcc_dgemm(ctx.h, ta, tb, M, N, K, 0.7, dA.data_ptr(),
                                     lda, dB.data_ptr(), ldb, -0.3,
                                     dC.data_ptr(), M, capi.PREC_FP64))
        torch.cuda.synchronize()  # device-wide: also waits for the context stream
        got = dC.cpu().numpy().reshape(N, M).T
        assert np.abs(got - ref).max() < 1e-12 * max(1, np.abs(ref).max()) * np.sqrt(K)


@pytest.mark.parametrize("prec", [capi.PREC_FP64, capi.PREC_EMU])
def test_matrix_vector_products(ctx, prec):
    # M = 1 or N = 1 runs as a deterministic FP64 GEMV in both precision
    # modes, with either operand layout and the ldc stride of a row result
    import torch  # device memory plumbing only
    rng = np.random.default_rng(4)
    cases = [(0, 0, 3000, 1, 5000), (1, 0, 3000, 1, 5000), (0, 1, 2500, 1, 700),
             (1, 1, 17, 1, 20000), (0, 0, 1, 3000, 4000), (1, 0, 1, 2999, 4001),
             (0, 1, 1, 1500, 9000), (1, 1, 1, 64, 33), (0, 0, 1, 1, 70000)]
    for (ta, tb, M, N, K) in cases:
        A = rng.normal(size=(K, M) if ta else (M, K))
        B = rng.normal(size=(N, K) if tb else (K, N))
        ldc = M + 3 if M == 1 else M
        Cfull = rng.normal(size=(ldc, N))
        ref = 0.7 * ((A.T if ta else A) @ (B.T if tb else B)) - 0.3 * Cfull[:M]
        dA = torch.tensor(A.T.copy().ravel(), device="cuda")
        dB = torch.tensor(B.T.copy().ravel(), device="cuda")
        dC = torch.tensor(Cfull.T.copy().ravel(), device="cuda")
        torch.cuda.synchronize()
        ctx.set_emulation(6, 0.0)
        ctx.check(ctx.lib.gbcc_dgemm(ctx.h, ta, tb, M, N, K, 0.7, dA.data_ptr(),
                                     A.shape[0], dB.data_ptr(), B.shape[0], -0.3,
                                     dC.data_ptr(), ldc, prec))
        torch.cuda.synchronize()
        ctx.set_emulation(6, 1e7)
        got_full = dC.cpu().numpy().reshape(N, ldc).T
        got = got_full[:M]
        scale = np.abs(A).max() * np.abs(B).max() * K
        assert np.abs(got - ref).max() < 1e-14 * scale, (ta, tb, M, N, K)
        assert np.array_equal(got_full[M:], Cfull[M:])  # padding rows untouched


def test_coulomb_integrals_match_oracle(ctx):
    s = make_system(6, 20, 48, seed=5)
    got = gpu.coulomb_integrals(ctx, s.gamma, 6)
    ref = oracle_ints(s.gamma, 6, keys=("PPHH", "PHPH", "HHHH", "HHHP", "HHPP"))
    for k in ("PPHH", "PHPH", "HHHH", "HHHP", "HHPP"):
        assert _rel(got[k], ref[k]) < 1e-13, k


@pytest.mark.parametrize("No,Nv,NG,dist,ppl,slice_size", [
    (4, 12, 30, 0, 1, -1),
    (5, 17, 41, 0, 1, 5),     # reference default slicing (No), ragged last slice
    (5, 17, 41, 1, 1, 3),     # distinguishable
    (3, 9, 20, 0, 0, -1),     # ppl = 0
    (1, 3, 5, 0, 1, 1),       # minimal sizes
])
def test_residual_matches_oracle(ctx, No, Nv, NG, dist, ppl, slice_size):
    s = make_system(No, Nv, NG, seed=No * 100 + Nv)
    ints = oracle_ints(s.gamma, No)
    T1, T2 = _rand_amplitudes(Nv, No, seed=Nv)
    r1, r2 = oracle_residual(1, T1, T2, ints, s.gamma, distinguishable=dist,
                             ppl=ppl, slice_size=slice_size)
    g1, g2 = gpu.ccsd_residual(ctx, 1, T1, T2, s.eps_h, s.eps_p, s.gamma,
                               distinguishable=dist, ppl=ppl,
                               slice_size=slice_size)
    assert _rel(g1, r1) < RTOL_RES
    assert _rel(g2, r2) < RTOL_RES


@pytest.mark.parametrize("No,Nv,NG,slice_size,dist", [(4, 23, 50, 5, 0), (3, 40, 64, 16, 0),
                                                      (5, 30, 70, 30, 1), (2, 9, 20, 4, 0),
                                                      (2, 40, 600, 10, 0), (3, 32, 64, 5, 0),
                                                      (4, 48, 96, 16, 0), (2, 64, 600, 24, 1),
                                                      (3, 40, 64, 5, 0), (2, 24, 50, 7, 1)])
def test_residual_emulated_matches_oracle(ctx, No, Nv, NG, slice_size, dist):
    # every GEMM emulated (threshold 0), ragged ladder slices: the ladder's
    # V_xycd is written by the emulated GEMM straight into its permuted layout
    # (with NG = 600 over two K-chunks and few tiles, through the K-split
    # reduction).  With Nv a multiple of 8 the ladder takes its fused form:
    # V_xycd goes straight into the digit panels of R = V.X, with row
    # exponents bounded from the vertex column norms (Nv = 32 with slices of
    # 5: blocks of 25 rows, panel rows padded; Nv = 48: whole 128-row tiles;
    # Nv = 64: two K-chunks over NG, distinguishable; Nv = 40 and 24 with
    # odd slices: product widths that end half-way through a 16-column group)
    s = make_system(No, Nv, NG, seed=No * 7 + Nv)
    ints = oracle_ints(s.gamma, No)
    T1, T2 = _rand_amplitudes(Nv, No, seed=Nv + 1)
    r1, r2 = oracle_residual(1, T1, T2, ints, s.gamma, distinguishable=dist,
                             slice_size=slice_size)
    ctx.set_emulation(6, 0.0)
    try:
        g1, g2 = gpu.ccsd_residual(ctx, 1, T1, T2, s.eps_h, s.eps_p, s.gamma,
                                   distinguishable=dist, slice_size=slice_size,
                                   precision="emu")
    finally:
        ctx.set_emulation(6, 1e7)
    # six bf16 digits: ~2^-42 K relative to the operand scales per product
    assert _rel(g1, r1) < 1e-10
    assert _rel(g2, r2) < 1e-10


def test_mp2_start_is_exact(ctx):
    s = make_system(4, 12, 30, seed=1)
    ints = oracle_ints(s.gamma, 4)
    T1, T2 = _rand_amplitudes(12, 4, seed=0)
    g1, g2 = gpu.ccsd_residual(ctx, 0, T1, T2, s.eps_h, s.eps_p, s.gamma,
                               ints=ints)
    assert np.array_equal(g2, ints["PPHH"]) and not g1.any()


def test_energy_matches_oracle(ctx):
    s = make_system(5, 15, 40, seed=2)
    r = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, max_iterations=3)
    ints = oracle_ints(s.gamma, 5)
    e = oracle_energy(r["T1"], r["T2"], ints["PPHH"])
    assert abs(e["value"] - r["energy"]) < 1e-12 * abs(e["value"])


@pytest.mark.parametrize("mixer,ratio", [("LinearMixer", 1.0),
                                         ("LinearMixer", 0.7),
                                         ("DiisMixer", 1.0)])
def test_iterations_match_oracle(ctx, mixer, ratio):
    s = make_system(4, 14, 36, seed=8)
    ints = oracle_ints(s.gamma, 4)
    kw = dict(mixer=mixer, mixing_ratio=ratio, max_residua=3,
              max_iterations=12, energy_convergence=1e-12,
              amplitudes_convergence=1e-9)
    ref = oracle_ccsd(s.eps_h, s.eps_p, ints, s.gamma, **kw)
    got = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    refh = [h["energy"]["value"] for h in ref["history"]]
    assert got["iterations"] == ref["iterations"]
    assert np.abs(np.array(got["history"]) - np.array(refh)).max() < ETOL
    assert _rel(got["T2"], ref["T2"]) < 1e-9


def test_c1_config_parity(ctx):
    """No=10, Nv=50, NG=300, MP2 start, DIIS(5), energyConvergence 3e-11,
    amplitudesConvergence 1e-7, maxIterations 100: same iteration count and
    |E_GPU - E_oracle| <= 1e-10 Ha at every iteration."""
    s = make_system(10, 50, 300, seed=1)
    ints = oracle_ints(s.gamma, 10)
    kw = dict(mixer="DiisMixer", max_residua=5, max_iterations=100,
              energy_convergence=3e-11, amplitudes_convergence=1e-7)
    ref = oracle_ccsd(s.eps_h, s.eps_p, ints, s.gamma, **kw)
    got = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    refh = np.array([h["energy"]["value"] for h in ref["history"]])
    assert got["iterations"] == ref["iterations"]
    assert got["converged"] == ref["converged"]
    assert np.abs(np.array(got["history"]) - refh).max() < ETOL
    assert abs(got["energy"] - ref["energy"]) < ETOL


def test_ueg_golden_through_gpu(ctx):
    """The reference golden CCSD and (T) energies reproduced on the GPU."""
    g = UEG_GOLDEN
    gamma, eh, ep = ueg_real_vertex(g["No"], g["Nv"], g["rs"])
    r = gpu.ccsd_solve(ctx, eh, ep, gamma, **g["ccsd_settings"])
    assert r["converged"]
    assert abs(r["energy"] - g["ccsd"]) < 2e-9
    et, etot = gpu.triples(ctx, eh, ep, gamma, r["T1"], r["T2"],
                           e_ccsd=r["energy"])
    assert abs(et - g["triples"]) < 1e-10
    assert abs(etot - (r["energy"] + et)) < 1e-15


@pytest.mark.parametrize("No,Nv,NG", [(3, 8, 20), (4, 11, 25), (1, 4, 6)])
def test_triples_match_oracle(ctx, No, Nv, NG):
    s = make_system(No, Nv, NG, seed=No + Nv)
    ints = oracle_ints(s.gamma, No)
    T1, T2 = _rand_amplitudes(Nv, No, seed=3, scale=0.05)
    ref = triples_dense(s.eps_h, s.eps_p, T1, T2, ints["PPHH"], ints["HHHP"],
                        s.gamma)
    et, _ = gpu.triples(ctx, s.eps_h, s.eps_p, s.gamma, T1, T2)
    assert abs(et - ref) < 1e-12 * max(1.0, abs(ref))


def test_complex_vertex_is_rejected(ctx):
    s = make_system(2, 4, 6, seed=1)
    inp = gpu.CcsdInput(s.eps_h, s.eps_p, s.gamma)
    im = np.zeros(s.gamma.size)
    im[3] = 1e-3
    inp.s.gamma_imag = capi.ptr(im)
    o = gpu.make_opts()
    out = capi.CcsdOut()
    st = ctx.lib.gbcc_ccsd_solve(ctx.h, C.byref(inp.s), C.byref(o), C.byref(out))
    assert st == capi.COMPLEX_UNSUPPORTED


def test_deterministic_bits(ctx):
    s = make_system(4, 12, 30, seed=6)
    kw = dict(mixer="DiisMixer", max_iterations=6)
    a = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    b = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    assert a["energy"] == b["energy"] and np.array_equal(a["T2"], b["T2"])


@pytest.mark.parametrize("mixer,precision", [("DiisMixer", "fp64"),
                                             ("DiisMixer", "emu"),
                                             ("LinearMixer", "fp64")])
def test_graph_replay_equals_eager(ctx, mixer, precision):
    """Steady-state iterations replayed from captured CUDA graphs give the
    same bits as eager execution."""
    s = make_system(4, 20, 60, seed=9)
    kw = dict(mixer=mixer, max_residua=3, mixing_ratio=0.8, max_iterations=10,
              energy_convergence=0.0, amplitudes_convergence=0.0,
              precision=precision)
    ctx.set_emulation(6, 1e4)
    ctx.set_graphs(False)
    eager = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    ctx.set_graphs(True)
    graph = gpu.ccsd_solve(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
    ctx.set_emulation(6, 1e7)
    assert np.array_equal(eager["history"], graph["history"])
    assert np.array_equal(eager["T2"], graph["T2"])


@pytest.mark.parametrize("No,Nv,NG", [(3, 8, 20), (4, 40, 90)])
def test_triples_emulated_matches_oracle(ctx, No, Nv, NG):
    s = make_system(No, Nv, NG, seed=No + Nv)
    ints = oracle_ints(s.gamma, No)
    T1, T2 = _rand_amplitudes(Nv, No, seed=3, scale=0.05)
    ref = triples_dense(s.eps_h, s.eps_p, T1, T2, ints["PPHH"], ints["HHHP"],
                        s.gamma)
    et, _ = gpu.triples(ctx, s.eps_h, s.eps_p, s.gamma, T1, T2, precision="emu")
    # six bf16 digits: ~2^-40 relative per contraction
    assert abs(et - ref) < 1e-10 * max(1.0, abs(ref))



@pytest.mark.parametrize("precision", ["fp64", "emu"])
def test_triples_batching_does_not_change_the_bits(ctx, precision):
    """(T) runs its hole triples in batches (grouped W products, one epilogue
    launch per batch); every batch size gives the same energy, bit for bit:
    one triple per batch, batches that end inside the i <= j <= k order at
    varying points, and the automatic size (all triples of this system in one
    batch).  Checked against the oracle as well."""
    No, Nv, NG = 5, 24, 60
    s = make_system(No, Nv, NG, seed=41)
    ints = oracle_ints(s.gamma, No)
    T1, T2 = _rand_amplitudes(Nv, No, seed=4, scale=0.05)
    ref = triples_dense(s.eps_h, s.eps_p, T1, T2, ints["PPHH"], ints["HHHP"], s.gamma)
    ctx.set_emulation(6, 0.0)
    got = []
    try:
        for images in (6, 7, 13, 0):
            ctx.set_triples_batch(images)
            got.append(gpu.triples(ctx, s.eps_h, s.eps_p, s.gamma, T1, T2,
                                   precision=precision)[0])
    finally:
        ctx.set_triples_batch(0)
        ctx.set_emulation(6, 1e7)
    assert got.count(got[0]) == len(got), got
    tol = 1e-12 if precision == "fp64" else 1e-10
    assert abs(got[0] - ref) < tol * max(1.0, abs(ref))


@pytest.mark.parametrize("mixer", ["DiisMixer", "LinearMixer"])
def test_operand_cache_gives_the_same_bits(ctx, mixer):
    """Precision mode keeps the digit panels of the integrals and vertex blocks
    (constant for a solve) instead of splitting them in every iteration; the
    iterations, captured graphs included, give the same bits with and without
    the cache, and so does (T)."""
    s = make_system(4, 32, 90, seed=61)
    kw = dict(mixer=mixer, max_residua=3, mixing_ratio=0.8, max_iterations=8,
              energy_convergence=0.0, amplitudes_convergence=0.0, precision="emu")
    ctx.set_emulation(6, 1e4)
    out = []
    try:
        for enable in (False, True):
            ctx.set_operand_cache(enable)
            sol = gpu.Solver(ctx, s.eps_h, s.eps_p, s.gamma, **kw)
            try:
                sol.step(8)
                r = sol.result()
                r["et"] = sol.triples("emu")[0]
            finally:
                sol.close()
            out.append(r)
    finally:
        ctx.set_operand_cache(True)
        ctx.set_emulation(6, 1e7)
    assert np.array_equal(out[0]["history"], out[1]["history"])
    assert np.array_equal(out[0]["T2"], out[1]["T2"])
    assert out[0]["et"] == out[1]["et"]
