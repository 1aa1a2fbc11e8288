"""The complex CCSD programs of the library, and its stored-integral
residual, run on the host (no GPU).

``sisi4s_gb300/csrc/ccsd_complex.hpp`` holds the complex branch's statement
sequence once, over a backend of real primitives, and
``sisi4s_gb300/csrc/ccsd_stored.hpp`` the stored-V_abcd residual
(CcsdEnergyFromCoulombIntegralsReference); the library runs both with its
CUDA backend.  Here the same source is compiled with the host backend in
``tests/harness/cx_host.cpp`` (naive loops restating each primitive, with the
contraction engine's restrictions) and compared with the complex oracle,
which is pinned to the reference's golden energies.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from oracle.ccsd_complex import (ccsd_complex, coulomb_integrals_complex, pair_energy_complex,
                                 residual_complex, triples_complex_loop)
from sisi4s_gb300.inputs import make_system

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HARNESS = os.path.join(ROOT, "tests", "harness")
_dp = C.POINTER(C.c_double)


@pytest.fixture(scope="module")
def lib():
    out = os.path.join(HARNESS, "_build")
    os.makedirs(out, exist_ok=True)
    so = os.path.join(out, "libcx_host.so")
    src = os.path.join(HARNESS, "cx_host.cpp")
    hdr = os.path.join(ROOT, "sisi4s_gb300", "csrc", "ccsd_complex.hpp")
    deps = [src, hdr, os.path.join(os.path.dirname(hdr), "ccsd_stored.hpp")]
    if not os.path.exists(so) or os.path.getmtime(so) < max(map(os.path.getmtime, deps)):
        subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Wextra", "-Werror",
                        "-fPIC", "-shared", "-I", os.path.dirname(hdr), src, "-o", so],
                       check=True, capture_output=True, text=True)
    lib = C.CDLL(so)
    lib.cx_last_error.restype = C.c_char_p
    return lib


def _p(a):
    return None if a is None else a.ctypes.data_as(_dp)


def _flat(a):
    """complex tensor -> interleaved (re, im), first index fastest"""
    z = np.ascontiguousarray(np.asarray(a, dtype=np.complex128).transpose(
        tuple(range(a.ndim - 1, -1, -1)))).ravel()
    return z.view(np.float64).copy()


def _unflat(f, shape):
    return f.view(np.complex128).reshape(tuple(reversed(shape))).transpose(
        tuple(range(len(shape) - 1, -1, -1)))


def _system(No, Nv, NG, seed):
    """A genuinely complex physical vertex: a real symmetric vertex with its
    rows mixed by a random unitary and random orbital phases."""
    s = make_system(No, Nv, NG, seed=seed)
    rng = np.random.default_rng(seed + 100)
    W, _ = np.linalg.qr(rng.normal(size=(NG, NG)) + 1j * rng.normal(size=(NG, NG)))
    ph = np.exp(1j * rng.uniform(0, 2 * np.pi, No + Nv))
    g = np.einsum("GH,Hpq->Gpq", W, np.conj(ph)[None, :, None] * s.gamma * ph[None, None, :])
    T1 = rng.normal(0, 0.05, (Nv, No)) + 1j * rng.normal(0, 0.05, (Nv, No))
    T2 = rng.normal(0, 0.05, (Nv, Nv, No, No)) + 1j * rng.normal(0, 0.05, (Nv, Nv, No, No))
    return s, g, T1, 0.5 * (T2 + T2.transpose(1, 0, 3, 2))


def _rel(a, b):
    return np.abs(a - b).max() / np.abs(b).max()


@pytest.mark.parametrize("it,init,dist,ppl,slice_size", [
    (1, 1, 0, 1, -1), (1, 1, 1, 1, 2), (1, 1, 0, 0, -1), (1, 1, 0, 1, 3),
    (0, 1, 0, 1, 2), (0, 0, 0, 1, -1)])
def test_residual_program_matches_oracle(lib, it, init, dist, ppl, slice_size):
    No, Nv, NG = 3, 7, 11
    s, g, T1, T2 = _system(No, Nv, NG, seed=4)
    ci = coulomb_integrals_complex(g, No)
    r1 = np.zeros(2 * Nv * No)
    r2 = np.zeros(2 * Nv * Nv * No * No)
    st = lib.cx_residual(No, Nv, NG, _p(s.eps_h), _p(s.eps_p), _p(_flat(g)), it, init,
                         dist, ppl, slice_size, _p(_flat(T1)), _p(_flat(T2)), _p(r1), _p(r2))
    assert st == 0, lib.cx_last_error()
    o1, o2 = residual_complex(it, T1, T2, ci, g, distinguishable=dist, ppl=ppl,
                              slice_size=slice_size, initial_doubles=bool(init))
    g1, g2 = _unflat(r1, (Nv, No)), _unflat(r2, (Nv, Nv, No, No))
    assert _rel(g2, o2) < 1e-13
    if it or init:
        assert _rel(g1, o1) < 1e-13
    else:  # MP2 start: R2 = Vabij and R1 = 0 (CcsdEnergyFromCoulombIntegrals.cxx:516-520)
        assert not np.any(g1) and not np.any(o1)


@pytest.mark.parametrize("ratio,shift,fock", [(1.0, 0.0, False), (0.7, 0.0, False),
                                              (1.0, 0.3, False), (1.0, 0.0, True)])
def test_solve_program_matches_oracle(lib, ratio, shift, fock):
    No, Nv, NG = 3, 7, 11
    s, g, _, _ = _system(No, Nv, NG, seed=6)
    ci = coulomb_integrals_complex(g, No)
    rng = np.random.default_rng(12)
    f = (rng.normal(0, 0.05, (No, Nv)) + 1j * rng.normal(0, 0.05, (No, Nv))) if fock else None
    n = 40
    e = np.zeros(2)
    hist = np.zeros(2 * n)
    it, conv = C.c_int(), C.c_int()
    t1 = np.zeros(2 * Nv * No)
    t2 = np.zeros(2 * Nv * Nv * No * No)
    st = lib.cx_solve(No, Nv, NG, _p(s.eps_h), _p(s.eps_p), _p(_flat(g)), None, None, n,
                      C.c_double(1e-10), C.c_double(1e-8), C.c_double(shift),
                      C.c_double(ratio), 0, 1, 2, _p(e), C.byref(it), C.byref(conv),
                      _p(hist), _p(t1), _p(t2), _p(None if f is None else _flat(f)))
    assert st == 0, lib.cx_last_error()
    ref = ccsd_complex(s.eps_h, s.eps_p, ci, g, mixing_ratio=ratio, level_shift=shift,
                       max_iterations=n, energy_convergence=1e-10,
                       amplitudes_convergence=1e-8, slice_size=2, fock_hp=f)
    assert it.value == ref["iterations"] and bool(conv.value) == ref["converged"]
    h = hist[:2 * it.value].view(np.complex128)
    rh = np.array([x["energy"]["value"] for x in ref["history"]])
    assert np.abs(h - rh).max() < 1e-14
    assert _rel(_unflat(t2, (Nv, Nv, No, No)), ref["T2"]) < 1e-12


def test_solve_and_triples_programs_match_the_committed_fixture(lib):
    """The complex trajectory and (T) of tests/golden/oracle_cases.json."""
    from tests.golden import cases
    f = cases.load(cases.ORACLE_FILE)["complex"]
    o = cases.COMPLEX_SOLVE
    s, g = cases.complex_system(**cases.COMPLEX)
    No, Nv, NG = s.No, s.Nv, s.NG
    n = o["max_iterations"]
    e, hist = np.zeros(2), np.zeros(2 * n)
    it, conv = C.c_int(), C.c_int()
    t1, t2 = np.zeros(2 * Nv * No), np.zeros(2 * Nv * Nv * No * No)
    st = lib.cx_solve(No, Nv, NG, _p(s.eps_h), _p(s.eps_p), _p(_flat(g)), None, None, n,
                      C.c_double(o["energy_convergence"]),
                      C.c_double(o["amplitudes_convergence"]), C.c_double(0.0),
                      C.c_double(o["mixing_ratio"]), 0, 1, o["slice_size"], _p(e),
                      C.byref(it), C.byref(conv), _p(hist), _p(t1), _p(t2), None)
    assert st == 0, lib.cx_last_error()
    want = cases.complex_list(f["history"])
    assert it.value == want.size
    assert np.abs(hist.view(np.complex128) - want).max() < 1e-13
    et = np.zeros(2)
    st = lib.cx_triples(No, Nv, NG, _p(s.eps_h), _p(s.eps_p), _p(_flat(g)), _p(t1), _p(t2),
                        _p(et))
    assert st == 0, lib.cx_last_error()
    assert abs(complex(et[0], et[1]) - cases.complex_list([f["triples"]])[0]) < 1e-13


def test_program_reports_missing_inputs(lib):
    st = lib.cx_residual(0, 4, 5, None, None, None, 1, 1, 0, 1, -1, None, None, None, None)
    assert st == 1 and b"required" in lib.cx_last_error()


@pytest.mark.parametrize("No,Nv,NG", [(3, 6, 9), (2, 5, 7), (4, 5, 8)])
def test_triples_program_matches_oracle(lib, No, Nv, NG):
    s, g, T1, T2 = _system(No, Nv, NG, seed=No + Nv)
    ci = coulomb_integrals_complex(g, No)
    ref = triples_complex_loop(s.eps_h, s.eps_p, T1, T2, ci["PPHH"], ci["PHHH"], g)
    et = np.zeros(2)
    st = lib.cx_triples(No, Nv, NG, _p(s.eps_h), _p(s.eps_p), _p(_flat(g)), _p(_flat(T1)),
                        _p(_flat(T2)), _p(et))
    assert st == 0, lib.cx_last_error()
    assert abs(complex(et[0], et[1]) - ref) < 1e-13 * abs(ref)


@pytest.mark.parametrize("it,init,only_ppl", [(1, 1, 0), (0, 1, 0), (0, 0, 0), (1, 1, 1)])
def test_stored_residual_program_matches_oracle(lib, it, init, only_ppl):
    from oracle.ccsd import residual_reference
    from oracle.coulomb import coulomb_integrals
    No, Nv, NG = 3, 7, 12
    s = make_system(No, Nv, NG, seed=8)
    ints = coulomb_integrals(s.gamma, No, keys=("PPHH", "PHPH", "HHHH", "HHHP", "PPPP", "PPPH"))
    rng = np.random.default_rng(2)
    T1 = rng.normal(0, 0.05, (Nv, No))
    T2 = rng.normal(0, 0.05, (Nv, Nv, No, No))
    T2 = 0.5 * (T2 + T2.transpose(1, 0, 3, 2))
    f = lambda a: np.ascontiguousarray(a.transpose(tuple(range(a.ndim - 1, -1, -1)))).ravel()
    r1 = np.zeros(Nv * No)
    r2 = np.zeros(Nv * Nv * No * No)
    args = [f(ints[k]) for k in ("PPHH", "PHPH", "HHHH", "HHHP", "PPPP", "PPPH")]
    st = lib.st_residual(No, Nv, it, init, only_ppl, *[_p(a) for a in args], _p(f(T1)),
                         _p(f(T2)), _p(r1), _p(r2))
    assert st == 0, lib.cx_last_error()
    o1, o2 = residual_reference(it, T1, T2, ints, initial_doubles=bool(init),
                                only_ppl=bool(only_ppl))
    g1 = r1.reshape(No, Nv).T
    g2 = r2.reshape(No, No, Nv, Nv).transpose(3, 2, 1, 0)
    assert np.abs(g2 - o2).max() < 1e-13 * np.abs(o2).max()
    if np.any(o1):
        assert np.abs(g1 - o1).max() < 1e-13 * np.abs(o1).max()
    else:
        assert not np.any(g1)


def test_pair_energy_program_matches_oracle(lib):
    No, Nv, NG = 3, 6, 9
    s, g, T1, T2 = _system(No, Nv, NG, seed=3)
    ci = coulomb_integrals_complex(g, No)
    ref = pair_energy_complex(T1, T2, ci["HHPP"])
    pe = np.zeros(2 * No * No)
    st = lib.cx_pair_energy(No, Nv, NG, _p(s.eps_h), _p(s.eps_p), _p(_flat(g)), _p(_flat(T1)),
                            _p(_flat(T2)), _p(pe))
    assert st == 0, lib.cx_last_error()
    got = _unflat(pe, (No, No))
    assert np.abs(got - ref).max() < 1e-13 * np.abs(ref).max()
