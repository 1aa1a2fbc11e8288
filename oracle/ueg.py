"""Uniform-electron-gas inputs for pinning the oracle to reference goldens.

Test infrastructure only (see ``oracle/__init__.py``).

``ueg_planewave`` restates ``UegVertexGenerator::run``
(src/algorithms/UegVertexGenerator.cxx:49-229): the integer k-grid sorted by
|k|^2 and cut at No+Nv orbitals (:67-85), the cell volume
v = rs^3 * 4/3 pi * 2 No (:88), the Madelung constant by Ewald summation
(``evalMadelung`` :10-30), Hartree-Fock eigenvalues 0.5 k^2 minus the
exchange with every occupied plane wave (:99-104), and vertex entries
sqrt(4 pi / (v |k_q - k_p|^2)), with the Madelung constant at zero momentum
transfer (:212-224).

The reference's real code path forms V_pqrs = sum_G Gamma_Gpr Gamma_Gqs, which
assumes real orbitals.  Plane waves are complex, so ``ueg_real_vertex``
rotates each degenerate pair (k, -k) to standing waves (cos, sin), a unitary
change of orbitals within degenerate shells that leaves the Fock matrix
diagonal and every CCSD/(T) energy unchanged.  In that basis the transformed
vertex A_G = U^H Gamma_G U is complex symmetric with A_{-G} = conj(A_G), and
V_pqrs = sum_G Re A_pr Re A_qs + Im A_pr Im A_qs, which is the reference's
formula; stacking Re and Im as separate rows gives a real vertex of 2*NF rows.
"""
import math

import numpy as np
from scipy.special import erfc

__all__ = ["eval_madelung", "ueg_planewave", "ueg_real_vertex", "UEG_GOLDEN"]

#: golden energies of the reference integration test
#: integration-tests/tests/cc4s/ueg/rs1.0-7occ-26virt/cc4s.correct.out.yaml:
#: CCSD correlation :153 (direct :154, exchange :155), its secondOrder :156
#: (DIIS, maxResidua 4, energy and amplitude convergence 1e-8, maxIterations
#: 20, :134-147), (T) :169.
UEG_GOLDEN = {
    "No": 7, "Nv": 26, "rs": 1.0,
    "mp2": -0.36143028565969504,
    "ccsd": -0.39269658954585018,
    "triples": -0.0063019625641725016,
    "ccsd_settings": {"mixer": "DiisMixer", "max_residua": 4,
                      "energy_convergence": 1e-8,
                      "amplitudes_convergence": 1e-8, "max_iterations": 20},
}


def eval_madelung(v):
    """UegVertexGenerator::evalMadelung (UegVertexGenerator.cxx:10-30)."""
    kappa = v ** (-1.0 / 3.0)
    term2 = math.pi / (kappa * kappa * v)
    term4 = 2 * kappa / math.sqrt(math.pi)
    box = 1.0 / kappa
    recip = 0.0
    real = 0.0
    for l1 in range(-6, 7):
        for l2 in range(-6, 7):
            for l3 in range(-6, 7):
                n2 = l1 * l1 + l2 * l2 + l3 * l3
                if n2 > 0:
                    modr = box * math.sqrt(n2)
                    k2 = kappa * kappa * n2
                    recip -= (1.0 / (math.pi * k2)
                              * math.exp(-math.pi * math.pi * k2 / kappa / kappa) / v)
                    real -= erfc(kappa * modr) / modr
    return real + term2 + term4 + recip


def ueg_planewave(No, Nv, rs):
    """Plane-wave grid, eigenvalues and momentum-conserving vertex.

    Returns (kgrid[Np,3] int, eps[Np], gamma_pw[NF,Np,Np], madelung) where
    gamma_pw[G, x, y] = sqrt(v(k_x - k_y)) at the row G of that momentum
    transfer, so that <pq|rs> = sum_G gamma_pw[G,p,r] gamma_pw[G,s,q].
    """
    Np = No + Nv
    maxg = int((5.0 * Np) ** (1.0 / 3.0))
    grid = [(a, b, c) for a in range(-maxg, maxg + 1)
            for b in range(-maxg, maxg + 1) for c in range(-maxg, maxg + 1)]
    grid.sort(key=lambda t: t[0] * t[0] + t[1] * t[1] + t[2] * t[2])
    sl = lambda t: t[0] * t[0] + t[1] * t[1] + t[2] * t[2]
    if sl(grid[No]) == sl(grid[No - 1]):
        raise ValueError("occupied orbitals do not form a closed shell")
    if sl(grid[Np]) == sl(grid[Np - 1]):
        raise ValueError("virtual orbitals do not form a closed shell")
    kg = np.array(grid[:Np], dtype=np.int64)
    v = rs * rs * rs / 3.0 * 4.0 * math.pi * No * 2
    a = v ** (1.0 / 3.0)
    b = 2.0 * math.pi / a
    mad = eval_madelung(v)
    d = b * kg.astype(np.float64)
    eps = 0.5 * (d * d).sum(1)
    for p in range(Np):
        ex = 0.0
        for o in range(No):
            q = d[p] - d[o]
            s = float((q * q).sum())
            ex += mad if s < 1e-8 else 4.0 * math.pi / v / s
        eps[p] -= ex
    fac = 4.0 * math.pi / v
    rows = {}
    for x in range(Np):
        for y in range(Np):
            rows.setdefault(tuple(kg[x] - kg[y]), len(rows))
    gam = np.zeros((len(rows), Np, Np))
    for x in range(Np):
        for y in range(Np):
            dd = tuple(kg[x] - kg[y])
            s2 = sl(dd)
            gam[rows[dd], x, y] = math.sqrt(fac / (b * b * s2)) if s2 else math.sqrt(mad)
    return kg, eps, gam, mad


def ueg_real_vertex(No, Nv, rs):
    """Real vertex Gamma[2*NF, Np, Np] (holes first) in the standing-wave
    basis, with hole and particle eigenvalues."""
    kg, eps, gam, _ = ueg_planewave(No, Nv, rs)
    Np = No + Nv
    index = {tuple(k): n for n, k in enumerate(kg)}
    U = np.zeros((Np, Np), dtype=np.complex128)
    done = set()
    r2 = 1.0 / math.sqrt(2.0)
    for n, k in enumerate(kg):
        if n in done:
            continue
        m = index[tuple(-k)]
        if m == n:
            U[n, n] = 1.0
            done.add(n)
            continue
        # column n: cos wave, column m: sin wave (same shell, same energy)
        U[n, n] = r2
        U[m, n] = r2
        U[n, m] = -1j * r2
        U[m, m] = 1j * r2
        done.update((n, m))
    A = np.einsum("xp,Gxz,zr->Gpr", U.conj(), gam, U, optimize=True)
    real = np.concatenate([A.real, A.imag], axis=0)
    keep = np.any(real != 0.0, axis=(1, 2))
    real = np.ascontiguousarray(real[keep])
    # the transformed vertex is symmetric in (p, q) up to round-off; make it
    # exactly symmetric so that it is a valid input for every code path
    real = 0.5 * (real + real.transpose(0, 2, 1))
    return real, eps[:No].copy(), eps[No:].copy()
