"""CPU check of the (T) epilogue's bookkeeping (no GPU).

triples_orbit_kernel gives each CTA one orbit of 8^3 tiles under the six
coordinate permutations, scatters every W_p tile into the permuted D.V
positions inside the orbit, and contracts with the spin/Fermi weights
regrouped by cycle type (Z_p = 6 G_p + 2 G_same - 4 G_other).  This test
restates exactly that index logic in numpy (tile lists, tile moves, stride
tables, parities) and compares it with the reference loop of the oracle on
sizes whose edge tiles are partial.
"""
import itertools

import numpy as np
import pytest

from oracle.coulomb import coulomb_integrals
from oracle.triples import SPIN_FERMI, _Inputs, _map_times, permutation, triples_loop
from sisi4s_gb300.inputs import make_system

OT, OP = 8, 9


def _orbit_energy(eps_h, eps_p, T1, T2, Vabij, Vijka, gamma):
    inp = _Inputs(eps_h, eps_p, T1, T2, Vabij, Vijka, gamma)
    No, Nv = inp.No, inp.Nv
    img = [permutation(p) for p in range(6)]
    dinv = [[0] * 3 for _ in range(6)]
    for p in range(6):
        for n in range(3):
            dinv[p][img[p][n]] = n
    odd = [sum(img[p][a] > img[p][b] for a in range(3) for b in range(a + 1, 3)) % 2
           for p in range(6)]
    # the spin/Fermi factor depends only on the cycle type of rho_r pi_p^-1
    for p in range(6):
        pinv = [0] * 3
        for n in range(3):
            pinv[img[p][n]] = n
        for r in range(6):
            f = SPIN_FERMI[sum(img[r][pinv[k]] == k for k in range(3))]
            assert f == (8.0 if r == p else (2.0 if odd[r] == odd[p] else -4.0))
    ps = [[OP ** img[q][k] for k in range(3)] for q in range(6)]  # smem strides
    nt = (Nv + OT - 1) // OT
    z = np.array(list(itertools.product(range(OT), repeat=3)))[:, ::-1]  # z0 fastest
    energy = 0.0
    covered = {}
    for i0 in range(No):
        for i1 in range(i0, No):
            for i2 in range(i1, No):
                iv = (i0, i1, i2)
                m = [_map_times(iv, img[p]) for p in range(6)]
                distinct = [all(m[q] != m[p] for q in range(p)) for p in range(6)]
                W = []
                for p in range(6):
                    q = next(q for q in range(p + 1) if m[q] == m[p])
                    W.append(W[q] if q < p else inp.doubles(m[p]))
                ehs = (eps_h[i0] + eps_h[i1]) + eps_h[i2]
                for A in range(nt):
                    for B in range(A, nt):
                        for Cc in range(B, nt):
                            tl = []
                            for q in range(6):
                                c = tuple((A, B, Cc)[img[q][k]] for k in range(3))
                                if c not in tl:
                                    tl.append(c)
                            n = len(tl)
                            jt = [[tl.index(tuple(tl[j][dinv[q][k]] for k in range(3)))
                                   for j in range(n)] for q in range(6)]
                            DV = np.zeros(6 * OP ** 3)
                            for p in range(6):          # pass 1: scatter W_p
                                for j in range(n):
                                    g = np.array(tl[j]) * OT + z
                                    ok = (g < Nv).all(1)
                                    gg = np.minimum(g, Nv - 1)
                                    v = np.where(ok, W[p][gg[:, 0], gg[:, 1], gg[:, 2]], 0.0)
                                    dst = jt[p][j] * OP ** 3 + z @ np.array(ps[p])
                                    assert len(set(dst.tolist())) == len(dst)  # no clash
                                    DV[dst] += v
                            for j in range(n):          # denominator
                                g = np.array(tl[j]) * OT + z
                                ok = (g < Nv).all(1)
                                gg = np.minimum(g, Nv - 1)
                                den = ((ehs - eps_p[gg[:, 0]]) - eps_p[gg[:, 1]]) - eps_p[gg[:, 2]]
                                at = j * OP ** 3 + z @ np.array(ps[0])
                                DV[at] = np.where(ok, DV[at] / den, 0.0)
                            for j in range(n):          # pass 2: energy
                                y = np.array(tl[j]) * OT + z
                                ok = (y < Nv).all(1)
                                y, zz = y[ok], z[ok]
                                if i0 == 0 and i1 == 0 and i2 == 0:
                                    for t in map(tuple, y):
                                        covered[t] = covered.get(t, 0) + 1
                                G = np.stack([DV[jt[r][j] * OP ** 3 + zz @ np.array(ps[r])]
                                              for r in range(6)])
                                ge = sum(G[r] for r in range(6) if not odd[r])
                                go = sum(G[r] for r in range(6) if odd[r])
                                for p in range(6):
                                    if not distinct[p]:
                                        continue
                                    s_p = 0.5 * T1[y[:, 0], m[p][0]] * Vabij[y[:, 1], y[:, 2], m[p][1], m[p][2]]
                                    x = W[p][y[:, 0], y[:, 1], y[:, 2]] + s_p
                                    zsum = 6 * G[p] + (2 * ge - 4 * go if not odd[p] else 2 * go - 4 * ge)
                                    energy += float(np.sum(x * zsum))
    # the orbits of one triple cover every (a, b, c) exactly once
    assert len(covered) == Nv ** 3 and set(covered.values()) == {1}
    return energy


@pytest.mark.parametrize("No,Nv,NG", [(2, 11, 16), (3, 9, 12), (1, 17, 10)])
def test_orbit_epilogue_bookkeeping_matches_reference_loop(No, Nv, NG):
    s = make_system(No, Nv, NG, seed=No + Nv)
    ints = coulomb_integrals(s.gamma, No)
    rng = np.random.default_rng(5)
    T1 = rng.normal(0, 0.05, (Nv, No))
    T2 = rng.normal(0, 0.05, (Nv, Nv, No, No))
    T2 = 0.5 * (T2 + T2.transpose(1, 0, 3, 2))
    ref = triples_loop(s.eps_h, s.eps_p, T1, T2, ints["PPHH"], ints["HHHP"], s.gamma)
    got = _orbit_energy(s.eps_h, s.eps_p, T1, T2, ints["PPHH"], ints["HHHP"], s.gamma)
    assert abs(got - ref) < 1e-12 * max(1.0, abs(ref))
