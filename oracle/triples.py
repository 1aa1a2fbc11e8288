"""Oracle restatement of ``CcsdPerturbativeTriples`` (closed-shell (T)).

Test infrastructure only (see ``oracle/__init__.py``).

``triples_loop`` follows the reference loop literally
(src/algorithms/CcsdPerturbativeTriples.cxx:119-248): all 0 <= i <= j <= k <
No, the six permutations of ``Permutation<3>`` with reuse of equivalent ones,
the permuted accumulation of D.V, the division by the denominator, and the
spin/Fermi factors {+2, -4, 0, +8}.  ``triples_dense`` is a second,
vectorised evaluation of the same energy over all ordered (i, j, k), used to
check the permutation bookkeeping independently.
"""
import numpy as np

from .coulomb import split_vertex

__all__ = ["permutation", "triples_loop", "triples_dense", "SPIN_FERMI"]

#: spinAndFermiFactors indexed by invariantElementsCount (CcsdPerturbativeTriples.cxx:143)
SPIN_FERMI = (2.0, -4.0, 0.0, 8.0)


def permutation(p, n=3):
    """``Permutation<N>(p)`` images (src/math/Permutation.hpp:52-62, 80-84)."""
    if n == 1:
        return [0]
    sub = permutation(p // n, n - 1)
    r = p % n
    img = [0] * n
    for i in range(r):
        img[i] = sub[i] + 1
    img[r] = 0
    for i in range(r + 1, n):
        img[i] = sub[i - 1] + 1
    return img


def _perm_string(s, pi):
    """``operator*(std::string, Permutation)`` (CcsdPerturbativeTriples.cxx:23-29):
    sPi[i] = s[pi(i)]."""
    return "".join(s[pi[i]] for i in range(len(pi)))


def _map_times(i, tau):
    """``Map * Permutation`` (Permutation.hpp:96-101): g(n) = f(tau(n))."""
    return tuple(i[tau[n]] for n in range(len(tau)))


def _invariant(pi):
    return sum(1 for n in range(len(pi)) if pi[n] == n)


class _Inputs:
    def __init__(self, eps_h, eps_p, T1, T2, Vabij, Vijka, gamma):
        self.eps_h = np.asarray(eps_h, dtype=np.float64)
        self.eps_p = np.asarray(eps_p, dtype=np.float64)
        self.No = self.eps_h.size
        self.Nv = self.eps_p.size
        self.T1, self.T2, self.Vabij, self.Vijka = T1, T2, Vabij, Vijka
        g = split_vertex(gamma, self.No)                          # :48-78
        self.Gab = g["ab"]
        self.Gai = g["ai"]

    def singles(self, m):
        """getSinglesContribution (:82-85): 0.5 T_a^{m0} V_bc^{m1 m2}."""
        return 0.5 * np.einsum("a,bc->abc", self.T1[:, m[0]],
                               self.Vabij[:, :, m[1], m[2]])

    def doubles(self, m):
        """getDoublesContribution (:88-96):
        W_abc = T_ad^{m0 m1} (G_Fbd G_Fc^{m2}) - T_ab^{m0 l} V_{m1 m2 l c}."""
        t = self.T2[:, :, m[0], m[1]]
        w = np.einsum("ad,Fbd,Fc->abc", t, self.Gab[0], self.Gai[0][:, :, m[2]],
                      optimize=True)
        if self.Gab[1] is not None:
            w = w + np.einsum("ad,Fbd,Fc->abc", t, self.Gab[1],
                              self.Gai[1][:, :, m[2]], optimize=True)
        w = w - np.einsum("abl,lc->abc", self.T2[:, :, m[0], :],
                          self.Vijka[m[1], m[2], :, :])
        return w

    def denominator(self, i):
        """getEnergyDenominator (:98-117) in the reference's order."""
        e = self.eps_p
        d = (self.eps_h[i[0]] + self.eps_h[i[1]]) + self.eps_h[i[2]]
        return ((d - e[:, None, None]) - e[None, :, None]) - e[None, None, :]


def triples_loop(eps_h, eps_p, T1, T2, Vabij, Vijka, gamma):
    """E_(T) by the reference loop (CcsdPerturbativeTriples.cxx:119-240).
    Returns the (T) energy alone; the reference's output key
    ``CcsdPerturbativeTriplesEnergy`` is E_CCSD + E_(T) (:241-247)."""
    inp = _Inputs(eps_h, eps_p, T1, T2, Vabij, Vijka, gamma)
    No = inp.No
    perms = [permutation(p) for p in range(6)]
    s = "abc"
    energy = 0.0
    for i0 in range(No):
        for i1 in range(i0, No):
            for i2 in range(i1, No):
                i = (i0, i1, i2)
                piDV = [None] * 6
                distinct = [False] * 6
                DV = 0.0
                for p in range(6):
                    pi = perms[p]
                    q = 0
                    while q < p:
                        if _map_times(i, perms[q]) == _map_times(i, pi):
                            break
                        q += 1
                    if q < p:
                        distinct[p] = False
                        piDV[p] = piDV[q]
                    else:
                        distinct[p] = True
                        piDV[p] = inp.doubles(_map_times(i, pi))
                    DV = DV + np.einsum(_perm_string(s, pi) + "->abc", piDV[p])
                DV = DV / inp.denominator(i)
                for p in range(6):
                    if not distinct[p]:
                        continue
                    pi = perms[p]
                    m = _map_times(i, pi)
                    Tabc = 0.0
                    for sg in range(6):
                        sigma = perms[sg]
                        sf = SPIN_FERMI[_invariant(sigma)]
                        u = _perm_string(_perm_string(s, sigma), pi)
                        Tabc = Tabc + sf * np.einsum(u + "->abc", piDV[p])
                        Tabc = Tabc + sf * np.einsum(u + "->abc", inp.singles(m))
                    energy += float(np.einsum("abc,abc->", DV, Tabc))
    return energy


def triples_dense(eps_h, eps_p, T1, T2, Vabij, Vijka, gamma):
    """Same energy as ``triples_loop`` summed over all ordered (i, j, k):

    E = sum_{ijk abc} DV^{ijk}_{abc} Z^{ijk}_{abc},
    DV^{ijk}_{abc} = sum_pi W^{pi(ijk)}_{pi(abc)} / D^{ijk}_{abc},
    Z^{ijk}_{abc}  = sum_sigma f(sigma) (W + S)^{ijk}_{sigma(abc)}.
    """
    inp = _Inputs(eps_h, eps_p, T1, T2, Vabij, Vijka, gamma)
    No, Nv = inp.No, inp.Nv
    # Wvv[b,d,c,k] = sum_F Gab[F,b,d] Gai[F,c,k]
    Wvv = np.einsum("Fbd,Fck->bdck", inp.Gab[0], inp.Gai[0], optimize=True)
    if inp.Gab[1] is not None:
        Wvv = Wvv + np.einsum("Fbd,Fck->bdck", inp.Gab[1], inp.Gai[1],
                              optimize=True)
    # W[a,b,c,i,j,k]
    W = np.einsum("adij,bdck->abcijk", T2, Wvv, optimize=True)
    W = W - np.einsum("abil,jklc->abcijk", T2, Vijka, optimize=True)
    S = 0.5 * np.einsum("ai,bcjk->abcijk", T1, Vabij)
    letters = "abc"
    holes = "ijk"
    perms = [permutation(p) for p in range(6)]
    DV = np.zeros_like(W)
    for pi in perms:
        # W^{pi(ijk)}_{pi(abc)} as a tensor indexed [a,b,c,i,j,k]
        src = _perm_string(letters, pi) + _perm_string(holes, pi)
        DV += np.einsum(src + "->abcijk", W)
    e = eps_p
    h = eps_h
    D = (h[None, None, None, :, None, None] + h[None, None, None, None, :, None]
         + h[None, None, None, None, None, :] - e[:, None, None, None, None, None]
         - e[None, :, None, None, None, None] - e[None, None, :, None, None, None])
    DV = DV / D
    X = W + S
    Z = np.zeros_like(W)
    for sigma in perms:
        sf = SPIN_FERMI[_invariant(sigma)]
        Z += sf * np.einsum(_perm_string(letters, sigma) + "ijk->abcijk", X)
    del No, Nv
    return float(np.einsum("abcijk,abcijk->", DV, Z))
