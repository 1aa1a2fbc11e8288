"""Oracle restatement of ``CoulombIntegralsFromVertex::calculateRealIntegrals``.

Test infrastructure only (see ``oracle/__init__.py``).

Index conventions follow the reference: every tensor is indexed exactly as its
CTF index string, e.g. ``Vabij[a, b, i, j]``.  The vertex is ``Gamma[G, p, q]``
with the holes first (p < No), then the particles.
"""
import numpy as np

__all__ = ["split_vertex", "coulomb_integrals"]


def split_vertex(gamma, no):
    """Return the (real, imag) parts of Gamma_ai, Gamma_ab and Gamma_ij.

    Mirrors the slices of ``CoulombIntegralsFromVertex::run``
    (src/algorithms/CoulombIntegralsFromVertex.cxx:121-136) and
    ``fromComplexTensor`` (src/math/ComplexTensor.cxx:28-80).
    ``imag`` is ``None`` when the vertex is real or has an all-zero imaginary
    part, in which case every Im*Im term of the reference is identically 0.
    """
    gamma = np.asarray(gamma)
    re = np.ascontiguousarray(gamma.real, dtype=np.float64)
    im = None
    if np.iscomplexobj(gamma) and np.any(gamma.imag != 0):
        im = np.ascontiguousarray(gamma.imag, dtype=np.float64)

    def parts(sl):
        return re[sl], (None if im is None else im[sl])

    return {
        "ai": parts(np.s_[:, no:, :no]),
        "ab": parts(np.s_[:, no:, no:]),
        "ij": parts(np.s_[:, :no, :no]),
        "ia": parts(np.s_[:, :no, no:]),
    }


def _rr(spec, a, b):
    """Re*Re + Im*Im product of two (re, im) pairs with one einsum each."""
    out = np.einsum(spec, a[0], b[0], optimize=True)
    if a[1] is not None and b[1] is not None:
        out = out + np.einsum(spec, a[1], b[1], optimize=True)
    return out


def coulomb_integrals(gamma, no, keys=("PPHH", "PHPH", "HHHH", "HHHP"),
                      with_vabcd=False):
    """Real Coulomb integrals from the vertex.

    Statements (src/algorithms/CoulombIntegralsFromVertex.cxx):
      Vaibj["aibj"] = Gab["Gab"] Gij["Gij"]           :395-396
      Vabij["abij"] = Gai["Gai"] Gai["Gbj"]           :402-403
      Vijkl["ijkl"] = Gij["Gik"] Gij["Gjl"]           :409-410
      Vijka["ijka"] = Gij["Gik"] Gai["Gaj"]           :416-417
      Vabcd["abcd"] = Gab["Gac"] Gab["Gbd"]           :423-424
      Vabci["abci"] = Gab["Gac"] Gai["Gbi"]           :430-431
      Vijab["ijab"] = Vabij["abij"]                   :491
    """
    g = split_vertex(gamma, no)
    out = {}
    keys = set(keys)
    if "PHPH" in keys:
        out["PHPH"] = _rr("Gab,Gij->aibj", g["ab"], g["ij"])
    if "PPHH" in keys or "HHPP" in keys:
        out["PPHH"] = _rr("Gai,Gbj->abij", g["ai"], g["ai"])
    if "HHHH" in keys:
        out["HHHH"] = _rr("Gik,Gjl->ijkl", g["ij"], g["ij"])
    if "HHHP" in keys:
        out["HHHP"] = _rr("Gik,Gaj->ijka", g["ij"], g["ai"])
    if "HHPP" in keys:
        out["HHPP"] = np.einsum("abij->ijab", out["PPHH"]).copy()
    if with_vabcd or "PPPP" in keys:
        out["PPPP"] = _rr("Gac,Gbd->abcd", g["ab"], g["ab"])
    if with_vabcd or "PPPH" in keys:
        out["PPPH"] = _rr("Gac,Gbi->abci", g["ab"], g["ai"])
    return out
