"""Oracle restatement of the complex (k-point) branch of sisi4s' CCSD(T).

Test infrastructure only (see ``oracle/__init__.py``).

The reference runs this branch when the Coulomb integrals are complex
(``ClusterSinglesDoublesAlgorithm::run`` dispatches on the type of
PPHHCoulombIntegrals, src/algorithms/ClusterSinglesDoublesAlgorithm.cxx:25-35).
Restated here, one numpy expression per CTF statement and in the same order:

* ``CoulombIntegralsFromVertex::calculateComplexIntegrals``
  (src/algorithms/CoulombIntegralsFromVertex.cxx:613-816)
* ``CcsdEnergyFromCoulombIntegrals::getResiduum`` for complex amplitudes
  (src/algorithms/CcsdEnergyFromCoulombIntegrals.cxx:496-891) with its ladder
  slices ``sliceCoupledCoulombIntegrals``
  (src/algorithms/ClusterSinglesDoublesAlgorithm.cxx:492-563) and
  ``sliceIntoResiduum`` (:887-915)
* ``getEnergy<complex>`` (:130-237), the driver ``run<complex>`` (:37-128)
  and ``LinearMixer<complex>`` (src/mixers/LinearMixer.cxx:30-44).  The
  reference's complex DIIS solve is unimplemented (src/mixers/DiisMixer.cxx:43-48
  throws), so ``DiisMixer`` is refused here too
* ``CcsdPerturbativeTriplesComplex`` with complex amplitudes
  (src/algorithms/CcsdPerturbativeTriplesComplex.cxx:32-268,306-311,342-348)

Conventions.  ``gamma[G, p, q]`` is complex, holes first.  The reference's
"conjugate transposed" vertex slices are cGxy[G, x, y] = conj(gamma[G, y, x]),
and a Coulomb integral is V_xyzw = sum_G cG[G, x, z] G[G, y, w], e.g.
Vabij = sum_G conj(Gamma_Gia) Gamma_Gbj.  The ladder mirror of
``sliceIntoResiduum`` assumes V_xycd = V_yxdc, which holds for a physical
vertex (Gamma^G' = Gamma^G conjugate-transposed for some row G'); the tests
build their vertices that way.
"""
import numpy as np

__all__ = ["cvertex", "coulomb_integrals_complex", "residual_complex",
           "energy_complex", "pair_energy_complex", "ccsd_complex",
           "triples_complex_loop", "ComplexDiisUnsupported"]


class ComplexDiisUnsupported(NotImplementedError):
    """``inverse(std::vector<complex>, N)`` throws "TODO"
    (src/mixers/DiisMixer.cxx:43-48): the reference has no complex DIIS."""


def _e(spec, *ops):
    return np.einsum(spec, *ops, optimize=True)


def cvertex(gamma, no):
    """Slices of the vertex and their conjugate transposes
    (CcsdEnergyFromCoulombIntegrals.cxx:552-566): Gij, Gia, Gai, Gab and
    cGai = conj(Gia)^T, cGia = conj(Gai)^T, cGab = conj(Gab)^T,
    cGij = conj(Gij)^T (transposes over the two orbital indices)."""
    g = np.asarray(gamma, dtype=np.complex128)
    Gij, Gia = g[:, :no, :no], g[:, :no, no:]
    Gai, Gab = g[:, no:, :no], g[:, no:, no:]
    ct = lambda x: np.ascontiguousarray(np.conj(x).transpose(0, 2, 1))
    return {"ij": Gij, "ia": Gia, "ai": Gai, "ab": Gab,
            "cai": ct(Gia), "cia": ct(Gai), "cab": ct(Gab), "cij": ct(Gij)}


def coulomb_integrals_complex(gamma, no, keys=("PPHH", "HHPP", "PHHP", "PHPH",
                                               "HHHH", "HHHP", "PHHH")):
    """``calculateComplexIntegrals`` (CoulombIntegralsFromVertex.cxx:613-816):
      Vabij["abij"] = cGai["Gai"] Gai["Gbj"]     :767
      Vaijb["aijb"] = cGai["Gaj"] Gia["Gib"]     :774
      Vijab["ijab"] = cGia["Gia"] Gia["Gjb"]     :781
      Vaibj["aibj"] = cGab["Gab"] Gij["Gij"]     :788
      Vijkl["ijkl"] = cGij["Gik"] Gij["Gjl"]     :795
      Vijka["ijka"] = cGij["Gik"] Gia["Gja"]     :802
      Vaijk["aijk"] = cGai["Gaj"] Gij["Gik"]     :809
      Vabcd["abcd"] = cGab["Gac"] Gab["Gbd"]     :816
    """
    v = cvertex(gamma, no)
    out = {}
    keys = set(keys)
    if "PPHH" in keys:
        out["PPHH"] = _e("Gai,Gbj->abij", v["cai"], v["ai"])
    if "PHHP" in keys:
        out["PHHP"] = _e("Gaj,Gib->aijb", v["cai"], v["ia"])
    if "HHPP" in keys:
        out["HHPP"] = _e("Gia,Gjb->ijab", v["cia"], v["ia"])
    if "PHPH" in keys:
        out["PHPH"] = _e("Gab,Gij->aibj", v["cab"], v["ij"])
    if "HHHH" in keys:
        out["HHHH"] = _e("Gik,Gjl->ijkl", v["cij"], v["ij"])
    if "HHHP" in keys:
        out["HHHP"] = _e("Gik,Gja->ijka", v["cij"], v["ia"])
    if "PHHH" in keys:
        out["PHHH"] = _e("Gaj,Gik->aijk", v["cai"], v["ij"])
    if "PPPP" in keys:
        out["PPPP"] = _e("Gac,Gbd->abcd", v["cab"], v["ab"])
    return out


def residual_complex(it, T1, T2, ints, gamma, distinguishable=0, ppl=1,
                     slice_size=-1, slice_factor=None, initial_doubles=False):
    """``getResiduum`` for complex amplitudes
    (CcsdEnergyFromCoulombIntegrals.cxx:496-891).  ``ints`` holds PPHH, PHHP,
    HHPP, PHPH, HHHH, HHHP and PHHH.  Returns (R1, R2)."""
    Vabij = ints["PPHH"]
    T1 = np.asarray(T1, dtype=np.complex128)
    T2 = np.asarray(T2, dtype=np.complex128)
    R1 = np.zeros_like(T1)
    R2 = np.zeros_like(T2)
    if it == 0 and not initial_doubles:
        return R1, np.array(Vabij, dtype=np.complex128)          # :516-520
    Vaijb, Vijab, Vaibj = ints["PHHP"], ints["HHPP"], ints["PHPH"]
    Vijkl, Vijka, Vaijk = ints["HHHH"], ints["HHHP"], ints["PHHH"]
    No, Nv = Vabij.shape[2], Vabij.shape[0]
    v = cvertex(gamma, No)                                        # :552-566
    Gij, Gia, Gab = v["ij"], v["ia"], v["ab"]
    cGai, cGia, cGab, cGij = v["cai"], v["cia"], v["cab"], v["cij"]
    dist = bool(distinguishable)

    Xabij = T2 + _e("ai,bj->abij", T1, T1)                       # :588-590
    Kac = (-2.0) * _e("klcd,adkl->ac", Vijab, Xabij)             # :598
    Kac = Kac + 1.0 * _e("kldc,adkl->ac", Vijab, Xabij)          # :599
    if not dist:
        Lac = Kac.copy()                                         # :603
    else:
        Y = T2 + 2.0 * _e("ai,bj->abij", T1, T1)                 # :606-608
        Lac = (-1.0) * _e("klcd,adkl->ac", Vijab, Y)             # :609-610
        Lac = Lac + 0.5 * _e("kldc,adkl->ac", Vijab, Y)          # :611-612
    Lac = Lac + 2.0 * _e("Gac,Gkd,dk->ac", cGab, Gia, T1)        # :614-615
    Lac = Lac + (-1.0) * _e("Gad,Gkc,dk->ac", cGab, Gia, T1)     # :616-617
    Kki = 2.0 * _e("klcd,cdil->ki", Vijab, Xabij)                # :620
    Kki = Kki + (-1.0) * _e("kldc,cdil->ki", Vijab, Xabij)       # :621
    if not dist:
        Lki = 1.0 * Kki                                          # :625
    else:
        Y = T2 + 2.0 * _e("ai,bj->abij", T1, T1)                 # :628-630
        Lki = 1.0 * _e("klcd,cdil->ki", Vijab, Y)                # :631-632
        Lki = Lki + (-0.5) * _e("kldc,cdil->ki", Vijab, Y)       # :633-634
    Lki = Lki + 2.0 * _e("klic,cl->ki", Vijka, T1)               # :636
    Lki = Lki + (-1.0) * _e("lkic,cl->ki", Vijka, T1)            # :637
    R2 = R2 + 1.0 * _e("ac,cbij->abij", Lac, T2)                 # :640
    R2 = R2 + (-1.0) * _e("ki,abkj->abij", Lki, T2)              # :643

    dGai = cGai + (-1.0) * _e("Gki,ak->Gai", cGij, T1)           # :646-651
    R2 = R2 + 1.0 * _e("Gai,Gbc,cj->abij", dGai, Gab, T1)        # :652-653
    R2 = R2 + (-1.0) * _e("akij,bk->abij", Vaijk, T1)            # :655
    R2 = R2 + (-1.0) * _e("bk,akic,cj->abij", T1, Vaijb, T1)     # :656-657

    dGai = cGai + (-1.0) * _e("Gli,al->Gai", cGij, T1)           # :664-668
    dGai = dGai + 1.0 * _e("Gad,di->Gai", cGab, T1)              # :670-671
    Y = T2 + 2.0 * _e("ai,bj->abij", T1, T1)                     # :674-676
    dGai = dGai + (-0.5) * _e("Gld,dail->Gai", cGia, Y)          # :678-679
    Xakic = 1.0 * _e("Gai,Gkc->akic", dGai, Gia)                 # :681-682
    Y = np.einsum("lkdc->dclk", Vijab).copy()                    # :684
    if not dist:
        Y = Y + (-0.5) * np.einsum("lkcd->dclk", Vijab)          # :685
    Xakic = Xakic + _e("dclk,adil->akic", Y, T2)                 # :686
    Y = 2.0 * T2                                                 # :689
    Y = Y + (-1.0) * np.einsum("bckj->cbkj", T2)                 # :690
    R2 = R2 + 1.0 * _e("akic,cbkj->abij", Xakic, Y)              # :692

    dcGab = cGab + (-1.0) * _e("Glc,al->Gac", cGia, T1)          # :704-708
    dGij = Gij + 1.0 * _e("Gkd,di->Gki", Gia, T1)                # :710
    Xakci = 1.0 * _e("Gac,Gki->akci", dcGab, dGij)               # :713-714
    if not dist:
        Xakci = Xakci + (-0.5) * _e("lkcd,dail->akci", Vijab, T2)  # :718
    R2 = R2 + (-1.0) * _e("akci,cbkj->abij", Xakci, T2)          # :722
    R2 = R2 + (-1.0) * _e("bkci,ackj->abij", Xakci, T2)          # :723
    R2 = R2 + np.einsum("baji->abij", R2)                        # :726

    R2 = R2 + Vabij                                              # :735
    Xklij = np.array(Vijkl, dtype=np.complex128)                 # :742
    Xklij = Xklij + _e("klic,cj->klij", Vijka, T1)               # :743
    Xklij = Xklij + _e("lkjc,ci->klij", Vijka, T1)               # :744
    R2 = R2 + _e("klij,abkl->abij", Xklij, Xabij)                # :747
    if not dist:
        Xklij = _e("klcd,cdij->klij", Vijab, Xabij)              # :751
    else:
        Xklij = _e("ci,klcd,dj->klij", T1, Vijab, T1)            # :753
    if ppl:
        R2 = R2 + _e("klij,abkl->abij", Xklij, T2)               # :764
    else:
        R2 = R2 + _e("klij,abkl->abij", Xklij, Xabij)            # :766

    if ppl:
        s = int(slice_size)
        if s == -1:                                              # :810-819
            s = int(Nv * slice_factor) if slice_factor is not None else No
        # sliceCoupledCoulombIntegrals (ClusterSinglesDoublesAlgorithm.cxx:532-560)
        dGab = Gab + (-1.0) * _e("Gkb,ak->Gab", Gia, T1)         # :534
        dcGab = cGab + (-1.0) * _e("Gkb,ak->Gab", cGia, T1)      # :538-539
        for b in range(0, Nv, s):                                # :823
            for a in range(b, Nv, s):                            # :824
                sa = slice(a, min(a + s, Nv))
                sb = slice(b, min(b + s, Nv))
                Vxycd = _e("Gxc,Gyd->xycd", dcGab[:, sa, :], dGab[:, sb, :])  # :560
                Rxyij = _e("xycd,cdij->xyij", Vxycd, Xabij)     # :840
                R2[sa, sb] += Rxyij                              # :899-900
                if a > b:                                        # :901-914
                    R2[sb, sa] += np.einsum("xyij->yxji", Rxyij)

    R1 = R1 + 1.0 * _e("ac,ci->ai", Kac, T1)                     # :862
    R1 = R1 + (-1.0) * _e("ki,ak->ai", Kki, T1)                  # :863
    Kck = 2.0 * _e("klcd,dl->ck", Vijab, T1)                     # :866
    Kck = Kck + (-1.0) * _e("kldc,dl->ck", Vijab, T1)            # :867
    R1 = R1 + 2.0 * _e("ck,caki->ai", Kck, T2)                   # :870
    R1 = R1 + (-1.0) * _e("ck,caik->ai", Kck, T2)                # :871
    R1 = R1 + 1.0 * _e("ak,ck,ci->ai", T1, Kck, T1)              # :872
    R1 = R1 + 2.0 * _e("akic,ck->ai", Vaijb, T1)                 # :873
    R1 = R1 + (-1.0) * _e("akci,ck->ai", Vaibj, T1)              # :874
    R1 = R1 + 2.0 * _e("Gac,Gkd,cdik->ai", cGab, Gia, Xabij)     # :876-877
    R1 = R1 + (-1.0) * _e("Gad,Gkc,cdik->ai", cGab, Gia, Xabij)  # :878-879
    R1 = R1 + (-2.0) * _e("klic,ackl->ai", Vijka, Xabij)         # :881
    R1 = R1 + 1.0 * _e("lkic,ackl->ai", Vijka, Xabij)            # :882
    return R1, R2


def energy_complex(T1, T2, Vijab, spins=2.0, fock_hp=None):
    """``getEnergy<complex>`` non-antisymmetrized branch
    (ClusterSinglesDoublesAlgorithm.cxx:131-209) with the given HHPP integrals
    (:137-139): direct = 0.5 s^2 (T2 + T1T1).Vijab["ijab"] (:170-172),
    exchange = -0.5 s (T2 + T1T1).Vijab["ijba"] (:175-177), and with
    HPFockMatrix f[i,a] the noncanonical s T1["ai"] f["ia"] (:199-206).
    Complex values; the emitted energies are their real parts (:189-196)."""
    d = 0.5 * spins * spins * _e("abij,ijab->", T2, Vijab)
    d = d + 0.5 * spins * spins * _e("ai,bj,ijab->", T1, T1, Vijab)
    x = (-0.5) * spins * _e("abij,ijba->", T2, Vijab)
    x = x + (-0.5) * spins * _e("ai,bj,ijba->", T1, T1, Vijab)
    d, x = complex(d), complex(x)
    out = {"direct": d, "exchange": x, "value": d + x}
    if fock_hp is not None:
        nc = complex(spins * _e("ai,ia->", T1, fock_hp))
        out["noncanonical"] = nc
        out["value"] = out["value"] + nc
    return out


def pair_energy_complex(T1, T2, Vijab):
    """PairEnergy[i,j] of ``getEnergy<complex>`` (ClusterSinglesDoublesAlgorithm.cxx:227-232):
    2 T2.V["ijab"] - T2.V["ijba"] + 2 T1T1.V["ijab"] - T1T1.V["ijba"]."""
    p = 2.0 * _e("abij,ijab->ij", T2, Vijab)
    p = p + (-1.0) * _e("abij,ijba->ij", T2, Vijab)
    p = p + 2.0 * _e("ai,bj,ijab->ij", T1, T1, Vijab)
    p = p + (-1.0) * _e("ai,bj,ijba->ij", T1, T1, Vijab)
    return p


def _fv_dot(x, y):
    """FockVector::dot (src/math/FockVector.hpp:226-236) with
    sisi4s::dot(x, y) = conj(x) y (src/math/MathFunctions.hpp:45-47)."""
    return complex(np.vdot(x[0], y[0])) + complex(np.vdot(x[1], y[1]))


def ccsd_complex(eps_h, eps_p, ints, gamma, *, mixer="LinearMixer",
                 mixing_ratio=1.0, max_iterations=16, energy_convergence=1e-6,
                 amplitudes_convergence=1e-5, level_shift=0.0,
                 distinguishable=0, ppl=1, slice_size=-1, slice_factor=None,
                 initial=None, fock_hp=None):
    """``run<complex>`` (ClusterSinglesDoublesAlgorithm.cxx:37-128).  Returns
    dict(energy (real part, :32), energy_complex, T1, T2, iterations,
    converged, history)."""
    if mixer == "DiisMixer":
        raise ComplexDiisUnsupported("TODO: complex DIIS (DiisMixer.cxx:43-48)")
    if mixer != "LinearMixer":
        raise ValueError("Mixer not implemented: %s" % mixer)
    eps_h = np.asarray(eps_h, dtype=np.float64)
    eps_p = np.asarray(eps_p, dtype=np.float64)
    No, Nv = eps_h.size, eps_p.size
    if initial is not None:
        T1 = np.array(initial[0], dtype=np.complex128)
        T2 = np.array(initial[1], dtype=np.complex128)
    else:
        T1 = np.zeros((Nv, No), dtype=np.complex128)
        T2 = np.zeros((Nv, Nv, No, No), dtype=np.complex128)
    # calculateExcitationEnergies (:343-364) in the same order as the real path
    d1 = eps_p[:, None] - eps_h[None, :]
    d2 = (((eps_p[:, None, None, None] - eps_h[None, None, :, None])
           + eps_p[None, :, None, None]) - eps_h[None, None, None, :])
    s = float(level_shift)
    r = float(mixing_ratio)
    last = None
    amp = (T1, T2)
    e = prev = 0.0
    history = []
    converged = False
    it = 0
    for it in range(max_iterations):                              # :89
        R1, R2 = residual_complex(it, amp[0], amp[1], ints, gamma,
                                  distinguishable=distinguishable, ppl=ppl,
                                  slice_size=slice_size, slice_factor=slice_factor,
                                  initial_doubles=initial is not None)
        R1, R2 = R1 - s * amp[0], R2 - s * amp[1]                 # :318
        N = [-R1 / (d1 + s), -R2 / (d2 + s)]                      # :311
        dT = [N[0] - amp[0], N[1] - amp[1]]                       # :97-98
        if last is not None:                                      # LinearMixer :33-41
            for c in range(2):
                last[0][c] = last[0][c] * (1 - r)
                N[c] = N[c] * r + last[0][c]
                last[1][c] = last[1][c] * (1 - r)
                dT[c] = dT[c] * r + last[1][c]
        last = (N, dT)
        amp = (N[0], N[1])
        en = energy_complex(amp[0], amp[1], ints["HHPP"], fock_hp=fock_hp)  # :102
        e = en["value"]
        history.append({"iteration": it + 1, "energy": en})
        if (abs((e - prev) / e) < abs(energy_convergence)
                and abs(_fv_dot(dT, dT) / _fv_dot(amp, amp))
                < abs(amplitudes_convergence * amplitudes_convergence)):  # :103-106
            converged = True
            break
        prev = e
    return {"energy": e.real, "energy_complex": e, "T1": amp[0], "T2": amp[1],
            "iterations": it + 1, "converged": converged, "history": history}


def _perm(p):
    """Permutation<3>(p) images (src/math/Permutation.hpp:52-62)."""
    from .triples import permutation
    return permutation(p)


def triples_complex_loop(eps_h, eps_p, T1, T2, Vabij, Vaijk, gamma):
    """E_(T) of ``CcsdPerturbativeTriplesComplex::Calculator<complex>::calculate``
    (CcsdPerturbativeTriplesComplex.cxx:166-268).  Per distinct image m of
    (i, j, k):
      DV_abc = T_ad^{m0 m1} conj(Gamma_Fdb) Gamma_Fc^{m2}       (:310, :346-347)
             - T_ab^{m0 l} V_{c l m2 m1}  (PHHH)                  (:141)
    then DV = conj(sum_pi DV_pi(abc) / D) (:224-229), and
    E += sum_abc DV_abc sum_sigma f_sigma (DV_p + S_p)[sigma pi (abc)] over
    the distinct images (:231-253), with S = 0.5 T_a^{m0} V_bc^{m1 m2} (:148).
    Returns the complex (T) energy; the reference keeps its real part (:77)."""
    from .triples import SPIN_FERMI, _invariant, _map_times, _perm_string
    eps_h = np.asarray(eps_h, dtype=np.float64)
    eps_p = np.asarray(eps_p, dtype=np.float64)
    No = eps_h.size
    g = np.asarray(gamma, dtype=np.complex128)
    conjGab = np.conj(g[:, No:, No:])                             # :306-311
    Gai = g[:, No:, :No]
    perms = [_perm(p) for p in range(6)]
    s = "abc"

    def doubles(m):
        w = np.einsum("ad,Fdb,Fc->abc", T2[:, :, m[0], m[1]], conjGab,
                      Gai[:, :, m[2]], optimize=True)
        return w - np.einsum("abl,cl->abc", T2[:, :, m[0], :],
                             Vaijk[:, :, m[2], m[1]])

    def singles(m):
        return 0.5 * np.einsum("a,bc->abc", T1[:, m[0]], Vabij[:, :, m[1], m[2]])

    energy = 0.0 + 0.0j
    for i0 in range(No):
        for i1 in range(i0, No):
            for i2 in range(i1, No):
                i = (i0, i1, i2)
                piDV = [None] * 6
                distinct = [False] * 6
                DV = 0.0
                for p in range(6):
                    pi = perms[p]
                    q = next((q for q in range(p)
                              if _map_times(i, perms[q]) == _map_times(i, pi)), p)
                    if q < p:
                        piDV[p] = piDV[q]
                    else:
                        distinct[p] = True
                        piDV[p] = doubles(_map_times(i, pi))
                    DV = DV + np.einsum(_perm_string(s, pi) + "->abc", piDV[p])
                e = eps_p
                den = (((eps_h[i0] + eps_h[i1]) + eps_h[i2]) - e[:, None, None]
                       - e[None, :, None]) - e[None, None, :]     # :156-161
                DV = np.conj(DV / den)
                for p in range(6):
                    if not distinct[p]:
                        continue
                    pi = perms[p]
                    m = _map_times(i, pi)
                    S = singles(m)
                    T = 0.0
                    for sg in range(6):
                        sf = SPIN_FERMI[_invariant(perms[sg])]
                        u = _perm_string(_perm_string(s, perms[sg]), pi)
                        T = T + sf * np.einsum(u + "->abc", piDV[p])
                        T = T + sf * np.einsum(u + "->abc", S)
                    energy += complex(np.einsum("abc,abc->", DV, T))
    return energy
