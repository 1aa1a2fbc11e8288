"""Oracle restatement of the closed-shell real CCSD iteration of sisi4s.

Test infrastructure only (see ``oracle/__init__.py``).

Every tensor keeps the reference's index order (``T2[a, b, i, j]``,
``Vijka[i, j, k, a]``, ``Gamma[G, p, q]``).  Each CTF statement of the
reference becomes one numpy expression, in the same order, with the source
line cited beside it.  Three-operand CTF products are evaluated by
``einsum(..., optimize=True)``; CTF chooses its own pairwise order, so these
agree with the reference to round-off, not bitwise.
"""
import math

import numpy as np

from .coulomb import split_vertex
from .mixers import DiisMixer, LinearMixer, fv_dot, make_mixer

__all__ = [
    "residual", "residual_reference", "update_amplitudes", "energy",
    "excitation_denominators", "ccsd", "mp2_energy",
]


def _e(spec, *ops):
    return np.einsum(spec, *ops, optimize=True)


def _rr(spec, a, b, *rest):
    """Re*Re (+ Im*Im) form of a vertex product; ``a``/``b`` are (re, im)."""
    out = _e(spec, a[0], b[0], *rest)
    if a[1] is not None and b[1] is not None:
        out = out + _e(spec, a[1], b[1], *rest)
    return out


def excitation_denominators(eps_h, eps_p):
    """``calculateExcitationEnergies`` (ClusterSinglesDoublesAlgorithm.cxx:343-364).

    D starts at zero and is updated as D += eps_a; D -= eps_i; D += eps_b;
    D -= eps_j, i.e. D_abij = ((eps_a - eps_i) + eps_b) - eps_j in this exact
    floating-point order.
    """
    ea = eps_p[:, None]
    ei = eps_h[None, :]
    d1 = ea - ei
    d2 = (((eps_p[:, None, None, None] - eps_h[None, None, :, None])
           + eps_p[None, :, None, None]) - eps_h[None, None, None, :])
    return d1, d2


def update_amplitudes(R1, R2, T1, T2, d1, d2, level_shift=0.0):
    """``estimateAmplitudesFromResiduum`` (ClusterSinglesDoublesAlgorithm.cxx:302-331):
    R -= shift*T (:318), then r = -r / (d + shift) elementwise (:311)."""
    s = float(level_shift)
    R1 = R1 - s * T1
    R2 = R2 - s * T2
    return -R1 / (d1 + s), -R2 / (d2 + s)


def energy(T1, T2, Vabij, spins=2.0, fock_hp=None):
    """``getEnergy`` non-antisymmetrized branch (ClusterSinglesDoublesAlgorithm.cxx:131-209).

    Vijab["ijab"] = Vabij["abij"] (:146), so Vijab[i,j,a,b] = Vabij[a,b,i,j]
    and Vijab[i,j,b,a] = Vabij[b,a,i,j].
      direct   = 0.5 s^2 (T2.V  + T1T1.V)           :170-172
      exchange = -0.5 s  (T2.Vx + T1T1.Vx)          :175-177
      noncanonical = s T1["ai"] f["ia"]             :199-206 (HPFockMatrix given)
    Returns a dict with the emitted keys (:190-196, :207-208).
    """
    Vx = np.einsum("baij->abij", Vabij)
    d = 0.5 * spins * spins * _e("abij,abij->", T2, Vabij)
    d = d + 0.5 * spins * spins * _e("ai,bj,abij->", T1, T1, Vabij)
    x = (-0.5) * spins * _e("abij,abij->", T2, Vx)
    x = x + (-0.5) * spins * _e("ai,bj,abij->", T1, T1, Vx)
    d = float(d)
    x = float(x)
    out = {"direct": d, "exchange": x, "singlet": 0.25 * d - 0.5 * x,
           "triplet": 0.75 * d + 1.5 * x, "value": d + x}
    if fock_hp is not None:
        nc = float(spins * _e("ai,ia->", T1, fock_hp))
        out["noncanonical"] = nc
        out["value"] = out["value"] + nc
    return out


def pair_energy(T1, T2, Vabij):
    """PairEnergy[i,j] (ClusterSinglesDoublesAlgorithm.cxx:227-232)."""
    Vx = np.einsum("baij->abij", Vabij)
    p = 2.0 * _e("abij,abij->ij", T2, Vabij)
    p = p + (-1.0) * _e("abij,abij->ij", T2, Vx)
    p = p + 2.0 * _e("ai,bj,abij->ij", T1, T1, Vabij)
    p = p + (-1.0) * _e("ai,bj,abij->ij", T1, T1, Vx)
    return p


def residual(it, T1, T2, ints, gamma, distinguishable=0, ppl=1,
             slice_size=-1, slice_factor=None, initial_doubles=False):
    """``CcsdEnergyFromCoulombIntegrals::getResiduum`` real path
    (src/algorithms/CcsdEnergyFromCoulombIntegrals.cxx:27-494).

    ``ints`` holds "PPHH" (Vabij), "PHPH" (Vaibj), "HHHH" (Vijkl) and
    "HHHP" (Vijka).  Returns (R1, R2).
    """
    Vabij = ints["PPHH"]
    R1 = np.zeros_like(T1)
    R2 = np.zeros_like(T2)
    if it == 0 and not initial_doubles:
        # :47-51 MP2 start
        R2 = Vabij.copy()
        return R1, R2

    Vaibj = ints["PHPH"]
    Vijkl = ints["HHHH"]
    Vijka = ints["HHHP"]
    No = Vabij.shape[2]
    Nv = Vabij.shape[0]
    g = split_vertex(gamma, No)                                  # :70-115
    Gai, Gab, Gij = g["ai"], g["ab"], g["ij"]
    dist = bool(distinguishable)

    Xabij = T2 + _e("ai,bj->abij", T1, T1)                       # :136-138

    # Kac, Lac, Kki, Lki -------------------------------------------- :140-196
    Kac = (-2.0) * _e("cdkl,adkl->ac", Vabij, Xabij)             # :146
    Kac = Kac + (1.0) * _e("dckl,adkl->ac", Vabij, Xabij)        # :147
    if not dist:
        Lac = Kac.copy()                                         # :151
    else:
        Y = T2 + 2.0 * _e("ai,bj->abij", T1, T1)                 # :154-156
        Lac = (-1.0) * _e("cdkl,adkl->ac", Vabij, Y)             # :157-158
        Lac = Lac + 0.5 * _e("dckl,adkl->ac", Vabij, Y)          # :159-160
    Lac = Lac + 2.0 * _rr("Gca,Gdk,dk->ac", Gab, Gai, T1)        # :162-165
    Lac = Lac + (-1.0) * _rr("Gck,Gda,dk->ac", Gai, Gab, T1)     # :166-169
    Kki = 2.0 * _e("cdkl,cdil->ki", Vabij, Xabij)                # :172
    Kki = Kki + (-1.0) * _e("dckl,cdil->ki", Vabij, Xabij)       # :173
    if not dist:
        Lki = 1.0 * Kki                                          # :177
    else:
        Y = T2 + 2.0 * _e("ai,bj->abij", T1, T1)                 # :180-182
        Lki = 1.0 * _e("cdkl,cdil->ki", Vabij, Y)                # :183-184
        Lki = Lki + (-0.5) * _e("dckl,cdil->ki", Vabij, Y)       # :185-186
    Lki = Lki + 2.0 * _e("klic,cl->ki", Vijka, T1)               # :188
    Lki = Lki + (-1.0) * _e("lkic,cl->ki", Vijka, T1)            # :189
    R2 = R2 + 1.0 * _e("ac,cbij->abij", Lac, T2)                 # :192
    R2 = R2 + (-1.0) * _e("ki,abkj->abij", Lki, T2)              # :195

    # Gamma-dressed singles terms ---------------------------------- :198-216
    dGai_r = Gai[0] + (-1.0) * _e("Gki,ak->Gai", Gij[0], T1)     # :205
    dGai_i = None if Gai[1] is None else \
        Gai[1] + (-1.0) * _e("Gki,ak->Gai", Gij[1], T1)          # :206
    R2 = R2 + 1.0 * _rr("Gai,Gbc,cj->abij", (dGai_r, dGai_i), Gab, T1)  # :208-211
    R2 = R2 + (-1.0) * _e("jika,bk->abij", Vijka, T1)            # :213
    R2 = R2 + (-1.0) * _e("bk,acik,cj->abij", T1, Vabij, T1)     # :214-215

    # Xakic --------------------------------------------------------- :218-252
    dGai_r = Gai[0] + (-1.0) * _e("Gil,al->Gai", Gij[0], T1)     # :227
    dGai_r = dGai_r + 1.0 * _e("Gad,di->Gai", Gab[0], T1)        # :230
    if Gai[1] is not None:
        dGai_i = Gai[1] + (-1.0) * _e("Gil,al->Gai", Gij[1], T1)  # :228
        dGai_i = dGai_i + 1.0 * _e("Gad,di->Gai", Gab[1], T1)    # :231
    else:
        dGai_i = None
    Xakic = 1.0 * _rr("Gai,Gck->akic", (dGai_r, dGai_i), Gai)    # :234-235
    Y = T2 + 2.0 * _e("ai,bj->abij", T1, T1)                     # :238-240
    Xakic = Xakic + (-0.5) * _e("dclk,dail->akic", Vabij, Y)     # :242
    Xakic = Xakic + 1.0 * _e("dclk,adil->akic", Vabij, T2)       # :243
    if not dist:
        Xakic = Xakic + (-0.5) * _e("cdlk,adil->akic", Vabij, T2)  # :245
    Y = 2.0 * T2                                                 # :248
    Y = Y + (-1.0) * np.einsum("bckj->cbkj", T2)                 # :249
    R2 = R2 + 1.0 * _e("akic,cbkj->abij", Xakic, Y)              # :251

    # Xakci --------------------------------------------------------- :254-293
    dGab_r = Gab[0] + (-1.0) * _e("Gcl,al->Gac", Gai[0], T1)     # :270
    dGij_r = Gij[0] + 1.0 * _e("Gdk,di->Gki", Gai[0], T1)        # :273
    if Gab[1] is not None:
        dGab_i = Gab[1] + (-1.0) * _e("Gcl,al->Gac", Gai[1], T1)  # :271
        dGij_i = Gij[1] + 1.0 * _e("Gdk,di->Gki", Gai[1], T1)    # :274
    else:
        dGab_i = dGij_i = None
    Xakci = 1.0 * _rr("Gac,Gki->akci", (dGab_r, dGab_i), (dGij_r, dGij_i))  # :277-280
    if not dist:
        Xakci = Xakci + (-0.5) * _e("cdlk,dail->akci", Vabij, T2)  # :284
    R2 = R2 + (-1.0) * _e("akci,cbkj->abij", Xakci, T2)          # :288
    R2 = R2 + (-1.0) * _e("bkci,ackj->abij", Xakci, T2)          # :289
    R2 = R2 + np.einsum("baji->abij", R2)                        # :292

    # terms that are not symmetrised -------------------------------- :300-334
    R2 = R2 + Vabij                                              # :301
    Xklij = Vijkl.copy()                                         # :308
    Xklij = Xklij + _e("klic,cj->klij", Vijka, T1)               # :309
    Xklij = Xklij + _e("lkjc,ci->klij", Vijka, T1)               # :310
    R2 = R2 + _e("klij,abkl->abij", Xklij, Xabij)                # :313
    if not dist:
        Xklij = _e("cdkl,cdij->klij", Vabij, Xabij)              # :317
    else:
        Xklij = _e("ci,cdkl,dj->klij", T1, Vabij, T1)            # :319
    if ppl:
        R2 = R2 + _e("klij,abkl->abij", Xklij, T2)               # :330
    else:
        R2 = R2 + _e("klij,abkl->abij", Xklij, Xabij)            # :332

    # particle-particle ladder from Gamma slices -------------------- :374-452
    if ppl:
        s = int(slice_size)
        if s == -1:
            s = int(Nv * slice_factor) if slice_factor is not None else No
        nslices = int(math.ceil(Nv / s))                          # :387
        dG_r = Gab[0] + (-1.0) * _e("Gbk,ak->Gab", Gai[0], T1)    # :397-398
        dG_i = None if Gab[1] is None else \
            Gab[1] + (-1.0) * _e("Gbk,ak->Gab", Gai[1], T1)       # :399-400
        for m in range(nslices):                                  # :418
            for n in range(m, nslices):                           # :419
                sn = slice(n * s, min((n + 1) * s, Nv))
                sm = slice(m * s, min((m + 1) * s, Nv))
                Vxycd = _e("Gxc,Gyd->xycd", dG_r[:, sn, :], dG_r[:, sm, :])  # :431-432
                if dG_i is not None:
                    Vxycd = Vxycd + _e("Gxc,Gyd->xycd", dG_i[:, sn, :],
                                       dG_i[:, sm, :])           # :433-434
                Rxyij = _e("xycd,cdij->xyij", Vxycd, Xabij)        # :443
                a = n * s
                b = m * s
                # sliceIntoResiduum (ClusterSinglesDoublesAlgorithm.cxx:888-915)
                R2[sn, sm] += Rxyij
                if a > b:
                    R2[sm, sn] += np.einsum("xyij->yxji", Rxyij)

    # T1 equations --------------------------------------------------- :458-491
    R1 = R1 + 1.0 * _e("ac,ci->ai", Kac, T1)                     # :466
    R1 = R1 + (-1.0) * _e("ki,ak->ai", Kki, T1)                  # :467
    Kck = 2.0 * _e("cdkl,dl->ck", Vabij, T1)                     # :470
    Kck = Kck + (-1.0) * _e("dckl,dl->ck", Vabij, T1)            # :471
    R1 = R1 + 2.0 * _e("ck,caki->ai", Kck, T2)                   # :474
    R1 = R1 + (-1.0) * _e("ck,caik->ai", Kck, T2)                # :475
    R1 = R1 + 1.0 * _e("ak,ck,ci->ai", T1, Kck, T1)              # :476
    R1 = R1 + 2.0 * _e("acik,ck->ai", Vabij, T1)                 # :477
    R1 = R1 + (-1.0) * _e("ciak,ck->ai", Vaibj, T1)              # :478
    R1 = R1 + 2.0 * _rr("Gca,Gdk,cdik->ai", Gab, Gai, Xabij)     # :480-483
    R1 = R1 + (-1.0) * _rr("Gda,Gck,cdik->ai", Gab, Gai, Xabij)  # :484-487
    R1 = R1 + (-2.0) * _e("klic,ackl->ai", Vijka, Xabij)         # :489
    R1 = R1 + 1.0 * _e("lkic,ackl->ai", Vijka, Xabij)            # :490
    return R1, R2


def residual_reference(it, T1, T2, ints, initial_doubles=False, only_ppl=False):
    """``CcsdEnergyFromCoulombIntegralsReference::getResiduum`` (stored
    Vabcd/Vabci; src/algorithms/CcsdEnergyFromCoulombIntegralsReference.cxx:29-292).
    An independent second formulation of the same residual; ``ints`` must
    also hold "PPPP" (Vabcd) and "PPPH" (Vabci).  ``only_ppl`` is the
    onlyPPL option: R2 = Vabcd (T2 + T1 T1) alone (:56-70)."""
    Vabij = ints["PPHH"]
    R1 = np.zeros_like(T1)
    R2 = np.zeros_like(T2)
    if it == 0 and not initial_doubles and not only_ppl:
        return R1, Vabij.copy()                                  # :50-54
    if only_ppl:
        X = T2 + _e("ai,bj->abij", T1, T1)                       # :66-67
        return R1, _e("abcd,cdij->abij", ints["PPPP"], X)        # :70
    Vabcd, Vaibj, Vijkl = ints["PPPP"], ints["PHPH"], ints["HHHH"]
    Vijka, Vabci = ints["HHHP"], ints["PPPH"]
    Kac = (-2.0) * _e("cdkl,adkl->ac", Vabij, T2)                # :171
    Kac = Kac + _e("dckl,adkl->ac", Vabij, T2)                   # :172
    Kac = Kac + (-2.0) * _e("cdkl,ak,dl->ac", Vabij, T1, T1)     # :173
    Kac = Kac + _e("dckl,ak,dl->ac", Vabij, T1, T1)              # :174
    Lac = Kac.copy()                                             # :177
    Lac = Lac + 2.0 * _e("cdak,dk->ac", Vabci, T1)               # :178
    Lac = Lac + (-1.0) * _e("dcak,dk->ac", Vabci, T1)            # :179
    Kki = 2.0 * _e("cdkl,cdil->ki", Vabij, T2)                   # :182
    Kki = Kki + (-1.0) * _e("dckl,cdil->ki", Vabij, T2)          # :183
    Kki = Kki + 2.0 * _e("cdkl,ci,dl->ki", Vabij, T1, T1)        # :184
    Kki = Kki + (-1.0) * _e("dckl,ci,dl->ki", Vabij, T1, T1)     # :185
    Lki = Kki.copy()                                             # :188
    Lki = Lki + 2.0 * _e("klic,cl->ki", Vijka, T1)               # :189
    Lki = Lki + (-1.0) * _e("lkic,cl->ki", Vijka, T1)            # :190
    R2 = R2 + _e("ac,cbij->abij", Lac, T2)                       # :193
    R2 = R2 + (-1.0) * _e("ki,abkj->abij", Lki, T2)              # :196
    R2 = R2 + _e("baci,cj->abij", Vabci, T1)                     # :199
    R2 = R2 + (-1.0) * _e("bkci,ak,cj->abij", Vaibj, T1, T1)     # :200
    R2 = R2 + (-1.0) * _e("jika,bk->abij", Vijka, T1)            # :201
    R2 = R2 + (-1.0) * _e("acik,cj,bk->abij", Vabij, T1, T1)     # :202
    Xakic = np.einsum("acik->akic", Vabij).copy()                # :205
    Xakic = Xakic + (-1.0) * _e("lkic,al->akic", Vijka, T1)      # :206
    Xakic = Xakic + _e("acdk,di->akic", Vabci, T1)               # :207
    Xakic = Xakic + (-0.5) * _e("dclk,dail->akic", Vabij, T2)    # :208
    Xakic = Xakic + (-1.0) * _e("dclk,di,al->akic", Vabij, T1, T1)  # :209
    Xakic = Xakic + _e("dclk,adil->akic", Vabij, T2)             # :210
    Xakic = Xakic + (-0.5) * _e("cdlk,adil->akic", Vabij, T2)    # :211
    Xakci = Vaibj.copy()                                         # :214 (akci)
    Xakci = Xakci + (-1.0) * _e("klic,al->akci", Vijka, T1)      # :215
    Xakci = Xakci + _e("adck,di->akci", Vabci, T1)               # :216
    Xakci = Xakci + (-0.5) * _e("cdlk,dail->akci", Vabij, T2)    # :217
    Xakci = Xakci + (-1.0) * _e("cdlk,di,al->akci", Vabij, T1, T1)  # :218
    R2 = R2 + 2.0 * _e("akic,cbkj->abij", Xakic, T2)             # :221
    R2 = R2 + (-1.0) * _e("akic,bckj->abij", Xakic, T2)          # :222
    R2 = R2 + (-1.0) * _e("akci,cbkj->abij", Xakci, T2)          # :224
    R2 = R2 + (-1.0) * _e("bkci,ackj->abij", Xakci, T2)          # :225
    R2 = R2 + np.einsum("baji->abij", R2)                        # :229-230
    R2 = R2 + Vabij                                              # :239
    Xklij = Vijkl.copy()                                         # :242
    Xklij = Xklij + _e("klic,cj->klij", Vijka, T1)               # :243
    Xklij = Xklij + _e("lkjc,ci->klij", Vijka, T1)               # :244
    Xklij = Xklij + _e("cdkl,cdij->klij", Vabij, T2)             # :245
    Xklij = Xklij + _e("cdkl,ci,dj->klij", Vabij, T1, T1)        # :246
    R2 = R2 + _e("klij,abkl->abij", Xklij, T2)                   # :249
    R2 = R2 + _e("klij,ak,bl->abij", Xklij, T1, T1)              # :252
    Xabcd = Vabcd.copy()                                         # :255
    Xabcd = Xabcd + (-1.0) * _e("cdak,bk->abcd", Vabci, T1)      # :256
    Xabcd = Xabcd + (-1.0) * _e("dcbk,ak->abcd", Vabci, T1)      # :257
    R2 = R2 + _e("abcd,cdij->abij", Xabcd, T2)                   # :260
    R2 = R2 + _e("abcd,ci,dj->abij", Xabcd, T1, T1)              # :261
    R1 = R1 + _e("ac,ci->ai", Kac, T1)                           # :271
    R1 = R1 + (-1.0) * _e("ki,ak->ai", Kki, T1)                  # :272
    Kck = 2.0 * _e("cdkl,dl->ck", Vabij, T1)                     # :275
    Kck = Kck + (-1.0) * _e("cdlk,dl->ck", Vabij, T1)            # :276
    R1 = R1 + 2.0 * _e("ck,caki->ai", Kck, T2)                   # :279
    R1 = R1 + (-1.0) * _e("ck,caik->ai", Kck, T2)                # :280
    R1 = R1 + _e("ck,ci,ak->ai", Kck, T1, T1)                    # :282
    R1 = R1 + 2.0 * _e("acik,ck->ai", Vabij, T1)                 # :283
    R1 = R1 + (-1.0) * _e("akci,ck->ai", Vaibj, T1)              # :284
    R1 = R1 + 2.0 * _e("cdak,cdik->ai", Vabci, T2)               # :285
    R1 = R1 + (-1.0) * _e("dcak,cdik->ai", Vabci, T2)            # :286
    R1 = R1 + 2.0 * _e("cdak,ci,dk->ai", Vabci, T1, T1)          # :287
    R1 = R1 + (-1.0) * _e("dcak,ci,dk->ai", Vabci, T1, T1)       # :288
    R1 = R1 + (-2.0) * _e("klic,ackl->ai", Vijka, T2)            # :289
    R1 = R1 + _e("lkic,ackl->ai", Vijka, T2)                     # :290
    R1 = R1 + (-2.0) * _e("klic,ak,cl->ai", Vijka, T1, T1)       # :291
    R1 = R1 + _e("lkic,ak,cl->ai", Vijka, T1, T1)                # :292
    return R1, R2


def mp2_energy(eps_h, eps_p, Vabij):
    """Closed-form MP2: E = sum (2 V_abij - V_baij) V_abij / (e_i+e_j-e_a-e_b),
    equal to the driver's energy after iteration 0 (MP2 start)."""
    _, d2 = excitation_denominators(eps_h, eps_p)
    T2 = -Vabij / d2
    return energy(np.zeros((Vabij.shape[0], Vabij.shape[2])), T2, Vabij)["value"]


def ccsd(eps_h, eps_p, ints, gamma=None, *, mixer="LinearMixer", max_residua=4,
         mixing_ratio=1.0, max_iterations=16, energy_convergence=1e-6,
         amplitudes_convergence=1e-5, level_shift=0.0, distinguishable=0,
         ppl=1, slice_size=-1, slice_factor=None, initial=None,
         formulation="vertex", callback=None, fock_hp=None):
    """``ClusterSinglesDoublesAlgorithm::run<double>``
    (src/algorithms/ClusterSinglesDoublesAlgorithm.cxx:38-128).

    Returns dict(energy, T1, T2, iterations, converged, history) where history
    holds the emitted per-iteration energy maps.  ``formulation`` is
    "vertex" (CcsdEnergyFromCoulombIntegrals) or "reference"
    (CcsdEnergyFromCoulombIntegralsReference).
    """
    eps_h = np.asarray(eps_h, dtype=np.float64)
    eps_p = np.asarray(eps_p, dtype=np.float64)
    No, Nv = eps_h.size, eps_p.size
    if initial is not None:                                       # :247-256
        T1 = np.array(initial[0], dtype=np.float64)
        T2 = np.array(initial[1], dtype=np.float64)
    else:
        T1 = np.zeros((Nv, No))
        T2 = np.zeros((Nv, Nv, No, No))
    initial_doubles = initial is not None
    mix = make_mixer(mixer, max_residua, mixing_ratio)
    d1, d2 = excitation_denominators(eps_h, eps_p)
    e = 0.0
    prev = 0.0
    history = []
    it = 0
    converged = False
    amp = (T1, T2)
    for it in range(max_iterations):                              # :89
        if formulation == "vertex":
            R1, R2 = residual(it, amp[0], amp[1], ints, gamma,
                              distinguishable=distinguishable, ppl=ppl,
                              slice_size=slice_size, slice_factor=slice_factor,
                              initial_doubles=initial_doubles)     # :95
        else:
            R1, R2 = residual_reference(it, amp[0], amp[1], ints,
                                        initial_doubles=initial_doubles)
        N1, N2 = update_amplitudes(R1, R2, amp[0], amp[1], d1, d2,
                                   level_shift)                    # :96
        dT = [N1 - amp[0], N2 - amp[1]]                           # :97-98
        est = [N1, N2]
        if isinstance(mix, DiisMixer):
            mix.append((N1, N2), (dT[0], dT[1]))                  # :99
        else:
            mix.append(est, dT)
        amp = mix.get()                                           # :101
        en = energy(amp[0], amp[1], ints["PPHH"], fock_hp=fock_hp)  # :102
        e = en["value"]
        rec = {"iteration": it + 1, "energy": en}
        if isinstance(mix, DiisMixer):
            rec["mixing"] = {"lambda": float(mix.last_lambda),
                             "weights": [float(w) for w in mix.last_weights]}
        history.append(rec)
        if callback is not None:
            callback(it, amp, en)
        ddot = fv_dot(dT, dT)
        adot = fv_dot(amp, amp)
        if (abs((e - prev) / e) < abs(energy_convergence)
                and abs(ddot / adot) < abs(amplitudes_convergence
                                           * amplitudes_convergence)):  # :103-106
            converged = True
            break
        prev = e
    n_iter = it + 1 if max_iterations > 0 else 0
    if max_iterations == 0:                                       # :116-119
        e = energy(amp[0], amp[1], ints["PPHH"], fock_hp=fock_hp)["value"]
    return {"energy": e, "T1": amp[0], "T2": amp[1], "iterations": n_iter,
            "converged": converged, "history": history}
