// The stored-integral CCSD residual, written once over a real backend.
//
// CcsdEnergyFromCoulombIntegralsReference::getResiduum (real path,
// src/algorithms/CcsdEnergyFromCoulombIntegralsReference.cxx:29-292) keeps
// V_abcd and V_abci resident instead of rebuilding the particle ladder from
// the vertex.  Its statements follow here in order; three-operand CTF
// products are evaluated as two contractions through a temporary.  The
// backend is the one of ccsd_complex.hpp (contract, assign, axpby, fill); the
// library runs it on the GPU, the test suite on the host against the oracle.
#pragma once

#include "ccsd_complex.hpp"

namespace gbcc {
namespace st {

using cx::View;

// integrals of the stored formulation (views of resident tensors)
struct Ints {
  View Vabij;  // PPHH [Nv,Nv,No,No]
  View Vaibj;  // PHPH [Nv,No,Nv,No]
  View Vijkl;  // HHHH [No,No,No,No]
  View Vijka;  // HHHP [No,No,No,Nv]
  View Vabcd;  // PPPP [Nv,Nv,Nv,Nv]
  View Vabci;  // PPPH [Nv,Nv,Nv,No]
};

struct Opts {
  bool init_doubles = false;  // initialDoublesAmplitudes given
  bool only_ppl = false;      // onlyPPL (:43, :56-70)
};

template <class RB>
void residual(RB &rb, const Ints &I, int it, const Opts &o, const View &T1, const View &T2,
              const View &R1, const View &R2) {
  const int64_t Nv = T1.lens[0], No = T1.lens[1];
  auto C = [&](double al, const View &A, const char *ia, const View &B, const char *ib,
               double be, const View &Cc, const char *ic) {
    rb.contract(al, A, ia, B, ib, be, Cc, ic);
  };
  const View &V = I.Vabij;
  rb.fill(R1, 0.0);                                                 // :37-38
  rb.fill(R2, 0.0);
  if (it == 0 && !o.init_doubles && !o.only_ppl) {                  // :50-54 MP2 start
    rb.axpby(1.0, V, 0.0, R2);
    return;
  }
  if (o.only_ppl) {                                                 // :56-70
    auto X = rb.alloc({Nv, Nv, No, No});
    rb.axpby(1.0, T2, 0.0, X.v);
    C(1.0, T1, "ai", T1, "bj", 1.0, X.v, "abij");
    C(1.0, I.Vabcd, "abcd", X.v, "cdij", 0.0, R2, "abij");
    return;
  }
  const View &Vaibj = I.Vaibj, &Vijkl = I.Vijkl, &Vijka = I.Vijka;
  const View &Vabcd = I.Vabcd, &Vabci = I.Vabci;
  auto Kac = rb.alloc({Nv, Nv}), Lac = rb.alloc({Nv, Nv});
  auto Kki = rb.alloc({No, No}), Lki = rb.alloc({No, No});
  auto u = rb.alloc({Nv, No}), u2 = rb.alloc({Nv, No});
  C(1.0, V, "cdkl", T1, "dl", 0.0, u.v, "ck");                      // V["cdkl"] T1["dl"]
  C(1.0, V, "dckl", T1, "dl", 0.0, u2.v, "ck");                     // V["dckl"] T1["dl"]
  C(-2.0, V, "cdkl", T2, "adkl", 0.0, Kac.v, "ac");                 // :171
  C(1.0, V, "dckl", T2, "adkl", 1.0, Kac.v, "ac");                  // :172
  C(-2.0, T1, "ak", u.v, "ck", 1.0, Kac.v, "ac");                   // :173
  C(1.0, T1, "ak", u2.v, "ck", 1.0, Kac.v, "ac");                   // :174
  rb.axpby(1.0, Kac.v, 0.0, Lac.v);                                 // :177
  C(2.0, Vabci, "cdak", T1, "dk", 1.0, Lac.v, "ac");                // :178
  C(-1.0, Vabci, "dcak", T1, "dk", 1.0, Lac.v, "ac");               // :179
  C(2.0, V, "cdkl", T2, "cdil", 0.0, Kki.v, "ki");                  // :182
  C(-1.0, V, "dckl", T2, "cdil", 1.0, Kki.v, "ki");                 // :183
  C(2.0, T1, "ci", u.v, "ck", 1.0, Kki.v, "ki");                    // :184
  C(-1.0, T1, "ci", u2.v, "ck", 1.0, Kki.v, "ki");                  // :185
  rb.axpby(1.0, Kki.v, 0.0, Lki.v);                                 // :188
  C(2.0, Vijka, "klic", T1, "cl", 1.0, Lki.v, "ki");                // :189
  C(-1.0, Vijka, "lkic", T1, "cl", 1.0, Lki.v, "ki");               // :190
  C(1.0, Lac.v, "ac", T2, "cbij", 1.0, R2, "abij");                 // :193
  C(-1.0, Lki.v, "ki", T2, "abkj", 1.0, R2, "abij");                // :196
  C(1.0, Vabci, "baci", T1, "cj", 1.0, R2, "abij");                 // :199
  {
    auto w = rb.alloc({Nv, No, No, No});                            // :200
    C(1.0, Vaibj, "bkci", T1, "cj", 0.0, w.v, "bkij");
    C(-1.0, T1, "ak", w.v, "bkij", 1.0, R2, "abij");
  }
  C(-1.0, Vijka, "jika", T1, "bk", 1.0, R2, "abij");                // :201
  {
    auto w = rb.alloc({Nv, No, No, No});                            // :202
    C(1.0, V, "acik", T1, "cj", 0.0, w.v, "aikj");
    C(-1.0, T1, "bk", w.v, "aikj", 1.0, R2, "abij");
  }
  auto Xakic = rb.alloc({Nv, No, No, Nv});
  rb.assign(1.0, V, "acik", 0.0, Xakic.v, "akic");                  // :205
  C(-1.0, Vijka, "lkic", T1, "al", 1.0, Xakic.v, "akic");           // :206
  C(1.0, Vabci, "acdk", T1, "di", 1.0, Xakic.v, "akic");            // :207
  C(-0.5, V, "dclk", T2, "dail", 1.0, Xakic.v, "akic");             // :208
  {
    auto w = rb.alloc({Nv, No, No, No});                            // :209
    C(1.0, V, "dclk", T1, "di", 0.0, w.v, "clki");
    C(-1.0, T1, "al", w.v, "clki", 1.0, Xakic.v, "akic");
  }
  C(1.0, V, "dclk", T2, "adil", 1.0, Xakic.v, "akic");              // :210
  C(-0.5, V, "cdlk", T2, "adil", 1.0, Xakic.v, "akic");             // :211
  auto Xakci = rb.alloc({Nv, No, Nv, No});
  rb.axpby(1.0, Vaibj, 0.0, Xakci.v);                               // :214
  C(-1.0, Vijka, "klic", T1, "al", 1.0, Xakci.v, "akci");           // :215
  C(1.0, Vabci, "adck", T1, "di", 1.0, Xakci.v, "akci");            // :216
  C(-0.5, V, "cdlk", T2, "dail", 1.0, Xakci.v, "akci");             // :217
  {
    auto w = rb.alloc({Nv, No, No, No});                            // :218
    C(1.0, V, "cdlk", T1, "di", 0.0, w.v, "clki");
    C(-1.0, T1, "al", w.v, "clki", 1.0, Xakci.v, "akci");
  }
  C(2.0, Xakic.v, "akic", T2, "cbkj", 1.0, R2, "abij");             // :221
  C(-1.0, Xakic.v, "akic", T2, "bckj", 1.0, R2, "abij");            // :222
  C(-1.0, Xakci.v, "akci", T2, "cbkj", 1.0, R2, "abij");            // :224
  C(-1.0, Xakci.v, "bkci", T2, "ackj", 1.0, R2, "abij");            // :225
  {
    auto Rc = rb.alloc({Nv, Nv, No, No});                           // :229-230
    rb.axpby(1.0, R2, 0.0, Rc.v);
    rb.assign(1.0, Rc.v, "baji", 1.0, R2, "abij");
  }
  rb.axpby(1.0, V, 1.0, R2);                                        // :239
  auto Xklij = rb.alloc({No, No, No, No});
  rb.axpby(1.0, Vijkl, 0.0, Xklij.v);                               // :242
  C(1.0, Vijka, "klic", T1, "cj", 1.0, Xklij.v, "klij");            // :243
  C(1.0, Vijka, "lkjc", T1, "ci", 1.0, Xklij.v, "klij");            // :244
  C(1.0, V, "cdkl", T2, "cdij", 1.0, Xklij.v, "klij");              // :245
  {
    auto w = rb.alloc({Nv, No, No, No});                            // :246
    C(1.0, V, "cdkl", T1, "ci", 0.0, w.v, "dkli");
    C(1.0, w.v, "dkli", T1, "dj", 1.0, Xklij.v, "klij");
  }
  C(1.0, Xklij.v, "klij", T2, "abkl", 1.0, R2, "abij");             // :249
  {
    auto w = rb.alloc({Nv, No, No, No});                            // :252
    C(1.0, Xklij.v, "klij", T1, "ak", 0.0, w.v, "alij");
    C(1.0, w.v, "alij", T1, "bl", 1.0, R2, "abij");
  }
  {
    // :255-263 add X_abcd (T2_cdij + T1_ci T1_dj) with the dressed
    //   X_abcd = V_abcd - Vabci_cdak T1_bk - Vabci_dcbk T1_ak.
    // The same sum, without a second Nv^4 tensor:
    //   V_abcd Xp_cdij - T1_bk Y_akij - T1_ak Y'_bkij,  Xp = T2 + T1 T1,
    //   Y_akij = Vabci_cdak Xp_cdij,  Y'_bkij = Vabci_dcbk Xp_cdij,
    // so the only Nv^4 operand is the resident V_abcd (one GEMM, no permute)
    auto Xp = rb.alloc({Nv, Nv, No, No});
    rb.axpby(1.0, T2, 0.0, Xp.v);
    C(1.0, T1, "ci", T1, "dj", 1.0, Xp.v, "cdij");
    C(1.0, Vabcd, "abcd", Xp.v, "cdij", 1.0, R2, "abij");
    auto Y = rb.alloc({Nv, No, No, No});
    C(1.0, Vabci, "cdak", Xp.v, "cdij", 0.0, Y.v, "akij");
    C(-1.0, T1, "bk", Y.v, "akij", 1.0, R2, "abij");
    C(1.0, Vabci, "dcbk", Xp.v, "cdij", 0.0, Y.v, "bkij");
    C(-1.0, T1, "ak", Y.v, "bkij", 1.0, R2, "abij");
  }
  C(1.0, Kac.v, "ac", T1, "ci", 1.0, R1, "ai");                     // :271
  C(-1.0, Kki.v, "ki", T1, "ak", 1.0, R1, "ai");                    // :272
  auto Kck = rb.alloc({Nv, No});
  C(2.0, V, "cdkl", T1, "dl", 0.0, Kck.v, "ck");                    // :275
  C(-1.0, V, "cdlk", T1, "dl", 1.0, Kck.v, "ck");                   // :276
  C(2.0, Kck.v, "ck", T2, "caki", 1.0, R1, "ai");                   // :279
  C(-1.0, Kck.v, "ck", T2, "caik", 1.0, R1, "ai");                  // :280
  {
    auto w = rb.alloc({No, No});                                    // :282
    C(1.0, Kck.v, "ck", T1, "ci", 0.0, w.v, "ki");
    C(1.0, T1, "ak", w.v, "ki", 1.0, R1, "ai");
  }
  C(2.0, V, "acik", T1, "ck", 1.0, R1, "ai");                       // :283
  C(-1.0, Vaibj, "akci", T1, "ck", 1.0, R1, "ai");                  // :284
  C(2.0, Vabci, "cdak", T2, "cdik", 1.0, R1, "ai");                 // :285
  C(-1.0, Vabci, "dcak", T2, "cdik", 1.0, R1, "ai");                // :286
  {
    auto w = rb.alloc({Nv, Nv, No, No});                            // :287
    C(1.0, Vabci, "cdak", T1, "ci", 0.0, w.v, "daki");
    C(2.0, w.v, "daki", T1, "dk", 1.0, R1, "ai");
    C(1.0, Vabci, "dcak", T1, "ci", 0.0, w.v, "daki");              // :288
    C(-1.0, w.v, "daki", T1, "dk", 1.0, R1, "ai");
  }
  C(-2.0, Vijka, "klic", T2, "ackl", 1.0, R1, "ai");                // :289
  C(1.0, Vijka, "lkic", T2, "ackl", 1.0, R1, "ai");                 // :290
  {
    auto w = rb.alloc({No, No});                                    // :291
    C(1.0, Vijka, "klic", T1, "cl", 0.0, w.v, "ki");
    C(-2.0, T1, "ak", w.v, "ki", 1.0, R1, "ai");
    C(1.0, Vijka, "lkic", T1, "cl", 0.0, w.v, "ki");                // :292
    C(1.0, T1, "ak", w.v, "ki", 1.0, R1, "ai");
  }
}

}  // namespace st
}  // namespace gbcc
