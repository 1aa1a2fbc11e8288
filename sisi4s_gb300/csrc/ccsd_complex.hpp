// Complex (k-point) closed-shell CCSD, written once over a real backend.
//
// A complex tensor is two real planes (re, im) in the reference's dense
// layout.  Every complex product is four real contractions of the planes,
// with the conjugations of the reference's "conjTranspose" vertex slices
// folded into signs, so the arithmetic runs on the same contraction engine,
// permutes and elementwise kernels as the real path.  The statements follow
// the complex branch of CcsdEnergyFromCoulombIntegrals::getResiduum
// (src/algorithms/CcsdEnergyFromCoulombIntegrals.cxx:496-891) in order.
//
// The backend RB supplies the real primitives listed below.  The library
// instantiates this code with its CUDA backend (ccsd_complex.cu); the test
// suite instantiates the same code with a host backend to check the
// statement sequence against the oracle.
//
// Conventions.  Gamma[G,p,q] is complex, holes first.  The reference's
// conjugate-transposed slices are cGxy[G,x,y] = conj(Gyx[G,y,x]); a product
// with cGxy["Gxy"] is written here as the plane pair of Gyx with index string
// "Gyx" and the conjugation flag set.
#pragma once

#include <algorithm>
#include <array>
#include <complex>
#include <cstdint>
#include <initializer_list>
#include <stdexcept>
#include <string>
#include <vector>

namespace gbcc {
namespace cx {

struct View {
  double *p = nullptr;
  int order = 0;
  std::array<int64_t, 6> lens{};
  int64_t size() const {
    int64_t s = 1;
    for (int d = 0; d < order; ++d) s *= lens[d];
    return s;
  }
};

inline View view(double *p, std::initializer_list<int64_t> l) {
  View v;
  v.p = p;
  v.order = static_cast<int>(l.size());
  int d = 0;
  for (int64_t x : l) v.lens[d++] = x;
  return v;
}

// complex tensor: two real planes of the same shape
struct CView {
  View re, im;
};

// Layout of one complex amplitude plane pair: T1 then T2 in one buffer per
// plane, T2 starting on a 32-element boundary (the real path's FockLayout).
struct Layout {
  int64_t Nv = 0, No = 0, n1 = 0, n2 = 0, off2 = 0, ntot = 0;
  Layout() = default;
  Layout(int64_t nv, int64_t no) : Nv(nv), No(no) {
    n1 = Nv * No;
    n2 = Nv * Nv * No * No;
    off2 = (n1 + 31) / 32 * 32;
    ntot = off2 + n2;
  }
};

// Real primitives the backend provides (all views are dense, first index
// fastest):
//   Buf alloc(lens)                       owning buffer, .v is its view
//   contract(al, A, ia, B, ib, be, C, ic) C = al A.B + be C (index strings)
//   assign(al, A, ia, be, C, ic)          C = al A[perm] + be C
//   fill(x, v); axpby(a, x, b, y)         y = a x + b y
//   gather_slice(dst, src, x0, nx)        dst[G,x,c] = src[G,x0+x,c]
//   slice_add(R, Rxy, a0, b0, mirror)     sliceIntoResiduum
//   jacobi(L, eps_h, eps_p, R, T, est, dT, shift, sums)
//                                         est = -(R - s T)/(D + s), dT = est - T,
//                                         sums = {dT.dT, est.est}
//   linear_mix(next, nres, last, lres, r, sums)      LinearMixer::append
//   vertex_block(dst, src, p0, np, q0, nq)            Gamma sub-block
//   double scalar(x)                      read an order-0 tensor (synchronises)
//   read(x, host)                         copy a tensor to host memory (synchronises)
//   conj_over_denominator(re, im, eps_h, eps_p, i, j, k)
//                                         z[a,b,c] = conj(z / D^{ijk}_{abc}) for
//                                         the (T) denominator of the reference

template <class RB>
struct CBuf {
  typename RB::Buf re, im;
  CView v() const { return CView{re.v, im.v}; }
};

template <class RB>
CBuf<RB> cbuf(RB &rb, std::initializer_list<int64_t> l) {
  CBuf<RB> b;
  b.re = rb.alloc(l);
  b.im = rb.alloc(l);
  return b;
}

// C = al op(A) op(B) + be C, op = complex conjugation where the flag is set
template <class RB>
void ccontract(RB &rb, double al, const CView &A, const char *ia, bool cA,
               const CView &B, const char *ib, bool cB, double be,
               const CView &C, const char *ic) {
  const double sa = cA ? -1.0 : 1.0, sb = cB ? -1.0 : 1.0;
  // (Ar + i sa Ai)(Br + i sb Bi) = Ar Br - sa sb Ai Bi + i (sb Ar Bi + sa Ai Br)
  rb.contract(al, A.re, ia, B.re, ib, be, C.re, ic);
  rb.contract(-al * sa * sb, A.im, ia, B.im, ib, 1.0, C.re, ic);
  rb.contract(al * sb, A.re, ia, B.im, ib, be, C.im, ic);
  rb.contract(al * sa, A.im, ia, B.re, ib, 1.0, C.im, ic);
}

// C = al op(A)[perm] + be C
template <class RB>
void cassign(RB &rb, double al, const CView &A, const char *ia, bool cA,
             double be, const CView &C, const char *ic) {
  rb.assign(al, A.re, ia, be, C.re, ic);
  rb.assign(cA ? -al : al, A.im, ia, be, C.im, ic);
}

template <class RB>
void ccopy(RB &rb, const CView &dst, const CView &src) {
  rb.axpby(1.0, src.re, 0.0, dst.re);
  rb.axpby(1.0, src.im, 0.0, dst.im);
}

template <class RB>
void caxpby(RB &rb, double a, const CView &x, double b, const CView &y) {
  rb.axpby(a, x.re, b, y.re);
  rb.axpby(a, x.im, b, y.im);
}

template <class RB>
void czero(RB &rb, const CView &x) {
  rb.fill(x.re, 0.0);
  rb.fill(x.im, 0.0);
}

// X = T2 + c T1["ai"] T1["bj"]
template <class RB>
void couter(RB &rb, const CView &X, const CView &T2, const CView &T1, double c) {
  ccopy(rb, X, T2);
  ccontract(rb, c, T1, "ai", false, T1, "bj", false, 1.0, X, "abij");
}

// scalar of an order-0 complex tensor
template <class RB>
std::complex<double> cscalar(RB &rb, const CView &s) {
  return {rb.scalar(s.re), rb.scalar(s.im)};
}

// ------------------------------------------------------------------ inputs
template <class RB>
struct Inputs {
  int64_t No = 0, Nv = 0, NG = 0;
  typename RB::Buf eps_h, eps_p;   // [No], [Nv]
  CBuf<RB> Gij, Gia, Gai, Gab;     // vertex blocks [NG,No,No] ... [NG,Nv,Nv]
  // integrals of calculateComplexIntegrals (CoulombIntegralsFromVertex.cxx:767-809)
  CBuf<RB> Vabij, Vaijb, Vijab, Vaibj, Vijkl, Vijka, Vaijk;
  // HPFockMatrix f[i,a] [No,Nv], if given
  bool has_fock = false;
  CBuf<RB> fock;
};

// Gamma planes [NG, Np, Np] -> blocks and integrals
template <class RB>
void build_inputs(RB &rb, Inputs<RB> &I, const CView &G) {
  const int64_t No = I.No, Nv = I.Nv, NG = I.NG;
  auto block = [&](CBuf<RB> &dst, int64_t p0, int64_t np, int64_t q0, int64_t nq) {
    dst = cbuf(rb, {NG, np, nq});
    rb.vertex_block(dst.re.v, G.re, p0, np, q0, nq);
    rb.vertex_block(dst.im.v, G.im, p0, np, q0, nq);
  };
  block(I.Gij, 0, No, 0, No);                    // CcsdEnergyFromCoulombIntegrals.cxx:552-555
  block(I.Gia, 0, No, No, Nv);
  block(I.Gai, No, Nv, 0, No);
  block(I.Gab, No, Nv, No, Nv);
  const CView gij = I.Gij.v(), gia = I.Gia.v(), gai = I.Gai.v(), gab = I.Gab.v();
  I.Vabij = cbuf(rb, {Nv, Nv, No, No});        // :767 cGai["Gai"] Gai["Gbj"]
  ccontract(rb, 1.0, gia, "Gia", true, gai, "Gbj", false, 0.0, I.Vabij.v(), "abij");
  I.Vaijb = cbuf(rb, {Nv, No, No, Nv});        // :774 cGai["Gaj"] Gia["Gib"]
  ccontract(rb, 1.0, gia, "Gja", true, gia, "Gib", false, 0.0, I.Vaijb.v(), "aijb");
  I.Vijab = cbuf(rb, {No, No, Nv, Nv});        // :781 cGia["Gia"] Gia["Gjb"]
  ccontract(rb, 1.0, gai, "Gai", true, gia, "Gjb", false, 0.0, I.Vijab.v(), "ijab");
  I.Vaibj = cbuf(rb, {Nv, No, Nv, No});        // :788 cGab["Gab"] Gij["Gij"]
  ccontract(rb, 1.0, gab, "Gba", true, gij, "Gij", false, 0.0, I.Vaibj.v(), "aibj");
  I.Vijkl = cbuf(rb, {No, No, No, No});        // :795 cGij["Gik"] Gij["Gjl"]
  ccontract(rb, 1.0, gij, "Gki", true, gij, "Gjl", false, 0.0, I.Vijkl.v(), "ijkl");
  I.Vijka = cbuf(rb, {No, No, No, Nv});        // :802 cGij["Gik"] Gia["Gja"]
  ccontract(rb, 1.0, gij, "Gki", true, gia, "Gja", false, 0.0, I.Vijka.v(), "ijka");
  I.Vaijk = cbuf(rb, {Nv, No, No, No});        // :809 cGai["Gaj"] Gij["Gik"]
  ccontract(rb, 1.0, gia, "Gja", true, gij, "Gik", false, 0.0, I.Vaijk.v(), "aijk");
}

// ---------------------------------------------------------------- residual
struct ResidualOpts {
  bool init_doubles = false;
  bool distinguishable = false;
  bool ppl = true;
  int64_t slice = 0;  // integralsSliceSize after defaults (> 0)
};

// R = getResiduum(it, T) for complex amplitudes; T1/T2 and R1/R2 are plane
// pairs of [Nv,No] and [Nv,Nv,No,No]
template <class RB>
void residual(RB &rb, const Inputs<RB> &I, int it, const ResidualOpts &o,
              const CView &T1, const CView &T2, const CView &R1, const CView &R2) {
  const int64_t No = I.No, Nv = I.Nv, NG = I.NG;
  const bool dist = o.distinguishable;
  czero(rb, R1);
  czero(rb, R2);
  const CView V = I.Vabij.v();
  if (it == 0 && !o.init_doubles) {              // :516-520 MP2 start
    ccopy(rb, R2, V);
    return;
  }
  const CView Vaijb = I.Vaijb.v(), Vijab = I.Vijab.v(), Vaibj = I.Vaibj.v();
  const CView Vijkl = I.Vijkl.v(), Vijka = I.Vijka.v(), Vaijk = I.Vaijk.v();
  const CView Gij = I.Gij.v(), Gia = I.Gia.v(), Gai = I.Gai.v(), Gab = I.Gab.v();
  auto C = [&](double al, const CView &A, const char *ia, bool cA, const CView &B,
               const char *ib, bool cB, double be, const CView &Cc, const char *ic) {
    ccontract(rb, al, A, ia, cA, B, ib, cB, be, Cc, ic);
  };

  CBuf<RB> Xb = cbuf(rb, {Nv, Nv, No, No});    // :588-590
  const CView X = Xb.v();
  couter(rb, X, T2, T1, 1.0);
  CBuf<RB> Kacb = cbuf(rb, {Nv, Nv}), Kkib = cbuf(rb, {No, No});
  const CView Kac = Kacb.v(), Kki = Kkib.v();
  {
    CBuf<RB> Lacb = cbuf(rb, {Nv, Nv}), Lkib = cbuf(rb, {No, No});
    const CView Lac = Lacb.v(), Lki = Lkib.v();
    C(-2.0, Vijab, "klcd", false, X, "adkl", false, 0.0, Kac, "ac");  // :598
    C(1.0, Vijab, "kldc", false, X, "adkl", false, 1.0, Kac, "ac");   // :599
    if (!dist) {
      ccopy(rb, Lac, Kac);                                          // :603
    } else {
      CBuf<RB> Yb = cbuf(rb, {Nv, Nv, No, No});                   // :606-608
      couter(rb, Yb.v(), T2, T1, 2.0);
      C(-1.0, Vijab, "klcd", false, Yb.v(), "adkl", false, 0.0, Lac, "ac");  // :609-610
      C(0.5, Vijab, "kldc", false, Yb.v(), "adkl", false, 1.0, Lac, "ac");   // :611-612
    }
    {
      // :614-615 Lac += 2 cGab["Gac"] Gia["Gkd"] T1["dk"]
      CBuf<RB> t = cbuf(rb, {NG});
      C(1.0, Gia, "Gkd", false, T1, "dk", false, 0.0, t.v(), "G");
      C(2.0, Gab, "Gca", true, t.v(), "G", false, 1.0, Lac, "ac");
      // :616-617 Lac += -1 cGab["Gad"] Gia["Gkc"] T1["dk"]
      CBuf<RB> Q = cbuf(rb, {NG, Nv, No});
      C(1.0, Gab, "Gda", true, T1, "dk", false, 0.0, Q.v(), "Gak");
      C(-1.0, Gia, "Gkc", false, Q.v(), "Gak", false, 1.0, Lac, "ac");
    }
    C(2.0, Vijab, "klcd", false, X, "cdil", false, 0.0, Kki, "ki");   // :620
    C(-1.0, Vijab, "kldc", false, X, "cdil", false, 1.0, Kki, "ki");  // :621
    if (!dist) {
      ccopy(rb, Lki, Kki);                                          // :625
    } else {
      CBuf<RB> Yb = cbuf(rb, {Nv, Nv, No, No});                   // :628-630
      couter(rb, Yb.v(), T2, T1, 2.0);
      C(1.0, Vijab, "klcd", false, Yb.v(), "cdil", false, 0.0, Lki, "ki");   // :631-632
      C(-0.5, Vijab, "kldc", false, Yb.v(), "cdil", false, 1.0, Lki, "ki");  // :633-634
    }
    C(2.0, Vijka, "klic", false, T1, "cl", false, 1.0, Lki, "ki");   // :636
    C(-1.0, Vijka, "lkic", false, T1, "cl", false, 1.0, Lki, "ki");  // :637
    C(1.0, Lac, "ac", false, T2, "cbij", false, 1.0, R2, "abij");    // :640
    C(-1.0, Lki, "ki", false, T2, "abkj", false, 1.0, R2, "abij");   // :643
  }
  {
    // :646-651 dGai = cGai - cGij["Gki"] T1["ak"]
    CBuf<RB> dGai = cbuf(rb, {NG, Nv, No});
    cassign(rb, 1.0, Gia, "Gia", true, 0.0, dGai.v(), "Gai");
    C(-1.0, Gij, "Gik", true, T1, "ak", false, 1.0, dGai.v(), "Gai");
    // :652-653 R2 += dGai["Gai"] Gab["Gbc"] T1["cj"]
    CBuf<RB> Z = cbuf(rb, {NG, Nv, No});
    C(1.0, Gab, "Gbc", false, T1, "cj", false, 0.0, Z.v(), "Gbj");
    C(1.0, dGai.v(), "Gai", false, Z.v(), "Gbj", false, 1.0, R2, "abij");
    C(-1.0, Vaijk, "akij", false, T1, "bk", false, 1.0, R2, "abij");  // :655
    // :656-657 R2 += -T1["bk"] Vaijb["akic"] T1["cj"]
    CBuf<RB> W = cbuf(rb, {Nv, No, No, No});
    C(1.0, Vaijb, "akic", false, T1, "cj", false, 0.0, W.v(), "akij");
    C(-1.0, T1, "bk", false, W.v(), "akij", false, 1.0, R2, "abij");
  }
  {
    CBuf<RB> Xb2 = cbuf(rb, {Nv, No, No, Nv});                    // :660-692
    const CView Xakic = Xb2.v();
    {
      CBuf<RB> dGai = cbuf(rb, {NG, Nv, No});
      cassign(rb, 1.0, Gia, "Gia", true, 0.0, dGai.v(), "Gai");
      C(-1.0, Gij, "Gil", true, T1, "al", false, 1.0, dGai.v(), "Gai");    // :667-668
      C(1.0, Gab, "Gda", true, T1, "di", false, 1.0, dGai.v(), "Gai");     // :670-671
      CBuf<RB> Y = cbuf(rb, {Nv, Nv, No, No});                            // :674-676
      couter(rb, Y.v(), T2, T1, 2.0);
      C(-0.5, Gai, "Gdl", true, Y.v(), "dail", false, 1.0, dGai.v(), "Gai");  // :678-679
      C(1.0, dGai.v(), "Gai", false, Gia, "Gkc", false, 0.0, Xakic, "akic");  // :681-682
    }
    CBuf<RB> Yb = cbuf(rb, {Nv, Nv, No, No});
    const CView Y = Yb.v();
    cassign(rb, 1.0, Vijab, "lkdc", false, 0.0, Y, "dclk");         // :684
    if (!dist) cassign(rb, -0.5, Vijab, "lkcd", false, 1.0, Y, "dclk");  // :685
    C(1.0, Y, "dclk", false, T2, "adil", false, 1.0, Xakic, "akic");  // :686
    caxpby(rb, 2.0, T2, 0.0, Y);                                    // :689
    cassign(rb, -1.0, T2, "bckj", false, 1.0, Y, "cbkj");           // :690
    C(1.0, Xakic, "akic", false, Y, "cbkj", false, 1.0, R2, "abij");  // :692
  }
  {
    CBuf<RB> Xb3 = cbuf(rb, {Nv, No, Nv, No});                    // :696-726
    const CView Xakci = Xb3.v();
    {
      CBuf<RB> dcGab = cbuf(rb, {NG, Nv, Nv}), dGij = cbuf(rb, {NG, No, No});
      cassign(rb, 1.0, Gab, "Gca", true, 0.0, dcGab.v(), "Gac");
      C(-1.0, Gai, "Gcl", true, T1, "al", false, 1.0, dcGab.v(), "Gac");   // :707-708
      ccopy(rb, dGij.v(), Gij);
      C(1.0, Gia, "Gkd", false, T1, "di", false, 1.0, dGij.v(), "Gki");    // :710
      C(1.0, dcGab.v(), "Gac", false, dGij.v(), "Gki", false, 0.0, Xakci, "akci");  // :713-714
    }
    if (!dist) C(-0.5, Vijab, "lkcd", false, T2, "dail", false, 1.0, Xakci, "akci");  // :718
    C(-1.0, Xakci, "akci", false, T2, "cbkj", false, 1.0, R2, "abij");  // :722
    C(-1.0, Xakci, "bkci", false, T2, "ackj", false, 1.0, R2, "abij");  // :723
    CBuf<RB> Rc = cbuf(rb, {Nv, Nv, No, No});                     // :726
    ccopy(rb, Rc.v(), R2);
    cassign(rb, 1.0, Rc.v(), "baji", false, 1.0, R2, "abij");
  }
  caxpby(rb, 1.0, V, 1.0, R2);                                      // :735
  {
    CBuf<RB> Xk = cbuf(rb, {No, No, No, No});                     // :738-767
    const CView Xklij = Xk.v();
    ccopy(rb, Xklij, Vijkl);                                        // :742
    C(1.0, Vijka, "klic", false, T1, "cj", false, 1.0, Xklij, "klij");  // :743
    C(1.0, Vijka, "lkjc", false, T1, "ci", false, 1.0, Xklij, "klij");  // :744
    C(1.0, Xklij, "klij", false, X, "abkl", false, 1.0, R2, "abij");    // :747
    if (!dist) {
      C(1.0, Vijab, "klcd", false, X, "cdij", false, 0.0, Xklij, "klij");  // :751
    } else {
      CBuf<RB> Wq = cbuf(rb, {Nv, No, No, No});                   // :753
      C(1.0, Vijab, "klcd", false, T1, "dj", false, 0.0, Wq.v(), "cklj");
      C(1.0, T1, "ci", false, Wq.v(), "cklj", false, 0.0, Xklij, "klij");
    }
    if (o.ppl) C(1.0, Xklij, "klij", false, T2, "abkl", false, 1.0, R2, "abij");  // :764
    else C(1.0, Xklij, "klij", false, X, "abkl", false, 1.0, R2, "abij");         // :766
  }
  if (o.ppl) {
    // sliceCoupledCoulombIntegrals (ClusterSinglesDoublesAlgorithm.cxx:492-563)
    CBuf<RB> dGab = cbuf(rb, {NG, Nv, Nv}), dcGab = cbuf(rb, {NG, Nv, Nv});
    ccopy(rb, dGab.v(), Gab);
    C(-1.0, Gia, "Gkb", false, T1, "ak", false, 1.0, dGab.v(), "Gab");     // :534
    cassign(rb, 1.0, Gab, "Gba", true, 0.0, dcGab.v(), "Gab");
    C(-1.0, Gai, "Gbk", true, T1, "ak", false, 1.0, dcGab.v(), "Gab");     // :538-539
    const int64_t s = std::max<int64_t>(1, std::min<int64_t>(o.slice, Nv));
    for (int64_t b = 0; b < Nv; b += s) {                           // :823
      for (int64_t a = b; a < Nv; a += s) {                         // :824
        const int64_t nx = std::min(s, Nv - a), ny = std::min(s, Nv - b);
        CBuf<RB> left = cbuf(rb, {NG, nx, Nv}), right = cbuf(rb, {NG, ny, Nv});
        rb.gather_slice(left.re.v, dcGab.re.v, a, nx);              // :549-556
        rb.gather_slice(left.im.v, dcGab.im.v, a, nx);
        rb.gather_slice(right.re.v, dGab.re.v, b, ny);
        rb.gather_slice(right.im.v, dGab.im.v, b, ny);
        CBuf<RB> Vs = cbuf(rb, {nx, ny, Nv, Nv});                 // :560
        C(1.0, left.v(), "Gxc", false, right.v(), "Gyd", false, 0.0, Vs.v(), "xycd");
        CBuf<RB> Rxy = cbuf(rb, {nx, ny, No, No});                // :840
        C(1.0, Vs.v(), "xycd", false, X, "cdij", false, 0.0, Rxy.v(), "xyij");
        rb.slice_add(R2.re, Rxy.re.v, a, b, a > b);                 // :887-915
        rb.slice_add(R2.im, Rxy.im.v, a, b, a > b);
      }
    }
  }
  {
    C(1.0, Kac, "ac", false, T1, "ci", false, 1.0, R1, "ai");        // :862
    C(-1.0, Kki, "ki", false, T1, "ak", false, 1.0, R1, "ai");       // :863
    CBuf<RB> Kckb = cbuf(rb, {Nv, No});
    const CView Kck = Kckb.v();
    C(2.0, Vijab, "klcd", false, T1, "dl", false, 0.0, Kck, "ck");   // :866
    C(-1.0, Vijab, "kldc", false, T1, "dl", false, 1.0, Kck, "ck");  // :867
    C(2.0, Kck, "ck", false, T2, "caki", false, 1.0, R1, "ai");      // :870
    C(-1.0, Kck, "ck", false, T2, "caik", false, 1.0, R1, "ai");     // :871
    CBuf<RB> u = cbuf(rb, {No, No});                              // :872
    C(1.0, Kck, "ck", false, T1, "ci", false, 0.0, u.v(), "ki");
    C(1.0, T1, "ak", false, u.v(), "ki", false, 1.0, R1, "ai");
    C(2.0, Vaijb, "akic", false, T1, "ck", false, 1.0, R1, "ai");    // :873
    C(-1.0, Vaibj, "akci", false, T1, "ck", false, 1.0, R1, "ai");   // :874
    CBuf<RB> H = cbuf(rb, {NG, Nv, No});                          // :876-877
    C(1.0, Gia, "Gkd", false, X, "cdik", false, 0.0, H.v(), "Gci");
    C(2.0, Gab, "Gca", true, H.v(), "Gci", false, 1.0, R1, "ai");
    C(1.0, Gia, "Gkc", false, X, "cdik", false, 0.0, H.v(), "Gdi");  // :878-879
    C(-1.0, Gab, "Gda", true, H.v(), "Gdi", false, 1.0, R1, "ai");
    C(-2.0, Vijka, "klic", false, X, "ackl", false, 1.0, R1, "ai");  // :881
    C(1.0, Vijka, "lkic", false, X, "ackl", false, 1.0, R1, "ai");   // :882
  }
}

// ------------------------------------------------------------------ energy
struct Energy {
  std::complex<double> direct, exchange, noncanonical, value;
};

// getEnergy<complex> with Vijab (ClusterSinglesDoublesAlgorithm.cxx:131-189)
template <class RB>
Energy energy(RB &rb, const Inputs<RB> &I, const CView &T1, const CView &T2) {
  const double spins = 2.0;
  const CView Vijab = I.Vijab.v();
  CBuf<RB> s = cbuf(rb, {});
  CBuf<RB> w = cbuf(rb, {I.Nv, I.No});
  auto dot = [&](const CView &A, const char *ia, const CView &B, const char *ib) {
    ccontract(rb, 1.0, A, ia, false, B, ib, false, 0.0, s.v(), "");
    return cscalar(rb, s.v());
  };
  Energy e;
  // :170-172 direct
  std::complex<double> d = 0.5 * spins * spins * dot(T2, "abij", Vijab, "ijab");
  ccontract(rb, 1.0, T1, "ai", false, Vijab, "ijab", false, 0.0, w.v(), "bj");
  d = d + 0.5 * spins * spins * dot(T1, "bj", w.v(), "bj");
  // :175-177 exchange
  std::complex<double> x = (-0.5) * spins * dot(T2, "abij", Vijab, "ijba");
  ccontract(rb, 1.0, T1, "ai", false, Vijab, "ijba", false, 0.0, w.v(), "bj");
  x = x + (-0.5) * spins * dot(T1, "bj", w.v(), "bj");
  e.direct = d;
  e.exchange = x;
  e.value = d + x;                                                  // :189
  if (I.has_fock) {                                                 // :199-206
    e.noncanonical = spins * dot(T1, "ai", I.fock.v(), "ia");
    e.value += e.noncanonical;
  }
  return e;
}

// PairEnergy[i,j] (ClusterSinglesDoublesAlgorithm.cxx:227-232) for complex
// amplitudes: 2 X.V["ijab"] - X.V["ijba"] with X = T2 + T1T1, per (i, j).
// Both operands carry i and j, which the contraction engine does not take as
// batch indices, so the full [i,j,k,l] products are formed (No^4 entries) and
// their diagonal k = i, l = j is read on the host.  Returns p[i + No j].
template <class RB>
std::vector<std::complex<double>> pair_energy(RB &rb, const Inputs<RB> &I, const CView &T1,
                                              const CView &T2) {
  const int64_t No = I.No, Nv = I.Nv;
  CBuf<RB> X = cbuf(rb, {Nv, Nv, No, No});
  couter(rb, X.v(), T2, T1, 1.0);
  CBuf<RB> P1 = cbuf(rb, {No, No, No, No}), P2 = cbuf(rb, {No, No, No, No});
  ccontract(rb, 1.0, X.v(), "abij", false, I.Vijab.v(), "klab", false, 0.0, P1.v(), "ijkl");
  ccontract(rb, 1.0, X.v(), "abij", false, I.Vijab.v(), "klba", false, 0.0, P2.v(), "ijkl");
  const size_t n = (size_t)(No * No * No * No);
  std::vector<double> h1r(n), h1i(n), h2r(n), h2i(n);
  rb.read(P1.re.v, h1r.data());
  rb.read(P1.im.v, h1i.data());
  rb.read(P2.re.v, h2r.data());
  rb.read(P2.im.v, h2i.data());
  std::vector<std::complex<double>> p((size_t)(No * No));
  for (int64_t j = 0; j < No; ++j)
    for (int64_t i = 0; i < No; ++i) {
      const size_t d = (size_t)(i + No * (j + No * (i + No * j)));
      p[i + No * j] = 2.0 * std::complex<double>(h1r[d], h1i[d]) -
                      std::complex<double>(h2r[d], h2i[d]);
    }
  return p;
}

// ------------------------------------------------------------------ driver
struct SolveOpts {
  int max_iterations = 16;
  double energy_convergence = 1e-6, amplitudes_convergence = 1e-5;
  double level_shift = 0.0, mixing_ratio = 1.0;
  ResidualOpts res;
};

struct SolveResult {
  Energy energy;
  int iterations = 0;
  bool converged = false;
  std::vector<std::complex<double>> history;
};

// run<complex> with the linear mixer (ClusterSinglesDoublesAlgorithm.cxx:37-128,
// LinearMixer.cxx:30-44).  T holds the starting amplitudes on entry (zero or
// given) and the final ones on return; both are plane pairs of one Layout.
template <class RB>
SolveResult solve(RB &rb, const Inputs<RB> &I, const SolveOpts &o, CBuf<RB> &T) {
  const Layout L(I.Nv, I.No);
  auto t1 = [&](const CBuf<RB> &b) { return t1_of(b, L); };
  auto t2 = [&](const CBuf<RB> &b) { return t2_of(b, L); };
  CBuf<RB> R = cbuf(rb, {L.ntot}), E = cbuf(rb, {L.ntot}),
           D = cbuf(rb, {L.ntot}), Lres = cbuf(rb, {L.ntot});
  czero(rb, R.v());
  SolveResult out;
  std::complex<double> e = 0.0, prev = 0.0;
  bool have_last = false;
  for (int it = 0; it < o.max_iterations; ++it) {                   // :89
    residual(rb, I, it, o.res, t1(T), t2(T), t1(R), t2(R));         // :95
    double s_re[2], s_im[2];
    rb.jacobi(L, I.eps_h.v, I.eps_p.v, R.re.v, T.re.v, E.re.v, D.re.v, o.level_shift, s_re);
    rb.jacobi(L, I.eps_h.v, I.eps_p.v, R.im.v, T.im.v, E.im.v, D.im.v, o.level_shift, s_im);
    if (have_last && o.mixing_ratio != 1.0) {                       // LinearMixer.cxx:33-41
      rb.linear_mix(E.re.v, D.re.v, T.re.v, Lres.re.v, o.mixing_ratio, s_re);
      rb.linear_mix(E.im.v, D.im.v, T.im.v, Lres.im.v, o.mixing_ratio, s_im);
    }
    std::swap(T, E);                                                // amplitudes = last
    std::swap(Lres, D);
    have_last = true;
    const Energy en = energy(rb, I, t1(T), t2(T));                  // :102
    e = en.value;
    out.energy = en;
    out.history.push_back(e);
    out.iterations = it + 1;
    const double dtdt = s_re[0] + s_im[0], tt = s_re[1] + s_im[1];
    if (std::abs((e - prev) / e) < std::abs(o.energy_convergence) &&
        std::abs(dtdt / tt) <
            std::abs(o.amplitudes_convergence * o.amplitudes_convergence)) {  // :103-106
      out.converged = true;
      break;
    }
    prev = e;
  }
  if (o.max_iterations == 0) out.energy = energy(rb, I, t1(T), t2(T));  // :116-119
  return out;
}

// ---------------------------------------------------------------------- (T)
// view of the dense sub-block starting at element `offset`
inline View sub(const View &v, int64_t offset, std::initializer_list<int64_t> l) {
  return view(v.p + offset, l);
}
inline CView csub(const CView &v, int64_t offset, std::initializer_list<int64_t> l) {
  return CView{sub(v.re, offset, l), sub(v.im, offset, l)};
}

// Permutation<3>(p) images (src/math/Permutation.hpp:52-62)
inline std::array<int, 3> perm3(int p) {
  std::array<int, 3> img{};
  std::array<int, 2> s2{};
  {  // Permutation<2>(p / 3)
    const int r = (p / 3) % 2;
    s2[r] = 0;
    s2[1 - r] = 1;
  }
  const int r = p % 3;
  for (int i = 0; i < r; ++i) img[i] = s2[i] + 1;
  img[r] = 0;
  for (int i = r + 1; i < 3; ++i) img[i] = s2[i - 1] + 1;
  return img;
}

// s * pi: sPi[i] = s[pi(i)] (CcsdPerturbativeTriplesComplex.cxx:23-29)
inline std::string pstr(const std::string &s, const std::array<int, 3> &pi) {
  std::string r(s);
  for (int i = 0; i < 3; ++i) r[i] = s[pi[i]];
  return r;
}

// (T) of CcsdPerturbativeTriplesComplex::Calculator<complex>::calculate
// (src/algorithms/CcsdPerturbativeTriplesComplex.cxx:166-268) on the complex
// amplitudes T1 [Nv,No], T2 [Nv,Nv,No,No]; returns the complex E_(T)
template <class RB>
std::complex<double> triples(RB &rb, const Inputs<RB> &I, const CView &T1, const CView &T2) {
  const int64_t No = I.No, Nv = I.Nv;
  // Wvv[d,b,c,k] = sum_F conj(Gamma_Fdb) Gamma_Fck, built once (the reference
  // forms it per image, :342-348)
  CBuf<RB> Wvv = cbuf(rb, {Nv, Nv, Nv, No});
  ccontract(rb, 1.0, I.Gab.v(), "Fdb", true, I.Gai.v(), "Fck", false, 0.0, Wvv.v(), "dbck");
  // T2 as [a,b,l,i], so that T2[a,b,i,l] for fixed i is one dense block
  CBuf<RB> T2p = cbuf(rb, {Nv, Nv, No, No});
  cassign(rb, 1.0, T2, "abil", false, 0.0, T2p.v(), "abli");
  const CView Vabij = I.Vabij.v(), Vaijk = I.Vaijk.v();
  const int64_t n3 = Nv * Nv * Nv;
  std::vector<CBuf<RB>> piDV(6);
  for (auto &b : piDV) b = cbuf(rb, {Nv, Nv, Nv});
  CBuf<RB> DV = cbuf(rb, {Nv, Nv, Nv}), S = cbuf(rb, {Nv, Nv, Nv}), Tabc = cbuf(rb, {Nv, Nv, Nv});
  CBuf<RB> E = cbuf(rb, {});
  czero(rb, E.v());
  static const double spin_fermi[4] = {+2.0, -4.0, 0.0, +8.0};  // :181
  const std::string abc = "abc";
  std::array<std::array<int, 3>, 6> pi;
  for (int p = 0; p < 6; ++p) pi[p] = perm3(p);
  for (int64_t i0 = 0; i0 < No; ++i0)
    for (int64_t i1 = i0; i1 < No; ++i1)
      for (int64_t i2 = i1; i2 < No; ++i2) {
        const int64_t iv[3] = {i0, i1, i2};
        std::array<std::array<int64_t, 3>, 6> m;
        std::array<int, 6> src;
        for (int p = 0; p < 6; ++p) {
          for (int k = 0; k < 3; ++k) m[p][k] = iv[pi[p][k]];  // Map * Permutation
          src[p] = p;
          for (int q = 0; q < p; ++q)
            if (m[q] == m[p]) { src[p] = q; break; }       // :206-215
        }
        czero(rb, DV.v());
        for (int p = 0; p < 6; ++p) {
          if (src[p] == p) {
            const CView W = piDV[p].v();
            // getDoublesParticleContribution (:346-347)
            ccontract(rb, 1.0, csub(T2, (m[p][0] + No * m[p][1]) * Nv * Nv, {Nv, Nv}), "ad",
                      false, csub(Wvv.v(), m[p][2] * n3, {Nv, Nv, Nv}), "dbc", false, 0.0, W,
                      "abc");
            // addDoublesHoleContribution (:141): T_ab^{m0 l} V_{c l m2 m1}
            ccontract(rb, -1.0, csub(T2p.v(), m[p][0] * Nv * Nv * No, {Nv, Nv, No}), "abl",
                      false, csub(Vaijk, (m[p][2] + No * m[p][1]) * Nv * No, {Nv, No}), "cl",
                      false, 1.0, W, "abc");
          }
          // :221 DV["abc"] += piDV[p]["abc" * pi]
          cassign(rb, 1.0, piDV[src[p]].v(), pstr(abc, pi[p]).c_str(), false, 1.0, DV.v(),
                  "abc");
        }
        // :224-229 DV = conj(DV / D)
        rb.conj_over_denominator(DV.re.v, DV.im.v, I.eps_h.v, I.eps_p.v, i0, i1, i2);
        for (int p = 0; p < 6; ++p) {
          if (src[p] != p) continue;
          // getSinglesContribution (:148): 0.5 T_a^{m0} V_bc^{m1 m2}
          ccontract(rb, 0.5, csub(T1, m[p][0] * Nv, {Nv}), "a", false,
                    csub(Vabij, (m[p][1] + No * m[p][2]) * Nv * Nv, {Nv, Nv}), "bc", false,
                    0.0, S.v(), "abc");
          czero(rb, Tabc.v());
          for (int sg = 0; sg < 6; ++sg) {                          // :237-249
            const std::array<int, 3> &sigma = pi[sg];
            int fixed = 0;
            for (int k = 0; k < 3; ++k) fixed += sigma[k] == k;
            const double sf = spin_fermi[fixed];
            const std::string u = pstr(pstr(abc, sigma), pi[p]);
            cassign(rb, sf, piDV[p].v(), u.c_str(), false, 1.0, Tabc.v(), "abc");
            cassign(rb, sf, S.v(), u.c_str(), false, 1.0, Tabc.v(), "abc");
          }
          // :253 energy += DV["abc"] Tabc["abc"]
          ccontract(rb, 1.0, DV.v(), "abc", false, Tabc.v(), "abc", false, 1.0, E.v(), "");
        }
      }
  return cscalar(rb, E.v());
}

// ------------------------------------------------------- host-side flow
// Host inputs in the reference's layout; complex tensors are interleaved
// (re, im) pairs, as CTF stores complex<double>.
struct HostIn {
  int64_t No = 0, Nv = 0, NG = 0;
  const double *eps_h = nullptr, *eps_p = nullptr;  // [No], [Nv]
  const double *gamma = nullptr;                    // CoulombVertex [NG,Np,Np]
  const double *init_T1 = nullptr;                  // [Nv,No] or null
  const double *init_T2 = nullptr;                  // [Nv,Nv,No,No] or null
  const double *fock_hp = nullptr;                  // HPFockMatrix [No,Nv] or null
};

// Backend host transfers used here:
//   Buf load_real(host, lens)               upload a real tensor
//   load_complex(host, dst)                 interleaved host -> plane pair
//   store_complex(src, host)                plane pair -> interleaved host

template <class RB>
CView t1_of(const CBuf<RB> &b, const Layout &L) {
  return CView{view(b.re.v.p, {L.Nv, L.No}), view(b.im.v.p, {L.Nv, L.No})};
}
template <class RB>
CView t2_of(const CBuf<RB> &b, const Layout &L) {
  return CView{view(b.re.v.p + L.off2, {L.Nv, L.Nv, L.No, L.No}),
               view(b.im.v.p + L.off2, {L.Nv, L.Nv, L.No, L.No})};
}

// inputs, integrals and the starting amplitudes T (zero, or the given ones)
template <class RB>
bool setup(RB &rb, Inputs<RB> &I, const HostIn &h, CBuf<RB> &T) {
  if (h.No <= 0 || h.Nv <= 0 || h.NG <= 0 || !h.eps_h || !h.eps_p || !h.gamma)
    throw std::invalid_argument("No, Nv, NG, eigenenergies and the vertex are required");
  I.No = h.No;
  I.Nv = h.Nv;
  I.NG = h.NG;
  const int64_t Np = h.No + h.Nv;
  I.eps_h = rb.load_real(h.eps_h, {h.No});
  I.eps_p = rb.load_real(h.eps_p, {h.Nv});
  {
    CBuf<RB> G = cbuf(rb, {h.NG, Np, Np});
    rb.load_complex(h.gamma, G.v());
    build_inputs(rb, I, G.v());
  }
  const Layout L(h.Nv, h.No);
  T = cbuf(rb, {L.ntot});
  czero(rb, T.v());
  if (h.init_T1) rb.load_complex(h.init_T1, t1_of(T, L));
  if (h.init_T2) rb.load_complex(h.init_T2, t2_of(T, L));
  if (h.fock_hp) {
    I.has_fock = true;
    I.fock = cbuf(rb, {h.No, h.Nv});
    rb.load_complex(h.fock_hp, I.fock.v());
  }
  return h.init_T2 != nullptr;                   // createAmplitudes: initial doubles given
}

}  // namespace cx
}  // namespace gbcc
