// Closed-shell real CCSD on the GPU: inputs, residual, mixers, driver.
//
// The residual mirrors CcsdEnergyFromCoulombIntegrals::getResiduum (real
// path, src/algorithms/CcsdEnergyFromCoulombIntegrals.cxx:27-494) statement by
// statement; each `C(...)` below is one contraction-engine call (permutes +
// one GEMM) and is annotated with the reference line it replaces.  The order
// of the statements is kept, so that the terms added after the P(ia,jb)
// symmetrisation (:292) are not symmetrised.
#include <algorithm>
#include <cmath>
#include <limits>
#include <cstring>
#include <string>

#include "ccsd.hpp"

namespace gbcc {

namespace {
Ten T1v(const FockLayout &L, double *p) { return ten(p, {L.Nv, L.No}); }
Ten T2v(const FockLayout &L, double *p) {
  return ten(p + L.off2, {L.Nv, L.Nv, L.No, L.No});
}
constexpr int SC_UPD = 0;      // [0..17]  jacobi sums
constexpr int SC_EN = 20;      // [20..23] energy sums
constexpr int SC_TT = 24;      // amp.amp from DIIS combine
constexpr int SC_LAMBDA = 25;  // DIIS lambda
constexpr int SC_LIN = 26;     // [26..27] linear mix sums
constexpr int SC_FOCK = 28;    // T1.f (HPFockMatrix given)
constexpr int SC_STATUS = 30;  // DIIS status (as double)
constexpr int SC_N = 32;
}  // namespace

std::unique_ptr<CcsdInputs> upload_inputs(Context &ctx, const gbcc_ccsd_in &in,
                                          int precision, bool need_vaibj, bool stored) {
  require(in.No > 0 && in.Nv > 0, "No and Nv must be positive");
  require(in.eps_h && in.eps_p, "eigenenergies are required");
  // the stored formulation (CcsdEnergyFromCoulombIntegralsReference) takes
  // its integrals and needs no vertex when all of them are given
  const bool all_ints = in.Vabij && in.Vaibj && in.Vijkl && in.Vijka && in.Vabcd && in.Vabci;
  require(in.gamma != nullptr || (stored && all_ints), "CoulombVertex is required");
  require(in.gamma == nullptr || in.NG > 0, "NG must be positive");
  auto p = std::make_unique<CcsdInputs>();
  const int64_t No = in.No, Nv = in.Nv, NG = in.NG, Np = No + Nv;
  p->No = No; p->Nv = Nv; p->NG = NG;
  p->eps_h = OTen(ctx, {No});
  p->eps_p = OTen(ctx, {Nv});
  GBCC_CUDA(cudaMemcpyAsync(p->eps_h.p(), in.eps_h, 8 * No,
                            cudaMemcpyHostToDevice, ctx.stream));
  GBCC_CUDA(cudaMemcpyAsync(p->eps_p.p(), in.eps_p, 8 * Nv,
                            cudaMemcpyHostToDevice, ctx.stream));
  if (in.gamma) {
    OTen G(ctx, {NG, Np, Np});
    if (in.gamma_imag) {
      GBCC_CUDA(cudaMemcpyAsync(G.p(), in.gamma_imag, 8 * G.t.size(),
                                cudaMemcpyHostToDevice, ctx.stream));
      DBuf flag(ctx, sizeof(int));
      any_nonzero(ctx, G.p(), G.t.size(), flag.as<int>());
      int h = 0;
      GBCC_CUDA(cudaMemcpyAsync(&h, flag.as<int>(), sizeof(int),
                                cudaMemcpyDeviceToHost, ctx.stream));
      GBCC_CUDA(cudaStreamSynchronize(ctx.stream));
      if (h)
        throw Error(GBCC_COMPLEX_UNSUPPORTED,
                    "CoulombVertex has a non-zero imaginary part; only the real "
                    "closed-shell path is implemented");
    }
    GBCC_CUDA(cudaMemcpyAsync(G.p(), in.gamma, 8 * G.t.size(),
                              cudaMemcpyHostToDevice, ctx.stream));
    // slices of CcsdEnergyFromCoulombIntegrals.cxx:70-78
    p->Gai = OTen(ctx, {NG, Nv, No});
    p->Gab = OTen(ctx, {NG, Nv, Nv});
    p->Gij = OTen(ctx, {NG, No, No});
    vertex_block(ctx, p->Gai.p(), G.p(), NG, Np, No, Nv, 0, No);
    vertex_block(ctx, p->Gab.p(), G.p(), NG, Np, No, Nv, No, Nv);
    vertex_block(ctx, p->Gij.p(), G.p(), NG, Np, 0, No, 0, No);
  }
  auto up = [&](OTen &dst, const double *src, std::initializer_list<int64_t> l) {
    dst = OTen(ctx, l);
    GBCC_CUDA(cudaMemcpyAsync(dst.p(), src, 8 * dst.t.size(),
                              cudaMemcpyHostToDevice, ctx.stream));
  };
  // CoulombIntegralsFromVertex.cxx:395-417 for missing blocks
  if (in.Vabij) up(p->Vabij, in.Vabij, {Nv, Nv, No, No});
  else {
    p->Vabij = OTen(ctx, {Nv, Nv, No, No});
    contract(ctx, 1.0, p->Gai, "Gai", p->Gai, "Gbj", 0.0, p->Vabij, "abij", precision);
  }
  if (need_vaibj) {
    if (in.Vaibj) up(p->Vaibj, in.Vaibj, {Nv, No, Nv, No});
    else {
      p->Vaibj = OTen(ctx, {Nv, No, Nv, No});
      contract(ctx, 1.0, p->Gab, "Gab", p->Gij, "Gij", 0.0, p->Vaibj, "aibj", precision);
    }
    if (in.Vijkl) up(p->Vijkl, in.Vijkl, {No, No, No, No});
    else {
      p->Vijkl = OTen(ctx, {No, No, No, No});
      contract(ctx, 1.0, p->Gij, "Gik", p->Gij, "Gjl", 0.0, p->Vijkl, "ijkl", precision);
    }
  }
  if (in.Vijka) up(p->Vijka, in.Vijka, {No, No, No, Nv});
  else {
    p->Vijka = OTen(ctx, {No, No, No, Nv});
    contract(ctx, 1.0, p->Gij, "Gik", p->Gai, "Gaj", 0.0, p->Vijka, "ijka", precision);
  }
  p->Vx = OTen(ctx, {Nv, Nv, No, No});
  assign(ctx, 1.0, p->Vabij, "baij", 0.0, p->Vx, "abij");
  if (stored) {
    // CoulombIntegralsFromVertex.cxx:423-431
    if (in.Vabcd) up(p->Vabcd, in.Vabcd, {Nv, Nv, Nv, Nv});
    else {
      p->Vabcd = OTen(ctx, {Nv, Nv, Nv, Nv});
      contract(ctx, 1.0, p->Gab, "Gac", p->Gab, "Gbd", 0.0, p->Vabcd, "abcd", precision);
    }
    if (in.Vabci) up(p->Vabci, in.Vabci, {Nv, Nv, Nv, No});
    else {
      p->Vabci = OTen(ctx, {Nv, Nv, Nv, No});
      contract(ctx, 1.0, p->Gab, "Gac", p->Gai, "Gbi", 0.0, p->Vabci, "abci", precision);
    }
  }
  // unchanged for the solver's life: their digit panels are split once
  p->ctx = &ctx;
  for (const OTen *t : {&p->Vabij, &p->Vx, &p->Vaibj, &p->Vijkl, &p->Vijka, &p->Gai,
                        &p->Gab, &p->Gij})
    if (t->p()) ctx.register_constant(t->p(), sizeof(double) * (size_t)t->t.size());
  if (in.fock_hp) {
    // f[i,a] is kept as f[a,i], so the noncanonical energy term is a plain
    // dot with T1[a,i]
    std::vector<double> fai((size_t)(Nv * No));
    for (int64_t i = 0; i < No; ++i)
      for (int64_t a = 0; a < Nv; ++a) fai[a + Nv * i] = in.fock_hp[i + No * a];
    up(p->fock_ai, fai.data(), {Nv, No});
    // fai is freed at the end of this block: the copy must have read it
    GBCC_CUDA(cudaStreamSynchronize(ctx.stream));
  }
  return p;
}

CcsdInputs::~CcsdInputs() {
  if (!ctx) return;
  for (const OTen *t : {&Vabij, &Vx, &Vaibj, &Vijkl, &Vijka, &Gai, &Gab, &Gij})
    if (t->p()) ctx->forget_constant(t->p());
}

Ccsd::Ccsd(Context &ctx, std::unique_ptr<CcsdInputs> in,
           const gbcc_ccsd_opts &o, const double *init_T1_host,
           const double *init_T2_host)
    : ctx_(ctx), in_(std::move(in)), o_(o), L_(in_->Nv, in_->No) {
  require(o_.max_residua >= 1 && o_.max_residua <= GBCC_MAX_DIIS,
          "maxResidua must be in [1, 16]");
  require(o_.mixer == 0 || o_.mixer == 1, "mixer must be LinearMixer or DiisMixer");
  const int64_t Nv = L_.Nv, No = L_.No;
  // integralsSliceSize (CcsdEnergyFromCoulombIntegrals.cxx:375-385)
  if (o_.integrals_slice_size > 0) slice_ = o_.integrals_slice_size;
  else if (o_.integrals_slice_factor >= 0) slice_ = (int64_t)(Nv * o_.integrals_slice_factor);
  else {
    // device default: Nv / 8 (at least 16), capped so that V_xycd plus its
    // digit panels stay within 4 GiB.  Slice pairs m <= n redo the diagonal
    // blocks, so smaller slices do less redundant ladder work (1/(2 ns) of
    // the a >= b half) while Nv / 8 keeps the GEMMs large; the energy does
    // not depend on the slicing
    const double budget = 4.0 * 1024 * 1024 * 1024 / 16.0;
    const int64_t cap = (int64_t)std::floor(std::sqrt(budget / (double)(Nv * Nv)));
    slice_ = std::min<int64_t>(cap, std::max<int64_t>(16, Nv / 8));
  }
  slice_ = std::max<int64_t>(1, std::min<int64_t>(slice_, Nv));
  const size_t fb = sizeof(double) * L_.ntot;
  T_.alloc(ctx_, fb);
  R_.alloc(ctx_, fb);
  fill(ctx_, T_.as<double>(), L_.ntot, 0.0);
  if (init_T1_host)
    GBCC_CUDA(cudaMemcpyAsync(T_.as<double>(), init_T1_host, 8 * L_.n1,
                              cudaMemcpyHostToDevice, ctx_.stream));
  if (init_T2_host) {
    GBCC_CUDA(cudaMemcpyAsync(T_.as<double>() + L_.off2, init_T2_host,
                              8 * L_.n2, cudaMemcpyHostToDevice, ctx_.stream));
    init_doubles_ = true;
  }
  if (init_T1_host || init_T2_host) {  // kept for restart()
    T0_.alloc(ctx_, fb);
    copy(ctx_, T0_.as<double>(), T_.as<double>(), L_.ntot);
  }
  (void)No;
  const int nb = reduction_blocks(ctx_, L_.ntot);
  partials_.alloc(ctx_, sizeof(double) * nb * (2 + GBCC_MAX_DIIS + 4));
  scal_.alloc(ctx_, sizeof(double) * SC_N);
  fill(ctx_, scal_.as<double>(), SC_N, 0.0);
  if (o_.mixer == 1) {
    const int N = o_.max_residua;
    slotA_.resize(N);
    slotD_.resize(N);
    B_.alloc(ctx_, sizeof(double) * (N + 1) * (N + 1));
    std::vector<double> b((N + 1) * (N + 1), 0.0);
    for (int i = 1; i <= N; ++i) b[0 + (N + 1) * i] = b[i + 0] = -1.0;  // DiisMixer.cxx:68-96
    GBCC_CUDA(cudaMemcpyAsync(B_.as<double>(), b.data(), 8 * b.size(),
                              cudaMemcpyHostToDevice, ctx_.stream));
    w_.alloc(ctx_, sizeof(double) * GBCC_MAX_DIIS);
    hist_slot_.alloc(ctx_, sizeof(int) * GBCC_MAX_DIIS * 2);
  } else {
    E_.alloc(ctx_, fb);
    D_.alloc(ctx_, fb);
    Lres_.alloc(ctx_, fb);
  }
  GBCC_CUDA(cudaMallocHost(&pinned_, sizeof(double) * SC_N));
}

Ccsd::~Ccsd() {
  cudaStreamSynchronize(ctx_.stream);
  for (auto &g : graphs_)
    if (g.exec) cudaGraphExecDestroy(g.exec);
  if (pinned_) cudaFreeHost(pinned_);
}

void Ccsd::pair_energies(double *dev_out) {
  double *T = T_.as<double>();
  gbcc::pair_energy(ctx_, T, T + L_.off2, in_->Vabij.p(), in_->Vx.p(), L_.Nv,
                    L_.No, dev_out);
}

void Ccsd::residual(int it, const double *Tp, double *Rp) {
  if (o_.formulation == 1) {  // CcsdEnergyFromCoulombIntegralsReference
    residual_stored(it, Tp, Rp);
    return;
  }
  fill(ctx_, Rp, L_.ntot, 0.0);                                    // :37-38
  ResidualArgs a;
  a.I = in_.get();
  a.o = &o_;
  a.nz = 1;
  a.slice = slice_;
  a.init_doubles = init_doubles_;
  a.T1 = T1v(L_, const_cast<double *>(Tp));
  a.T2 = T2v(L_, const_cast<double *>(Tp));
  a.R1 = T1v(L_, Rp);
  a.R2 = T2v(L_, Rp);
  residual_program(ctx_, a, it);
}

// The statements of getResiduum over nz systems of one shape at once.  With
// nz > 1 every tensor (amplitudes, residuals, inputs and intermediates)
// carries a trailing system index Z, its slowest, so each system's data is
// one contiguous block and every contraction below is one batched product
// (a grouped tensor-core launch in precision mode).  R arrives zeroed.
void residual_program(Context &ctx, const ResidualArgs &ra, int it) {
  const CcsdInputs &I = *ra.I;
  const gbcc_ccsd_opts &o = *ra.o;
  const int prec = o.precision;
  const int64_t nz = ra.nz;
  const int64_t No = I.No, Nv = I.Nv, NG = I.NG;
  const int64_t n2 = Nv * Nv * No * No;
  const bool dist = o.distinguishable != 0;
  // index strings and shapes gain the system index when nz > 1
  auto ix = [&](const char *s) { return nz > 1 ? std::string(s) + "Z" : std::string(s); };
  auto C = [&](double al, const Ten &A, const char *ia, const Ten &B,
               const char *ib, double be, const Ten &Cc, const char *ic) {
    contract(ctx, al, A, ix(ia).c_str(), B, ix(ib).c_str(), be, Cc, ix(ic).c_str(), prec);
  };
  auto shp = [&](std::initializer_list<int64_t> l) {
    std::vector<int64_t> v(l);
    if (nz > 1) v.push_back(nz);
    return v;
  };
  const Ten &T1 = ra.T1, &T2 = ra.T2, &R1 = ra.R1, &R2 = ra.R2;
  const Ten &V = I.Vabij, &Vx = I.Vx;
  if (it == 0 && !ra.init_doubles) {                               // :47-51
    copy(ctx, R2.p, V.p, n2 * nz);
    return;
  }
  const Ten &Vaibj = I.Vaibj, &Vijkl = I.Vijkl, &Vijka = I.Vijka;
  const Ten &Gai = I.Gai, &Gab = I.Gab, &Gij = I.Gij;

  OTen X(ctx, shp({Nv, Nv, No, No}));                                   // :136-138
  outer_add(ctx, X.p(), T2.p, T1.p, 1.0, Nv, No, nz);
  // T1, T2 and X stay unchanged until the residual is complete: operands
  // taken from them in the same layout are split once
  FrozenScope frozen(ctx);
  frozen.add(T1.p, sizeof(double) * (size_t)T1.size());
  frozen.add(T2.p, sizeof(double) * (size_t)T2.size());
  frozen.add(X.p(), sizeof(double) * (size_t)X.t.size());
  OTen Kac(ctx, shp({Nv, Nv})), Kki(ctx, shp({No, No}));
  {
    OTen Lac(ctx, shp({Nv, Nv})), Lki(ctx, shp({No, No}));
    C(-2.0, V, "cdkl", X, "adkl", 0.0, Kac, "ac");                 // :146
    C(1.0, Vx, "cdkl", X, "adkl", 1.0, Kac, "ac");                 // :147 V["dckl"]
    if (!dist) copy(ctx, Lac.p(), Kac.p(), Nv * Nv * nz);               // :151
    else {
      OTen Y(ctx, shp({Nv, Nv, No, No}));                               // :154-156
      outer_add(ctx, Y.p(), T2.p, T1.p, 2.0, Nv, No, nz);
      C(-1.0, V, "cdkl", Y, "adkl", 0.0, Lac, "ac");               // :157-158
      C(0.5, Vx, "cdkl", Y, "adkl", 1.0, Lac, "ac");               // :159-160
    }
    {
      OTen t(ctx, shp({NG}));                                           // :162-163
      C(1.0, Gai, "Gdk", T1, "dk", 0.0, t, "G");
      C(2.0, Gab, "Gca", t, "G", 1.0, Lac, "ac");
      OTen Q(ctx, shp({NG, Nv, No}));                                   // :166-167
      C(1.0, Gab, "Gda", T1, "dk", 0.0, Q, "Gak");
      C(-1.0, Gai, "Gck", Q, "Gak", 1.0, Lac, "ac");
    }
    C(2.0, V, "cdkl", X, "cdil", 0.0, Kki, "ki");                  // :172
    C(-1.0, Vx, "cdkl", X, "cdil", 1.0, Kki, "ki");                // :173 V["dckl"]
    if (!dist) copy(ctx, Lki.p(), Kki.p(), No * No * nz);               // :177
    else {
      OTen Y(ctx, shp({Nv, Nv, No, No}));                               // :180-182
      outer_add(ctx, Y.p(), T2.p, T1.p, 2.0, Nv, No, nz);
      C(1.0, V, "cdkl", Y, "cdil", 0.0, Lki, "ki");                // :183-184
      C(-0.5, Vx, "cdkl", Y, "cdil", 1.0, Lki, "ki");              // :185-186
    }
    C(2.0, Vijka, "klic", T1, "cl", 1.0, Lki, "ki");               // :188
    C(-1.0, Vijka, "lkic", T1, "cl", 1.0, Lki, "ki");              // :189
    C(1.0, Lac, "ac", T2, "cbij", 1.0, R2, "abij");                // :192
    C(-1.0, Lki, "ki", T2, "abkj", 1.0, R2, "abij");               // :195
  }
  {
    OTen dGai(ctx, shp({NG, Nv, No}));                                  // :200-206
    copy(ctx, dGai.p(), Gai.p, Gai.size());
    C(-1.0, Gij, "Gki", T1, "ak", 1.0, dGai, "Gai");
    OTen Z(ctx, shp({NG, Nv, No}));                                     // :208-209
    C(1.0, Gab, "Gbc", T1, "cj", 0.0, Z, "Gbj");
    C(1.0, dGai, "Gai", Z, "Gbj", 1.0, R2, "abij");
    C(-1.0, Vijka, "jika", T1, "bk", 1.0, R2, "abij");             // :213
    OTen W(ctx, shp({Nv, No, No, No}));                                 // :214-215
    C(1.0, V, "acik", T1, "cj", 0.0, W, "aikj");
    C(-1.0, T1, "bk", W, "aikj", 1.0, R2, "abij");
  }
  {
    OTen Xakic(ctx, shp({Nv, No, No, Nv}));                             // :218-252
    {
      OTen dGai(ctx, shp({NG, Nv, No}));                                // :222-231
      copy(ctx, dGai.p(), Gai.p, Gai.size());
      C(-1.0, Gij, "Gil", T1, "al", 1.0, dGai, "Gai");
      C(1.0, Gab, "Gad", T1, "di", 1.0, dGai, "Gai");
      C(1.0, dGai, "Gai", Gai, "Gck", 0.0, Xakic, "akic");         // :234-235
    }
    OTen Y(ctx, shp({Nv, Nv, No, No}));                                 // :238-240
    outer_add(ctx, Y.p(), T2.p, T1.p, 2.0, Nv, No, nz);
    C(-0.5, V, "dclk", Y, "dail", 1.0, Xakic, "akic");             // :242
    C(1.0, V, "dclk", T2, "adil", 1.0, Xakic, "akic");             // :243
    if (!dist) C(-0.5, V, "cdlk", T2, "adil", 1.0, Xakic, "akic"); // :245
    axpby(ctx, n2 * nz, 2.0, T2.p, 0.0, Y.p());                      // :248
    assign(ctx, -1.0, T2, ix("bckj").c_str(), 1.0, Y, ix("cbkj").c_str());                 // :249
    C(1.0, Xakic, "akic", Y, "cbkj", 1.0, R2, "abij");             // :251
  }
  {
    OTen Xakci(ctx, shp({Nv, No, Nv, No}));                             // :254-293
    {
      OTen dGab(ctx, shp({NG, Nv, Nv})), dGij(ctx, shp({NG, No, No}));
      copy(ctx, dGab.p(), Gab.p, Gab.size());
      copy(ctx, dGij.p(), Gij.p, Gij.size());
      C(-1.0, Gai, "Gcl", T1, "al", 1.0, dGab, "Gac");             // :270
      C(1.0, Gai, "Gdk", T1, "di", 1.0, dGij, "Gki");              // :273
      C(1.0, dGab, "Gac", dGij, "Gki", 0.0, Xakci, "akci");        // :277-280
    }
    if (!dist) C(-0.5, V, "cdlk", T2, "dail", 1.0, Xakci, "akci"); // :284
    C(-1.0, Xakci, "akci", T2, "cbkj", 1.0, R2, "abij");           // :288
    C(-1.0, Xakci, "bkci", T2, "ackj", 1.0, R2, "abij");           // :289
    OTen Rc(ctx, shp({Nv, Nv, No, No}));                                // :292
    copy(ctx, Rc.p(), R2.p, n2 * nz);
    assign(ctx, 1.0, Rc, ix("baji").c_str(), 1.0, R2, ix("abij").c_str());
  }
  axpby(ctx, n2 * nz, 1.0, V.p, 1.0, R2.p);                          // :301
  {
    OTen Xklij(ctx, shp({No, No, No, No}));                             // :305-333
    copy(ctx, Xklij.p(), Vijkl.p, No * No * No * No * nz);              // :308
    C(1.0, Vijka, "klic", T1, "cj", 1.0, Xklij, "klij");           // :309
    C(1.0, Vijka, "lkjc", T1, "ci", 1.0, Xklij, "klij");           // :310
    C(1.0, Xklij, "klij", X, "abkl", 1.0, R2, "abij");             // :313
    if (!dist) C(1.0, V, "cdkl", X, "cdij", 0.0, Xklij, "klij");   // :317
    else {
      OTen Wq(ctx, shp({Nv, No, No, No}));                              // :319
      C(1.0, V, "cdkl", T1, "dj", 0.0, Wq, "cklj");
      C(1.0, T1, "ci", Wq, "cklj", 0.0, Xklij, "klij");
    }
    if (o.ppl) C(1.0, Xklij, "klij", T2, "abkl", 1.0, R2, "abij");  // :330
    else C(1.0, Xklij, "klij", X, "abkl", 1.0, R2, "abij");          // :332
  }
  if (o.ppl) {                                                    // :374-452
    // the ladder holds the largest temporaries: no kept panels meanwhile
    ctx.drop_frozen_panels();
    OTen dG(ctx, shp({NG, Nv, Nv}));                               // :392-400
    copy(ctx, dG.p(), Gab.p, Gab.size());
    C(-1.0, Gai, "Gbk", T1, "ak", 1.0, dG, "Gab");
    const int64_t s = ra.slice;
    const int64_t ns = (Nv + s - 1) / s;                           // :387
    std::vector<OTen> sl;                                          // :402-416
    for (int64_t v = 0; v < ns; ++v) {
      const int64_t x0 = v * s, nx = std::min(s, Nv - x0);
      sl.emplace_back(ctx, shp({NG, nx, Nv}));
      gather_slice(ctx, sl.back().p(), dG.p(), NG, Nv, x0, nx, nz);
    }
    // precision mode: X[c,d,i,j] (rows ij, K = cd) is the B operand of every
    // slice pair's R = V.X, so its digit panels are split once
    const bool emu = prec == GBCC_PREC_EMU;
    auto emulated = [&](int64_t M, int64_t N, int64_t K) {
      return emu && 2.0 * (double)M * (double)N * (double)K >= ctx.emu_min_flops;
    };
    // Fused form (every pair emulated, Nv a multiple of 8): each V block
    // goes from the tensor cores straight into the digit panels of R = V.X,
    // its row exponents bounded in advance from the column norms of the
    // dressed vertex (Cauchy-Schwarz), so V never exists in FP64 and is
    // neither re-read for its exponents nor re-split.  The V product then
    // takes its B operand as [G, d, y] and R sums over k = d + Nv c, so X
    // enters as X'[d,c,i,j] = X[c,d,i,j].
    const int64_t s_last = Nv - (ns - 1) * s;
    // (over a batch, when one system's V block alone fills half the GPU
    // with output tiles; smaller ladders run as batched products below)
    const int64_t vtiles = ((s * Nv + 127) / 128) * ((s * Nv + 63) / 64);
    const bool fused = (nz == 1 || 2 * vtiles >= ctx.sm_count) && Nv % 8 == 0 &&
                       emulated(s_last * Nv, s_last * Nv, NG) &&
                       emulated(s_last * s_last, No * No, Nv * Nv);
    if (fused) {
      // system by system over a batch (each system's V blocks fill the GPU)
      for (int64_t z = 0; z < nz; ++z) {
        const int64_t sz_dG = NG * Nv * Nv;
        DBuf amax(ctx, sizeof(unsigned long long) * Nv);
        ladder_amax(ctx, dG.p() + z * sz_dG, NG, Nv, amax.as<void>());
        // every slice's digit panels, split once for all its slice pairs: as
        // the A operand sl[G,(x,c)] and, transposed, as the B operand
        // slT[G,(d,y)]
        std::vector<EmuPanels> slA, slB;
        for (int64_t v = 0; v < ns; ++v) {
          const int64_t nx = sl[v].t.lens[1];
          double *slz = sl[v].p() + z * NG * nx * Nv;
          {
            OTen slT(ctx, {NG, Nv, nx});
            assign(ctx, 1.0, ten(slz, {NG, nx, Nv}), "Gyd", 0.0, slT, "Gdy");
            slB.push_back(emu_split(ctx, false, slT.p(), nx * Nv, NG, NG, 1, 1, 0));
          }
          slA.push_back(emu_split(ctx, true, slz, nx * Nv, NG, NG, 1, 1, 0));
        }
        EmuPanels Xq;
        {
          OTen Xt(ctx, {Nv, Nv, No, No});
          assign(ctx, 1.0, ten(X.p() + z * n2, {Nv, Nv, No, No}), "cdij", 0.0, Xt, "dcij");
          Xq = emu_split(ctx, false, Xt.p(), No * No, Nv * Nv, Nv * Nv, 1, 1, 0);
        }
        for (int64_t m = 0; m < ns; ++m) {                         // :418
          for (int64_t n = m; n < ns; ++n) {                       // :419
            const int64_t nx = sl[n].t.lens[1], ny = sl[m].t.lens[1];
            const int64_t a0 = n * s, b0 = m * s;
            EmuPanels Vp = emu_panels_alloc(ctx, true, nx * ny, Nv * Nv);
            ladder_row_exponents(ctx, amax.as<void>(), a0, nx, b0, ny, Vp.exps.as<int>());
            // V[(x,c),(d,y)] = sum_G sl_n[G,(x,c)] slT_m[G,(d,y)]   :425-434
            emu_gemm_panels_to_panels(ctx, slA[n], 0, slB[m], 0, nx, Nv, Vp);
            OTen Rxy(ctx, {nx, ny, No, No});                       // :443
            emu_gemm_panels(ctx, Vp, 0, Xq, 0, 1.0, 0.0, Rxy.p(), nx * ny);
            slice_add(ctx, R2.p + z * n2, Rxy.p(), Nv, No, a0, b0, nx, ny,
                      a0 > b0);                                    // :444-447
          }
        }
      }
    }
    EmuPanels Xp;
    if (!fused && nz == 1 && emulated(s * s, No * No, Nv * Nv))
      Xp = emu_split(ctx, false, X.p(), No * No, Nv * Nv, Nv * Nv, 1, 1, 0);
    for (int64_t m = 0; m < ns && !fused; ++m) {                   // :418
      for (int64_t n = m; n < ns; ++n) {                           // :419
        const int64_t nx = sl[n].t.lens[1], ny = sl[m].t.lens[1];
        OTen Vs(ctx, shp({nx, ny, Nv, Nv}));                       // :425-434
        if (nz == 1 && emulated(nx * Nv, ny * Nv, NG)) {
          // V[(x,c),(y,d)] = sum_G sl_n[G,(x,c)] sl_m[G,(y,d)], written
          // straight into the V[x,y,c,d] layout of the next product
          const OutMap vmap{nx, 1, nx * ny, ny, nx, nx * ny * Nv};
          gemm_emu_mapped(ctx, true, false, nx * Nv, ny * Nv, NG, 1.0, sl[n].p(), NG,
                          sl[m].p(), NG, Vs.p(), vmap);
        } else {
          C(1.0, sl[n], "Gxc", sl[m], "Gyd", 0.0, Vs, "xycd");
        }
        OTen Rxy(ctx, shp({nx, ny, No, No}));                      // :443
        if (Xp.count > 0 && emulated(nx * ny, No * No, Nv * Nv)) {
          const EmuPanels Vp = emu_split(ctx, true, Vs.p(), nx * ny, Nv * Nv, 1, nx * ny, 1, 0);
          emu_gemm_panels(ctx, Vp, 0, Xp, 0, 1.0, 0.0, Rxy.p(), nx * ny);
        } else {
          C(1.0, Vs, "xycd", X, "cdij", 0.0, Rxy, "xyij");
        }
        const int64_t a0 = n * s, b0 = m * s;                      // :444-447
        slice_add(ctx, R2.p, Rxy.p(), Nv, No, a0, b0, nx, ny, a0 > b0, nz);
      }
    }
  }
  {
    C(1.0, Kac, "ac", T1, "ci", 1.0, R1, "ai");                    // :466
    C(-1.0, Kki, "ki", T1, "ak", 1.0, R1, "ai");                   // :467
    OTen Kck(ctx, shp({Nv, No}));
    C(2.0, V, "cdkl", T1, "dl", 0.0, Kck, "ck");                   // :470
    C(-1.0, Vx, "cdkl", T1, "dl", 1.0, Kck, "ck");                 // :471 V["dckl"]
    C(2.0, Kck, "ck", T2, "caki", 1.0, R1, "ai");                  // :474
    C(-1.0, Kck, "ck", T2, "caik", 1.0, R1, "ai");                 // :475
    OTen u(ctx, shp({No, No}));                                         // :476
    C(1.0, Kck, "ck", T1, "ci", 0.0, u, "ki");
    C(1.0, T1, "ak", u, "ki", 1.0, R1, "ai");
    C(2.0, V, "acik", T1, "ck", 1.0, R1, "ai");                    // :477
    C(-1.0, Vaibj, "ciak", T1, "ck", 1.0, R1, "ai");               // :478
    OTen H(ctx, shp({NG, Nv, No}));                                     // :480-483
    C(1.0, Gai, "Gdk", X, "cdik", 0.0, H, "Gci");
    C(2.0, Gab, "Gca", H, "Gci", 1.0, R1, "ai");
    C(1.0, Gai, "Gck", X, "cdik", 0.0, H, "Gdi");                  // :484-487
    C(-1.0, Gab, "Gda", H, "Gdi", 1.0, R1, "ai");
    C(-2.0, Vijka, "klic", X, "ackl", 1.0, R1, "ai");              // :489
    C(1.0, Vijka, "lkic", X, "ackl", 1.0, R1, "ai");               // :490
  }
}

// Device work of one iteration for the current host state (mixer position,
// DIIS count, buffer parity); it only reads that state, so that it can be
// captured into a CUDA graph and replayed for every later iteration that
// starts from the same state.
void Ccsd::iteration_body() {
  residual(it_, T_.as<double>(), R_.as<double>());                 // :95
  mix_body();
}

// the device work of an iteration after the residual: update, mixer, energy
// sums and their copy to the host
void Ccsd::mix_body() {
  Context &ctx = ctx_;
  double *sc = scal_.as<double>();
  const int64_t n = L_.ntot;
  double *amp = nullptr;
  if (o_.mixer == 1) {                                             // DiisMixer
    const int N = o_.max_residua;
    const int k = next_;
    std::vector<const double *> hist;
    std::vector<int> hslot;
    // slots filled since the start (or the last restart): 0 .. count_-1
    // while the ring fills, all of them once it is full
    for (int i = 0; i < N; ++i)
      if (i != k && i < count_) {
        hist.push_back(slotD_[i].as<double>());
        hslot.push_back(i);
      }
    jacobi_update(ctx, L_, R_.as<double>(), T_.as<double>(),
                  slotA_[k].as<double>(), slotD_[k].as<double>(),
                  in_->eps_h.p(), in_->eps_p.p(), o_.level_shift,
                  (int)hist.size(), hist.data(), partials_.as<double>(),
                  sc + SC_UPD);                                    // :96-98
    const int count = std::min(count_ + 1, N);                     // DiisMixer.cxx:141
    // status as int in the double slot SC_STATUS (reinterpreted)
    diis_solve(ctx, B_.as<double>(), N, k, count, sc + SC_UPD,
               (int)hslot.size(), hslot.data(), w_.as<double>(),
               sc + SC_LAMBDA, reinterpret_cast<int *>(sc + SC_STATUS));
    std::vector<const double *> src;
    for (int j = 0; j < count; ++j) src.push_back(slotA_[(k + N - j) % N].as<double>());
    diis_combine(ctx, count, src.data(), w_.as<double>(), T_.as<double>(), n,
                 partials_.as<double>(), sc + SC_TT);              // :160-174
    amp = T_.as<double>();
  } else {                                                         // LinearMixer
    jacobi_update(ctx, L_, R_.as<double>(), T_.as<double>(), E_.as<double>(),
                  D_.as<double>(), in_->eps_h.p(), in_->eps_p.p(),
                  o_.level_shift, 0, nullptr, partials_.as<double>(),
                  sc + SC_UPD);
    if (have_last_ && o_.mixing_ratio != 1.0) {
      linear_mix(ctx, E_.as<double>(), D_.as<double>(), T_.as<double>(),
                 Lres_.as<double>(), o_.mixing_ratio, n,
                 partials_.as<double>(), sc + SC_LIN);
      // convergence sums come from the mixed vectors
      copy(ctx, sc + SC_UPD, sc + SC_LIN, 2);
    }
    amp = E_.as<double>();                                         // becomes T below
  }
  energy_sums(amp);                                                // :102
  GBCC_CUDA(cudaMemcpyAsync(pinned_, sc, sizeof(double) * SC_N,
                            cudaMemcpyDeviceToHost, ctx.stream));
}

// the device sums getEnergy needs for the amplitudes at amp (T1 then T2)
void Ccsd::energy_sums(const double *amp) {
  Context &ctx = ctx_;
  double *sc = scal_.as<double>();
  energy_terms(ctx, amp, amp + L_.off2, in_->Vabij.p(), in_->Vx.p(), L_.Nv,
               L_.No, partials_.as<double>(), sc + SC_EN);
  if (in_->fock_ai.p())                                            // :199-202
    gemm(ctx, false, false, 1, 1, L_.Nv * L_.No, 1.0, amp, 1, in_->fock_ai.p(),
         L_.Nv * L_.No, 0.0, sc + SC_FOCK, 1);
}

// getEnergy (ClusterSinglesDoublesAlgorithm.cxx:131-209) from the sums
void Ccsd::energy_from_sums(const double *h, IterInfo &info) const {
  const double spins = 2.0;
  double d = 0.5 * spins * spins * h[SC_EN + 0];                   // :170-172
  d = d + 0.5 * spins * spins * h[SC_EN + 1];
  double x = (-0.5) * spins * h[SC_EN + 2];                        // :175-177
  x = x + (-0.5) * spins * h[SC_EN + 3];
  info.direct = d;
  info.exchange = x;
  info.energy = d + x;                                             // :189
  if (in_->fock_ai.p()) {                                          // :202-206
    info.noncanonical = spins * h[SC_FOCK];
    info.energy += info.noncanonical;
  }
}

void Ccsd::evaluate_energy() {
  // ClusterSinglesDoublesAlgorithm.cxx:116-119: with maxIterations 0 the
  // energy of the given amplitudes is reported
  Context &ctx = ctx_;
  energy_sums(T_.as<double>());
  GBCC_CUDA(cudaMemcpyAsync(pinned_, scal_.as<double>(), sizeof(double) * SC_N,
                            cudaMemcpyDeviceToHost, ctx.stream));
  ctx.check_device_errors();
  IterInfo info;
  energy_from_sums(pinned_, info);
  e_ = info.energy;
  dir_ = info.direct;
  exc_ = info.exchange;
}

// graph key of the state the next iteration starts from (-1: run eagerly);
// allocates the DIIS slot that iteration writes
int Ccsd::graph_key() {
  Context &ctx = ctx_;
  const int64_t n = L_.ntot;
  int key = -1;
  if (o_.mixer == 1) {
    const int k = next_;
    if (!slotA_[k].bytes()) {
      slotA_[k].alloc(ctx, 8 * n);
      slotD_[k].alloc(ctx, 8 * n);
    }
    if (count_ == o_.max_residua && it_ >= 1) key = k;
  } else if (have_last_ && it_ >= 1) {
    key = (int)(swaps_ & 1);
  }
  return key;
}

IterInfo Ccsd::iterate() {
  Context &ctx = ctx_;
  const int key = graph_key();
  if (key >= 0 && ctx.use_graphs && !ctx.prof) {
    if ((int)graphs_.size() <= key) graphs_.resize(key + 1);
    Graph &g = graphs_[key];
    if (!g.exec) {
      const uint64_t l0 = ctx.launches;
      const double f0 = ctx.flops;
      GBCC_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
      try {
        iteration_body();
      } catch (...) {
        cudaGraph_t bad = nullptr;
        cudaStreamEndCapture(ctx.stream, &bad);
        if (bad) cudaGraphDestroy(bad);
        throw;
      }
      cudaGraph_t graph = nullptr;
      GBCC_CUDA(cudaStreamEndCapture(ctx.stream, &graph));
      const cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
      cudaGraphDestroy(graph);
      GBCC_CUDA(ie);
      g.launches = ctx.launches - l0;
      g.flops = ctx.flops - f0;
      ctx.launches = l0;
      ctx.flops = f0;
    }
    GBCC_CUDA(cudaGraphLaunch(g.exec, ctx.stream));
    ctx.launches += g.launches;
    ctx.flops += g.flops;
  } else {
    iteration_body();
  }
  return finish_iteration();
}

// host state after the iteration's device work; waits for it and reads the
// sums back
IterInfo Ccsd::finish_iteration() {
  Context &ctx = ctx_;
  IterInfo info;
  if (o_.mixer == 1) {
    if (count_ < o_.max_residua) ++count_;                         // DiisMixer.cxx:141
    next_ = (next_ + 1) % o_.max_residua;                          // :179
  } else {
    have_last_ = true;
    std::swap(T_, E_);                                             // amplitudes = last
    std::swap(Lres_, D_);
    ++swaps_;
  }
  ctx.check_device_errors();  // the one host synchronisation per iteration
  const double *h = pinned_;
  energy_from_sums(h, info);
  info.dtdt = h[SC_UPD + 0];
  info.tt = (o_.mixer == 1) ? h[SC_TT] : h[SC_UPD + 1];
  info.lambda = h[SC_LAMBDA];
  int st = 0;
  std::memcpy(&st, h + SC_STATUS, sizeof(int));
  info.diis_status = (o_.mixer == 1) ? st : 0;
  return info;
}

void Ccsd::restart() {
  if (T0_.bytes()) copy(ctx_, T_.as<double>(), T0_.as<double>(), L_.ntot);
  else fill(ctx_, T_.as<double>(), L_.ntot, 0.0);
  it_ = 0;
  count_ = 0;
  next_ = 0;
  have_last_ = false;  // swaps_ keeps the linear mixer's buffer parity
  converged_ = false;
  e_ = prev_ = dir_ = exc_ = 0.0;
  hist_.clear();
  ctx_.check_device_errors();
}

gbcc_status Ccsd::run(int n, double *energy, int *converged) {
  gbcc_status st = GBCC_OK;
  for (int c = 0; c < n && !converged_; ++c) {
    if (it_ >= o_.max_iterations) break;
    if (absorb(iterate(), st)) break;
  }
  if (energy) *energy = e_;
  if (converged) *converged = converged_ ? 1 : 0;
  return st;
}

// takes in one iteration's results (ClusterSinglesDoublesAlgorithm.cxx:
// 98-112); true when the solve stops here: converged, or an error in st
bool Ccsd::absorb(IterInfo info, gbcc_status &st) {
  e_ = info.energy;
  dir_ = info.direct;
  exc_ = info.exchange;
  hist_.push_back(e_);
  ++it_;
  if (o_.mixer == 1 && ctx_.take_fault(GBCC_FAULT_DIIS_SINGULAR)) info.diis_status = 1;
  if (ctx_.take_fault(GBCC_FAULT_NAN)) info.dtdt = std::numeric_limits<double>::quiet_NaN();
  if (info.diis_status == 1) {
    // an exact zero pivot: dsysv's info != 0 (DiisMixer.cxx:37-41)
    ctx_.last_error = "DIIS subspace matrix singular at iteration " +
                      std::to_string(it_ - 1) + " (|dT|^2 = " +
                      std::to_string(info.dtdt) + ")";
    st = GBCC_DIIS_SINGULAR;
    return true;
  }
  if (info.diis_status == 2) {
    // overlaps or weights overflowed: the reference's dsysv returns
    // info == 0 there and its amplitudes become NaN
    ctx_.last_error = "DIIS subspace matrix or weights not finite at iteration " +
                      std::to_string(it_ - 1) + " (|dT|^2 = " +
                      std::to_string(info.dtdt) + ", E = " + std::to_string(e_) + ")";
    st = GBCC_DIVERGED;
    return true;
  }
  if (!std::isfinite(e_) || !std::isfinite(info.dtdt) || !std::isfinite(info.tt)) {
    ctx_.last_error = "energy or amplitude norms not finite at iteration " +
                      std::to_string(it_ - 1);
    st = GBCC_DIVERGED;
    return true;
  }
  // ClusterSinglesDoublesAlgorithm.cxx:103-106
  if (std::abs((e_ - prev_) / e_) < std::abs(o_.energy_convergence) &&
      std::abs(info.dtdt / info.tt) <
          std::abs(o_.amplitudes_convergence * o_.amplitudes_convergence)) {
    converged_ = true;
    return true;
  }
  prev_ = e_;
  return false;
}

}  // namespace gbcc
