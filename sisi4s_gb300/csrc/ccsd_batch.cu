// Lockstep CCSD over several closed-shell systems of one shape: one residual
// program over all of them (each contraction one batched product), the
// update, mixer and energy per system.
#include <algorithm>
#include <cmath>
#include <string>

#include "ccsd_batch.hpp"

namespace gbcc {

BatchCcsd::BatchCcsd(Context &ctx, std::vector<std::unique_ptr<Ccsd>> systems)
    : ctx_(ctx), sys_(std::move(systems)) {
  nz_ = (int64_t)sys_.size();
  require(nz_ >= 2 && nz_ <= 64, "a batch holds 2 to 64 systems");
  Ccsd &s0 = *sys_[0];
  o_ = s0.options();
  L_ = s0.layout();
  const CcsdInputs &I0 = s0.inputs();
  require(o_.mixer == 1, "a batch of systems runs the DiisMixer");
  require(o_.formulation == 0, "a batch of systems runs CcsdEnergyFromCoulombIntegrals");
  require(I0.Gab.p() && I0.Vaibj.p(), "a batch of systems needs the CoulombVertex");
  for (auto &s : sys_) {
    const CcsdInputs &I = s->inputs();
    const gbcc_ccsd_opts &o = s->options();
    require(I.No == I0.No && I.Nv == I0.Nv && I.NG == I0.NG,
            "the systems of a batch must have the same No, Nv and NG");
    require(o.mixer == o_.mixer && o.formulation == o_.formulation &&
                o.precision == o_.precision && o.ppl == o_.ppl &&
                o.distinguishable == o_.distinguishable && o.max_residua == o_.max_residua,
            "the systems of a batch must share mixer, formulation, precision, ppl, "
            "distinguishable and maxResidua");
    require(s->has_initial_doubles() == s0.has_initial_doubles(),
            "either every system of a batch starts from given doubles or none does");
    require(s->iterations_done() == s0.iterations_done(),
            "the systems of a batch must start at the same iteration");
  }
  it_ = s0.iterations_done();
  st_.assign(sys_.size(), GBCC_OK);
  active_.assign(sys_.size(), 1);
  const int64_t No = L_.No, Nv = L_.Nv;
  // integralsSliceSize (CcsdEnergyFromCoulombIntegrals.cxx:375-385); the
  // device default of one system with its V_xycd budget shared by the batch
  if (o_.integrals_slice_size > 0) slice_ = o_.integrals_slice_size;
  else if (o_.integrals_slice_factor >= 0) slice_ = (int64_t)(Nv * o_.integrals_slice_factor);
  else {
    const double budget = 4.0 * 1024 * 1024 * 1024 / 16.0 / (double)nz_;
    const int64_t cap = (int64_t)std::floor(std::sqrt(budget / (double)(Nv * Nv)));
    slice_ = std::min<int64_t>(cap, std::max<int64_t>(16, Nv / 8));
  }
  slice_ = std::max<int64_t>(1, std::min<int64_t>(slice_, Nv));
  // the residual inputs, system after system
  in_.No = No;
  in_.Nv = Nv;
  in_.NG = I0.NG;
  auto stack = [&](OTen &dst, OTen CcsdInputs::*field) {
    const Ten &t0 = sys_[0]->inputs().*field;
    std::vector<int64_t> l(t0.lens.begin(), t0.lens.begin() + t0.order);
    l.push_back(nz_);
    dst = OTen(ctx_, l);
    const int64_t n = t0.size();
    for (int64_t z = 0; z < nz_; ++z) {
      const Ten &t = sys_[z]->inputs().*field;
      require(t.p != nullptr && t.size() == n, "batch: missing input block");
      GBCC_CUDA(cudaMemcpyAsync(dst.p() + z * n, t.p, sizeof(double) * n,
                                cudaMemcpyDeviceToDevice, ctx_.stream));
    }
  };
  stack(in_.Vabij, &CcsdInputs::Vabij);
  stack(in_.Vx, &CcsdInputs::Vx);
  stack(in_.Vaibj, &CcsdInputs::Vaibj);
  stack(in_.Vijkl, &CcsdInputs::Vijkl);
  stack(in_.Vijka, &CcsdInputs::Vijka);
  stack(in_.Gai, &CcsdInputs::Gai);
  stack(in_.Gab, &CcsdInputs::Gab);
  stack(in_.Gij, &CcsdInputs::Gij);
  T1b_.alloc(ctx_, sizeof(double) * L_.n1 * nz_);
  T2b_.alloc(ctx_, sizeof(double) * L_.n2 * nz_);
  R1b_.alloc(ctx_, sizeof(double) * L_.n1 * nz_);
  R2b_.alloc(ctx_, sizeof(double) * L_.n2 * nz_);
  // the residual is scattered into each system's T1 and T2 blocks only: the
  // padding between them stays zero, as the update's reductions expect
  for (auto &s : sys_) fill(ctx_, s->residual_buffer(), L_.ntot, 0.0);
  zeros_.alloc(ctx_, sizeof(double) * std::max(L_.n1, L_.n2));
  fill(ctx_, zeros_.as<double>(), std::max(L_.n1, L_.n2), 0.0);
  ptrs_.alloc(ctx_, sizeof(double *) * 4 * nz_);
  upload_pointers(~0ull);
  ctx_.check_device_errors();
}

BatchCcsd::~BatchCcsd() {
  cudaStreamSynchronize(ctx_.stream);
  for (auto &g : graphs_)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
}

// the gather and scatter pointers: a system that no longer runs gives zero
// amplitudes to the residual program, so that its own amplitudes (not finite
// after a failure) never reach a product; its residual buffer takes a
// residual that nothing reads
void BatchCcsd::upload_pointers(uint64_t mask) {
  std::vector<double *> p((size_t)(4 * nz_));
  for (int64_t z = 0; z < nz_; ++z) {
    const bool on = (mask >> z) & 1;
    double *T = sys_[z]->amplitude_buffer(), *R = sys_[z]->residual_buffer();
    p[0 * nz_ + z] = on ? T : zeros_.as<double>();
    p[1 * nz_ + z] = on ? T + L_.off2 : zeros_.as<double>();
    p[2 * nz_ + z] = R;
    p[3 * nz_ + z] = R + L_.off2;
  }
  GBCC_CUDA(cudaMemcpyAsync(ptrs_.as<double *>(), p.data(), sizeof(double *) * p.size(),
                            cudaMemcpyHostToDevice, ctx_.stream));
  ptr_mask_ = mask;
}

// device work of one lockstep iteration for the running systems in mask
void BatchCcsd::body(uint64_t mask) {
  Context &ctx = ctx_;
  const int64_t No = L_.No, Nv = L_.Nv;
  double *const *p = ptrs_.as<double *>();
  batch_gather(ctx, p + 0 * nz_, L_.n1, nz_, T1b_.as<double>());
  batch_gather(ctx, p + 1 * nz_, L_.n2, nz_, T2b_.as<double>());
  fill(ctx, R1b_.as<double>(), L_.n1 * nz_, 0.0);                 // :37-38
  fill(ctx, R2b_.as<double>(), L_.n2 * nz_, 0.0);
  ResidualArgs a;
  a.I = &in_;
  a.o = &o_;
  a.nz = nz_;
  a.slice = slice_;
  a.init_doubles = sys_[0]->has_initial_doubles();
  a.T1 = ten(T1b_.as<double>(), {Nv, No, nz_});
  a.T2 = ten(T2b_.as<double>(), {Nv, Nv, No, No, nz_});
  a.R1 = ten(R1b_.as<double>(), {Nv, No, nz_});
  a.R2 = ten(R2b_.as<double>(), {Nv, Nv, No, No, nz_});
  residual_program(ctx, a, it_);
  batch_scatter(ctx, R1b_.as<double>(), L_.n1, nz_, p + 2 * nz_);
  batch_scatter(ctx, R2b_.as<double>(), L_.n2, nz_, p + 3 * nz_);
  for (int64_t z = 0; z < nz_; ++z)
    if ((mask >> z) & 1) sys_[z]->mix_body();
}

void BatchCcsd::run(int n) {
  Context &ctx = ctx_;
  for (int c = 0; c < n; ++c) {
    uint64_t mask = 0;
    for (int64_t z = 0; z < nz_; ++z) {
      Ccsd &s = *sys_[z];
      if (active_[z] && s.iterations_done() >= s.options().max_iterations) active_[z] = 0;
      if (active_[z]) mask |= 1ull << z;
    }
    if (!mask) break;
    if (mask != ptr_mask_) upload_pointers(mask);
    // the running systems have iterated together, so their DIIS rings are
    // in the same state and their graph keys agree
    int key = -2;
    for (int64_t z = 0; z < nz_; ++z) {
      if (!((mask >> z) & 1)) continue;
      const int k = sys_[z]->graph_key();
      require(key == -2 || key == k, "batch: systems out of step");
      key = k;
    }
    if (key >= 0 && ctx.use_graphs && !ctx.prof) {
      Graph &g = graphs_[{key, mask}];
      if (!g.exec) {
        const uint64_t l0 = ctx.launches;
        const double f0 = ctx.flops;
        GBCC_CUDA(cudaStreamBeginCapture(ctx.stream, cudaStreamCaptureModeThreadLocal));
        try {
          body(mask);
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
      body(mask);
    }
    ++it_;
    for (int64_t z = 0; z < nz_; ++z) {
      if (!((mask >> z) & 1)) continue;
      const IterInfo info = sys_[z]->finish_iteration();
      if (sys_[z]->absorb(info, st_[z])) active_[z] = 0;
    }
  }
}

}  // namespace gbcc
