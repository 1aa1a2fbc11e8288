// Lockstep CCSD over several closed-shell systems of one shape: one residual
// program over all of them (each contraction one batched product), the
// update, mixer and energy per system.
#include <algorithm>
#include <cmath>
#include <string>

#include "ccsd_batch.hpp"

namespace gbcc {

namespace {
// the residual's inputs, stacked over the running systems
constexpr OTen CcsdInputs::*kStacked[] = {
    &CcsdInputs::Vabij, &CcsdInputs::Vx,  &CcsdInputs::Vaibj, &CcsdInputs::Vijkl,
    &CcsdInputs::Vijka, &CcsdInputs::Gai, &CcsdInputs::Gab,   &CcsdInputs::Gij};
}  // namespace

BatchCcsd::BatchCcsd(Context &ctx, std::vector<std::unique_ptr<Ccsd>> systems)
    : ctx_(ctx), sys_(std::move(systems)) {
  nz_ = (int64_t)sys_.size();
  require(nz_ >= 1 && nz_ <= 64, "a batch holds 1 to 64 systems");
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
  for (auto f : kStacked) {
    OTen &dst = in_.*f;
    const Ten &t0 = sys_[0]->inputs().*f;
    if (nz_ == 1) {  // a batch of one: the system's own inputs, viewed
      dst.t = t0;
      continue;
    }
    std::vector<int64_t> l(t0.lens.begin(), t0.lens.begin() + t0.order);
    l.push_back(nz_);
    dst = OTen(ctx_, l);
    const int64_t n = t0.size();
    for (int64_t z = 0; z < nz_; ++z) {
      const Ten &t = sys_[z]->inputs().*f;
      require(t.p != nullptr && t.size() == n, "batch: missing input block");
      GBCC_CUDA(cudaMemcpyAsync(dst.p() + z * n, t.p, sizeof(double) * n,
                                cudaMemcpyDeviceToDevice, ctx_.stream));
    }
    // unchanged while the set of running systems is: their digit panels are
    // split once (and dropped when the batch shrinks)
    ctx_.register_constant(dst.p(), sizeof(double) * (size_t)dst.t.size());
  }
  if (nz_ > 1) in_.ctx = &ctx_;  // forgets the stacked inputs on destruction
  T1b_.alloc(ctx_, sizeof(double) * L_.n1 * nz_);
  T2b_.alloc(ctx_, sizeof(double) * L_.n2 * nz_);
  R1b_.alloc(ctx_, sizeof(double) * L_.n1 * nz_);
  R2b_.alloc(ctx_, sizeof(double) * L_.n2 * nz_);
  // the residual is scattered into each system's T1 and T2 blocks only: the
  // padding between them stays zero, as the update's reductions expect
  for (auto &s : sys_) fill(ctx_, s->residual_buffer(), L_.ntot, 0.0);
  ptrs_.alloc(ctx_, sizeof(double *) * 4 * nz_);
  run_.resize(nz_);
  for (int64_t z = 0; z < nz_; ++z) run_[z] = (int)z;
  upload_pointers();
  ctx_.check_device_errors();
}

BatchCcsd::~BatchCcsd() {
  cudaStreamSynchronize(ctx_.stream);
  for (auto &g : graphs_)
    if (g.second.exec) cudaGraphExecDestroy(g.second.exec);
}

// the gather and scatter pointers of the running systems, in stacked order
void BatchCcsd::upload_pointers() {
  const int64_t n = (int64_t)run_.size();
  std::vector<double *> p((size_t)(4 * n));
  for (int64_t j = 0; j < n; ++j) {
    double *T = sys_[run_[j]]->amplitude_buffer(), *R = sys_[run_[j]]->residual_buffer();
    p[0 * n + j] = T;
    p[1 * n + j] = T + L_.off2;
    p[2 * n + j] = R;
    p[3 * n + j] = R + L_.off2;
  }
  GBCC_CUDA(cudaMemcpyAsync(ptrs_.as<double *>(), p.data(), sizeof(double *) * p.size(),
                            cudaMemcpyHostToDevice, ctx_.stream));
}

// Drops the systems that stopped from the stacked inputs: the blocks of the
// running ones move down in place (in order, so no block overwrites one
// still to be moved), and the residual program then works on them alone.
void BatchCcsd::compact(uint64_t mask) {
  std::vector<int> keep;
  for (int z : run_)
    if ((mask >> z) & 1) keep.push_back(z);
  for (auto f : kStacked) {
    OTen &t = in_.*f;
    ctx_.forget_constant(t.p());
    const int64_t n = t.t.size() / t.t.lens[t.t.order - 1];
    for (size_t j = 0, p = 0; j < keep.size(); ++j) {
      while (run_[p] != keep[j]) ++p;
      if (p != j)
        GBCC_CUDA(cudaMemcpyAsync(t.p() + j * n, t.p() + p * n, sizeof(double) * n,
                                  cudaMemcpyDeviceToDevice, ctx_.stream));
    }
    // one system left: its inputs lose the system index (the plain program)
    if (keep.size() == 1) t.t.order -= 1;
    else t.t.lens[t.t.order - 1] = (int64_t)keep.size();
    ctx_.register_constant(t.p(), sizeof(double) * (size_t)t.t.size());
  }
  run_ = keep;
  upload_pointers();
}

// device work of one lockstep iteration of the running systems
void BatchCcsd::body() {
  Context &ctx = ctx_;
  const int64_t No = L_.No, Nv = L_.Nv, nz = (int64_t)run_.size();
  double *const *p = ptrs_.as<double *>();
  batch_gather(ctx, p + 0 * nz, L_.n1, nz, T1b_.as<double>());
  batch_gather(ctx, p + 1 * nz, L_.n2, nz, T2b_.as<double>());
  fill(ctx, R1b_.as<double>(), L_.n1 * nz, 0.0);                  // :37-38
  fill(ctx, R2b_.as<double>(), L_.n2 * nz, 0.0);
  ResidualArgs a;
  a.I = &in_;
  a.o = &o_;
  a.nz = nz;
  a.slice = slice_;
  a.init_doubles = sys_[0]->has_initial_doubles();
  if (nz > 1) {
    a.T1 = ten(T1b_.as<double>(), {Nv, No, nz});
    a.T2 = ten(T2b_.as<double>(), {Nv, Nv, No, No, nz});
    a.R1 = ten(R1b_.as<double>(), {Nv, No, nz});
    a.R2 = ten(R2b_.as<double>(), {Nv, Nv, No, No, nz});
  } else {
    // one system left: the plain program, on the stacked inputs without
    // their system index
    a.T1 = ten(T1b_.as<double>(), {Nv, No});
    a.T2 = ten(T2b_.as<double>(), {Nv, Nv, No, No});
    a.R1 = ten(R1b_.as<double>(), {Nv, No});
    a.R2 = ten(R2b_.as<double>(), {Nv, Nv, No, No});
  }
  residual_program(ctx, a, it_);
  batch_scatter(ctx, R1b_.as<double>(), L_.n1, nz, p + 2 * nz);
  batch_scatter(ctx, R2b_.as<double>(), L_.n2, nz, p + 3 * nz);
  for (int z : run_) sys_[z]->mix_body();
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
    uint64_t cur = 0;
    for (int z : run_) cur |= 1ull << z;
    if (mask != cur) compact(mask);
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
          body();
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
      body();
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
