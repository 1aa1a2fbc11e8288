// Serving layer: continuous admission of CCSD(T) solves of uneven size.
//
// A server owns `slots` workers, each with its own host thread and its own
// context (CUDA stream) on one device.  Requests are queued in arrival order
// and admitted (FIFO) as soon as a worker is free and the request's estimated
// device footprint fits in what is left of the HBM budget; requests that
// arrive while others run are admitted as slots and memory free up, and their
// kernels run concurrently with the others' on the device.  A solve keeps its
// integrals, amplitudes and DIIS history resident from admission to result.
// Every kernel is deterministic (fixed reduction orders, no floating-point
// atomics), so a request gives bit-identical energies alone and in a mix.
// A slot that admits a request of a small shape (lockstep_pays) also takes
// queued requests of the same shape, options and (T) flag (up to max_batch
// in all) and solves them in lockstep, one batched product per contraction
// for all of them; their energies then agree with the solve alone up to the
// rounding of the batched products.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "ccsd.hpp"

namespace gbcc {
double triples_energy(Context &ctx, const CcsdInputs &I, const double *T1,
                      const double *T2, int precision);
}

namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Request {
  int64_t id = 0;
  std::vector<double> eps_h, eps_p, gamma;
  gbcc_ccsd_in in{};
  gbcc_ccsd_opts opts{};
  int triples = 0;
  size_t bytes = 0;
  gbcc_result res{};
  bool done = false;
};

// Device footprint of one solve (bytes), from the tensors the solver keeps
// resident plus the peak of its temporaries, with a 1.5x margin.
// (T) of a served solve runs its hole triples in batches of at most this many
// W work arrays (Nv^3 doubles each, about 512 MiB in all), so that its memory
// is known at admission
int served_triples_images(int64_t Nv) {
  const double per = 8.0 * (double)Nv * (double)Nv * (double)Nv;
  return (int)std::max(6.0, std::min(192.0, std::floor(512.0 * (1 << 20) / per)));
}

size_t estimate_bytes(const gbcc_ccsd_in &in, const gbcc_ccsd_opts &o, int triples) {
  const double No = in.No, Nv = in.Nv, NG = in.NG;
  const double n2 = Nv * Nv * No * No, n1 = Nv * No;
  const double m = o.mixer == 1 ? o.max_residua : 1;
  double s = o.integrals_slice_size > 0 ? o.integrals_slice_size : Nv;
  s = std::min(s, Nv);
  double words = NG * (n1 + Nv * Nv + No * No) * 2.0   // vertex blocks + dressed copies
                 + 4.0 * n2 + 2.0 * No * No * No * Nv  // integrals
                 + 2.0 * (n1 + n2) * (2.0 + 2.0 * m)   // T, R, history / mixer
                 + 6.0 * n2                            // residual temporaries
                 + 2.0 * s * s * Nv * Nv;              // ladder block
  if (triples) words += Nv * Nv * Nv * No + served_triples_images(in.Nv) * Nv * Nv * Nv;
  // stored formulation: resident Vabcd / Vabci (the residual adds no other
  // Nv^4 tensor) and a permuted copy of Vabci
  if (o.formulation == 1) words += 1.0 * Nv * Nv * Nv * Nv + 2.0 * Nv * Nv * Nv * No;
  double bytes = 8.0 * words;
  // digit panels, including those kept for the constant integrals and
  // vertex blocks (one set per layout the contractions use)
  if (o.precision == GBCC_PREC_EMU) bytes *= 2.4;
  return (size_t)(1.5 * bytes) + (64u << 20);
}

// what a request adds in a lockstep batch: its copy in the stacked residual
// inputs (vertex blocks and integrals), with the same margins
size_t batch_extra_bytes(const gbcc_ccsd_in &in, const gbcc_ccsd_opts &o) {
  const double No = in.No, Nv = in.Nv, NG = in.NG;
  const double n2 = Nv * Nv * No * No;
  double bytes = 8.0 * (NG * (Nv * No + Nv * Nv + No * No) + 3.0 * n2 +
                        No * No * No * No + No * No * No * Nv);
  if (o.precision == GBCC_PREC_EMU) bytes *= 2.4;
  return (size_t)(1.5 * bytes);
}

bool same_opts(const gbcc_ccsd_opts &a, const gbcc_ccsd_opts &b) {
  return a.mixer == b.mixer && a.max_residua == b.max_residua &&
         a.mixing_ratio == b.mixing_ratio && a.max_iterations == b.max_iterations &&
         a.energy_convergence == b.energy_convergence &&
         a.amplitudes_convergence == b.amplitudes_convergence &&
         a.level_shift == b.level_shift && a.distinguishable == b.distinguishable &&
         a.ppl == b.ppl && a.integrals_slice_size == b.integrals_slice_size &&
         a.integrals_slice_factor == b.integrals_slice_factor && a.precision == b.precision &&
         a.emu_slices == b.emu_slices && a.formulation == b.formulation &&
         a.only_ppl == b.only_ppl && a.emu_min_flops == b.emu_min_flops &&
         a.f64_split_blocks == b.f64_split_blocks && a.emu_max_ksplit == b.emu_max_ksplit;
}

// Lockstep batches pay where one system's kernels leave most of the GPU
// idle.  The proxy is the particle ladder's V block, the largest product of
// an iteration: a batch is formed when one system's block (at the default
// integralsSliceSize of a batch) covers less than half the SMs with output
// tiles.  Above that, requests on their own streams run faster side by side
// (measured: No=8, Nv=64 and No=10, Nv=96 served faster unbatched, No=6,
// Nv=40 faster in lockstep).
bool lockstep_pays(const gbcc_ccsd_in &in, const gbcc_ccsd_opts &o, int sm_count) {
  const int64_t Nv = in.Nv;
  int64_t s = o.integrals_slice_size > 0 ? o.integrals_slice_size
                                         : std::max<int64_t>(16, Nv / 8);
  s = std::min<int64_t>(s, Nv);
  const int64_t vtiles = ((s * Nv + 127) / 128) * ((s * Nv + 63) / 64);
  return 2 * vtiles < sm_count;
}

// requests that can share a lockstep batch (DiisMixer, vertex formulation)
bool batchable(const Request &a, const Request &b) {
  return a.in.No == b.in.No && a.in.Nv == b.in.Nv && a.in.NG == b.in.NG &&
         a.triples == b.triples && same_opts(a.opts, b.opts) && a.opts.mixer == 1 &&
         a.opts.formulation == 0 && a.opts.max_iterations >= 1;
}

}  // namespace

struct gbcc_server {
  int device = 0;
  size_t budget = 0, in_use = 0;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::deque<Request *> pending;
  std::map<int64_t, std::unique_ptr<Request>> all;
  std::vector<std::thread> workers;
  bool stop = false;
  int64_t next_id = 1;
  int running = 0;
  int busy = 0;  // slots solving a request or a batch
  int max_batch = 8;
  int sm_count = 152;

  void worker_main(int w);
  void run_one(gbcc_ctx *ctx, Request &r);
  void run_batch(gbcc_ctx *ctx, const std::vector<Request *> &g);
};

// every request starts from the library's execution defaults; its own
// options (e.g. a tuned configuration of its shape) are applied at setup
static gbcc_status reset_ctx(gbcc_ctx *ctx, int64_t Nv) {
  gbcc_status st = gbcc_ctx_set_emulation(ctx, 6, 1e7);
  if (st == GBCC_OK) st = gbcc_ctx_set_splits(ctx, 3, 64);
  if (st == GBCC_OK) st = gbcc_ctx_set_triples_batch(ctx, served_triples_images(Nv));
  return st;
}

void gbcc_server::run_batch(gbcc_ctx *ctx, const std::vector<Request *> &g) {
  const int n = (int)g.size();
  const double t0 = now_s();
  for (Request *r : g) r->res.t_start = t0;
  const Request &r0 = *g[0];
  gbcc_status st = reset_ctx(ctx, r0.in.Nv);
  std::vector<gbcc_ccsd_in> ins;
  for (Request *r : g) ins.push_back(r->in);
  gbcc_batch *b = nullptr;
  if (st == GBCC_OK) st = gbcc_ccsd_batch_setup(ctx, n, ins.data(), &r0.opts, &b);
  std::vector<gbcc_status> sst((size_t)n, st);
  if (st == GBCC_OK) st = gbcc_ccsd_batch_step(b, r0.opts.max_iterations, sst.data());
  for (int z = 0; z < n; ++z) {
    Request &r = *g[z];
    gbcc_status s = st != GBCC_OK ? st : sst[z];
    if (st == GBCC_OK) {
      gbcc_ccsd_out out{};
      const gbcc_status s2 = gbcc_ccsd_batch_result(b, z, &out);
      r.res.e_ccsd = out.energy;
      r.res.iterations = out.iterations;
      r.res.converged = out.converged;
      r.res.e_total = out.energy;
      if (s2 != GBCC_OK) s = s2;
      // as for a request alone: (T) also on amplitudes that did not converge
      if ((s == GBCC_OK || s == GBCC_NOT_CONVERGED) && r.triples) {
        double et = 0, etot = 0;
        const gbcc_status s3 = gbcc_ccsd_batch_triples(b, z, r.opts.precision, &etot, &et);
        r.res.e_t = et;
        r.res.e_total = etot;
        if (s3 != GBCC_OK) s = s3;
      }
    }
    r.res.status = s;
    r.res.t_done = now_s();
  }
  if (b) gbcc_ccsd_batch_destroy(b);
}

void gbcc_server::run_one(gbcc_ctx *ctx, Request &r) {
  gbcc_solver *s = nullptr;
  r.res.t_start = now_s();
  gbcc_status st = reset_ctx(ctx, r.in.Nv);
  if (st == GBCC_OK) st = gbcc_ccsd_setup(ctx, &r.in, &r.opts, &s);
  if (st == GBCC_OK) {
    double e = 0;
    int conv = 0;
    st = gbcc_ccsd_step(s, r.opts.max_iterations, &e, &conv);
    gbcc_ccsd_out out{};
    if (st == GBCC_OK) st = gbcc_ccsd_result(s, &out);
    r.res.e_ccsd = out.energy;
    r.res.iterations = out.iterations;
    r.res.converged = out.converged;
    if (st == GBCC_OK && r.triples) {
      double et = 0, etot = 0;
      st = gbcc_triples_from_solver(s, r.opts.precision, &etot, &et);
      r.res.e_t = et;
      r.res.e_total = etot;
    } else {
      r.res.e_total = out.energy;
    }
    if (st == GBCC_OK && !out.converged) st = GBCC_NOT_CONVERGED;
  }
  if (s) gbcc_ccsd_destroy(s);
  r.res.status = st;
  r.res.t_done = now_s();
}

void gbcc_server::worker_main(int w) {
  (void)w;
  gbcc_ctx *ctx = nullptr;
  cudaSetDevice(device);
  const gbcc_status cst = gbcc_ctx_create(device, nullptr, &ctx);
  for (;;) {
    std::vector<Request *> g;
    size_t bytes = 0;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] {
        return stop || (!pending.empty() &&
                        (in_use + pending.front()->bytes <= budget || in_use == 0));
      });
      if (stop && pending.empty()) break;
      if (pending.empty()) continue;
      Request *r = pending.front();
      pending.pop_front();
      g.push_back(r);
      bytes = r->bytes;
      // queued requests of the same shape join it, while the budget allows;
      // the queued requests of the shape are shared out over the idle slots
      // (a batch of ceil(m / idle)), so that no slot is left without work
      if (max_batch > 1 && batchable(*r, *r) && lockstep_pays(r->in, r->opts, sm_count)) {
        int m = 1;
        for (Request *q : pending) m += batchable(*r, *q) ? 1 : 0;
        const int idle = std::max(1, (int)workers.size() - busy);
        const int take = std::min(max_batch, (m + idle - 1) / idle);
        const size_t first_extra = batch_extra_bytes(r->in, r->opts);
        for (auto it = pending.begin(); it != pending.end() && (int)g.size() < take;) {
          Request *q = *it;
          const size_t add = q->bytes + batch_extra_bytes(q->in, q->opts) +
                             (g.size() == 1 ? first_extra : 0);
          if (batchable(*r, *q) && in_use + bytes + add <= budget) {
            g.push_back(q);
            bytes += add;
            it = pending.erase(it);
          } else {
            ++it;
          }
        }
      }
      in_use += bytes;
      running += (int)g.size();
      ++busy;
      const double t = now_s();
      for (Request *q : g) q->res.t_admit = t;
    }
    if (cst != GBCC_OK) {
      for (Request *q : g) {
        q->res.status = cst;
        q->res.t_done = now_s();
      }
    } else if (g.size() == 1) {
      run_one(ctx, *g[0]);
    } else {
      run_batch(ctx, g);
    }
    {
      std::lock_guard<std::mutex> lk(mu);
      in_use -= bytes;
      running -= (int)g.size();
      --busy;
      for (Request *q : g) q->done = true;
    }
    cv_work.notify_all();
    cv_done.notify_all();
  }
  if (ctx) gbcc_ctx_destroy(ctx);
}

extern "C" {

void gbcc_server_opts_default(gbcc_server_opts *o) {
  if (!o) return;
  o->device = 0;
  o->slots = 8;
  o->hbm_budget_bytes = 0;  // 0: 80 % of the free device memory at creation
  o->max_batch = 8;
}

gbcc_status gbcc_server_create(const gbcc_server_opts *opts, gbcc_server **out) {
  if (!out) return GBCC_BAD_ARG;
  *out = nullptr;
  gbcc_server_opts o;
  if (opts) o = *opts; else gbcc_server_opts_default(&o);
  if (o.slots < 1 || o.slots > 64 || o.max_batch < 0 || o.max_batch > 64) return GBCC_BAD_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return GBCC_NO_DEVICE;
  }
  if (o.device < 0 || o.device >= n) return GBCC_BAD_ARG;
  auto *s = new gbcc_server();
  s->device = o.device;
  s->max_batch = std::max(1, o.max_batch);
  int sms = 0;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, o.device) == cudaSuccess &&
      sms > 0)
    s->sm_count = sms;
  else
    cudaGetLastError();
  if (o.hbm_budget_bytes > 0) {
    s->budget = (size_t)o.hbm_budget_bytes;
  } else {
    size_t fr = 0, tot = 0;
    cudaSetDevice(o.device);
    cudaMemGetInfo(&fr, &tot);
    s->budget = (size_t)(0.8 * (double)fr);
  }
  for (int w = 0; w < o.slots; ++w) s->workers.emplace_back([s, w] { s->worker_main(w); });
  *out = s;
  return GBCC_OK;
}

gbcc_status gbcc_server_submit(gbcc_server *s, const gbcc_ccsd_in *in,
                               const gbcc_ccsd_opts *opts, int triples,
                               int64_t *id) {
  if (!s || !in || !in->eps_h || !in->eps_p || !in->gamma) return GBCC_BAD_ARG;
  if (in->No <= 0 || in->Nv <= 0 || in->NG <= 0) return GBCC_BAD_ARG;
  if (in->Vabij || in->Vaibj || in->Vijkl || in->Vijka || in->init_T1 || in->init_T2 ||
      in->gamma_imag || in->fock_hp || in->Vabcd || in->Vabci)
    return GBCC_BAD_ARG;  // requests carry the vertex only; integrals are built on device
  auto r = std::make_unique<Request>();
  const size_t Np = (size_t)in->No + in->Nv;
  r->eps_h.assign(in->eps_h, in->eps_h + in->No);
  r->eps_p.assign(in->eps_p, in->eps_p + in->Nv);
  r->gamma.assign(in->gamma, in->gamma + (size_t)in->NG * Np * Np);
  r->in = *in;
  r->in.eps_h = r->eps_h.data();
  r->in.eps_p = r->eps_p.data();
  r->in.gamma = r->gamma.data();
  if (opts) r->opts = *opts; else gbcc_ccsd_opts_default(&r->opts);
  r->triples = triples;
  r->bytes = estimate_bytes(r->in, r->opts, triples);
  r->res.t_submit = now_s();
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return GBCC_BAD_ARG;
    r->id = s->next_id++;
    r->res.id = r->id;
    if (id) *id = r->id;
    s->pending.push_back(r.get());
    s->all[r->id] = std::move(r);
  }
  s->cv_work.notify_one();
  return GBCC_OK;
}

gbcc_status gbcc_server_poll(gbcc_server *s, int64_t id, gbcc_result *res, int *done) {
  if (!s) return GBCC_BAD_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return GBCC_BAD_ARG;
  if (done) *done = it->second->done ? 1 : 0;
  if (res && it->second->done) *res = it->second->res;
  return GBCC_OK;
}

gbcc_status gbcc_server_wait(gbcc_server *s, int64_t id, gbcc_result *res) {
  if (!s) return GBCC_BAD_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  auto it = s->all.find(id);
  if (it == s->all.end()) return GBCC_BAD_ARG;
  Request *r = it->second.get();
  s->cv_done.wait(lk, [&] { return r->done; });
  if (res) *res = r->res;
  return GBCC_OK;
}

gbcc_status gbcc_server_stats(gbcc_server *s, int *pending, int *running,
                              int64_t *bytes_in_use) {
  if (!s) return GBCC_BAD_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  if (pending) *pending = (int)s->pending.size();
  if (running) *running = s->running;
  if (bytes_in_use) *bytes_in_use = (int64_t)s->in_use;
  return GBCC_OK;
}

void gbcc_server_destroy(gbcc_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  for (auto &t : s->workers) t.join();
  delete s;
}

}  // extern "C"
