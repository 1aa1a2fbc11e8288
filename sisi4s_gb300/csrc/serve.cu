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

  void worker_main(int w);
  void run_one(gbcc_ctx *ctx, Request &r);
};

void gbcc_server::run_one(gbcc_ctx *ctx, Request &r) {
  gbcc_solver *s = nullptr;
  r.res.t_start = now_s();
  // every request starts from the library's execution defaults; its own
  // options (e.g. a tuned configuration of its shape) are applied at setup
  gbcc_status st = gbcc_ctx_set_emulation(ctx, 6, 1e7);
  if (st == GBCC_OK) st = gbcc_ctx_set_splits(ctx, 3, 64);
  if (st == GBCC_OK) st = gbcc_ctx_set_triples_batch(ctx, served_triples_images(r.in.Nv));
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
    Request *r = nullptr;
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_work.wait(lk, [&] {
        return stop || (!pending.empty() &&
                        (in_use + pending.front()->bytes <= budget || in_use == 0));
      });
      if (stop && pending.empty()) break;
      if (pending.empty()) continue;
      r = pending.front();
      pending.pop_front();
      in_use += r->bytes;
      ++running;
      r->res.t_admit = now_s();
    }
    if (cst == GBCC_OK) {
      run_one(ctx, *r);
    } else {
      r->res.status = cst;
      r->res.t_done = now_s();
    }
    {
      std::lock_guard<std::mutex> lk(mu);
      in_use -= r->bytes;
      --running;
      r->done = true;
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
}

gbcc_status gbcc_server_create(const gbcc_server_opts *opts, gbcc_server **out) {
  if (!out) return GBCC_BAD_ARG;
  *out = nullptr;
  gbcc_server_opts o;
  if (opts) o = *opts; else gbcc_server_opts_default(&o);
  if (o.slots < 1 || o.slots > 64) return GBCC_BAD_ARG;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    return GBCC_NO_DEVICE;
  }
  if (o.device < 0 || o.device >= n) return GBCC_BAD_ARG;
  auto *s = new gbcc_server();
  s->device = o.device;
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
