// C ABI of libgbcc (include/gbcc.h).  Every entry point catches all
// exceptions and returns a gbcc_status; messages go to gbcc_last_error().
#include <cstring>
#include <memory>
#include <string>

#include "ccsd.hpp"
#include "ccsd_batch.hpp"

namespace gbcc {
double triples_energy(Context &ctx, const CcsdInputs &I, const double *T1,
                      const double *T2, int precision);
gbcc_status complex_solve(Context &ctx, const gbcc_ccsd_complex_in &in,
                          const gbcc_ccsd_opts &o, gbcc_ccsd_complex_out *out);
void complex_residual(Context &ctx, const gbcc_ccsd_complex_in &in, const gbcc_ccsd_opts &o,
                      int it, const double *T1, const double *T2, double *R1, double *R2);
void complex_triples(Context &ctx, const gbcc_triples_complex_in &in, int precision,
                     double *e_total, double *e_t);
void complex_integrals(Context &ctx, int No, int Nv, int NG, const double *gamma,
                       double *const out[7]);
}

struct gbcc_ctx {
  gbcc::Context c;
};

struct gbcc_solver {
  gbcc_ctx *ctx;
  std::unique_ptr<gbcc::Ccsd> s;
  gbcc_ccsd_opts opts;
};

struct gbcc_batch {
  gbcc_ctx *ctx;
  std::unique_ptr<gbcc::BatchCcsd> b;
  gbcc_ccsd_opts opts;
};

namespace {

thread_local std::string g_err;

template <class F>
gbcc_status guard(gbcc_ctx *ctx, F &&f) {
  try {
    if (ctx) {
      int cur = -1;
      cudaGetDevice(&cur);
      if (cur != ctx->c.device) {
        cudaError_t e = cudaSetDevice(ctx->c.device);
        if (e != cudaSuccess)
          throw gbcc::Error(GBCC_CUDA_ERROR, cudaGetErrorString(e));
      }
    }
    return f();
  } catch (const gbcc::Error &e) {
    if (ctx) ctx->c.last_error = e.what();
    g_err = e.what();
    return e.status;
  } catch (const std::bad_alloc &) {
    if (ctx) ctx->c.last_error = "host allocation failed";
    g_err = "host allocation failed";
    return GBCC_OOM;
  } catch (const std::exception &e) {
    if (ctx) ctx->c.last_error = e.what();
    g_err = e.what();
    return GBCC_CUDA_ERROR;
  }
}

void check_opts(const gbcc_ccsd_opts &o) {
  gbcc::require(o.max_iterations >= 0, "maxIterations must be >= 0");
  gbcc::require(o.mixer == 0 || o.mixer == 1, "unknown mixer");
  gbcc::require(o.precision == GBCC_PREC_FP64 || o.precision == GBCC_PREC_EMU,
                "unknown precision");
  gbcc::require(o.formulation == 0 || o.formulation == 1, "unknown formulation");
  gbcc::require(o.only_ppl == 0 || o.formulation == 1,
                "onlyPPL belongs to CcsdEnergyFromCoulombIntegralsReference");
}

void apply_precision_opts(gbcc::Context &c, const gbcc_ccsd_opts &o) {
  if (o.emu_slices > 0) c.emu_slices = o.emu_slices;
  if (o.emu_min_flops > 0) c.emu_min_flops = o.emu_min_flops;
  if (o.f64_split_blocks >= 0) c.f64_split_blocks = o.f64_split_blocks;
  if (o.emu_max_ksplit >= 1) c.emu_max_ksplit = std::min(o.emu_max_ksplit, 64);
}

}  // namespace

extern "C" {

int gbcc_abi_version(void) { return GBCC_ABI_VERSION; }

gbcc_status gbcc_device_pool_high_water(int device, int reset, int64_t *bytes) {
  if (!bytes) return GBCC_BAD_ARG;
  *bytes = 0;
  return guard(nullptr, [&]() {
    cudaMemPool_t pool = nullptr;
    GBCC_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    unsigned long long v = 0;  // the attribute is a 64-bit unsigned value
    GBCC_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &v));
    *bytes = (int64_t)v;
    if (reset) {
      unsigned long long z = 0;
      GBCC_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &z));
    }
    return GBCC_OK;
  });
}

const char *gbcc_status_string(int s) {
  switch (s) {
    case GBCC_OK: return "OK";
    case GBCC_NOT_CONVERGED: return "NOT_CONVERGED";
    case GBCC_DIIS_SINGULAR: return "DIIS_SINGULAR";
    case GBCC_DIVERGED: return "DIVERGED";
    case GBCC_OOM: return "OOM";
    case GBCC_BAD_ARG: return "BAD_ARG";
    case GBCC_CUDA_ERROR: return "CUDA_ERROR";
    case GBCC_TIMEOUT: return "TIMEOUT";
    case GBCC_COMPLEX_UNSUPPORTED: return "COMPLEX_UNSUPPORTED";
    case GBCC_NO_DEVICE: return "NO_DEVICE";
    default: return "UNKNOWN";
  }
}

gbcc_status gbcc_ctx_create(int device, void *stream, gbcc_ctx **out) {
  if (!out) return GBCC_BAD_ARG;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    g_err = "no CUDA device";
    return GBCC_NO_DEVICE;
  }
  if (device < 0 || device >= n) {
    g_err = "device index out of range";
    return GBCC_BAD_ARG;
  }
  auto *ctx = new gbcc_ctx();
  gbcc_status st = guard(nullptr, [&]() {
    ctx->c.device = device;
    GBCC_CUDA(cudaSetDevice(device));
    GBCC_CUDA(cudaDeviceGetAttribute(&ctx->c.sm_count,
                                     cudaDevAttrMultiProcessorCount, device));
    // Temporaries are stream-ordered allocations from the device's default
    // pool.  By default the pool hands freed memory back to the driver at
    // every synchronisation, so each CCSD iteration would re-map its
    // multi-GB working set; keep it in the pool instead.
    cudaMemPool_t pool;
    GBCC_CUDA(cudaDeviceGetDefaultMemPool(&pool, device));
    uint64_t keep = UINT64_MAX;
    GBCC_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    if (stream) {
      ctx->c.stream = static_cast<cudaStream_t>(stream);
    } else {
      GBCC_CUDA(cudaStreamCreateWithFlags(&ctx->c.stream, cudaStreamNonBlocking));
      ctx->c.own_stream = true;
    }
    return GBCC_OK;
  });
  if (st != GBCC_OK) {
    delete ctx;
    return st;
  }
  *out = ctx;
  return GBCC_OK;
}

void gbcc_ctx_destroy(gbcc_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->c.device);
  cudaStreamSynchronize(ctx->c.stream);
  if (ctx->c.dev_err) cudaFree(ctx->c.dev_err);
  ctx->c.prof_harvest();
  for (auto e : ctx->c.prof_pool) cudaEventDestroy(e);
  if (ctx->c.own_stream) cudaStreamDestroy(ctx->c.stream);
  delete ctx;
}

const char *gbcc_last_error(const gbcc_ctx *ctx) {
  return ctx ? ctx->c.last_error.c_str() : g_err.c_str();
}

uint64_t gbcc_ctx_kernel_launches(const gbcc_ctx *ctx) {
  return ctx ? ctx->c.launches : 0;
}

double gbcc_ctx_flops(const gbcc_ctx *ctx) { return ctx ? ctx->c.flops : 0.0; }

void *gbcc_ctx_stream(const gbcc_ctx *ctx) {
  return ctx ? static_cast<void *>(ctx->c.stream) : nullptr;
}

gbcc_status gbcc_ctx_set_operand_cache(gbcc_ctx *ctx, int enable) {
  if (!ctx) return GBCC_BAD_ARG;
  ctx->c.use_panel_cache = enable != 0;
  return GBCC_OK;
}

gbcc_status gbcc_ctx_set_splits(gbcc_ctx *ctx, int f64_blocks_per_sm, int emu_max_ksplit) {
  if (!ctx || f64_blocks_per_sm < 0 || emu_max_ksplit < 1 || emu_max_ksplit > 64)
    return GBCC_BAD_ARG;
  ctx->c.f64_split_blocks = f64_blocks_per_sm;
  ctx->c.emu_max_ksplit = emu_max_ksplit;
  return GBCC_OK;
}

gbcc_status gbcc_ctx_set_triples_batch(gbcc_ctx *ctx, int max_images) {
  if (!ctx || max_images < 0 || (max_images > 0 && max_images < 6)) return GBCC_BAD_ARG;
  ctx->c.triples_batch_images = max_images;
  return GBCC_OK;
}

gbcc_status gbcc_ctx_set_emulation(gbcc_ctx *ctx, int emu_slices,
                                   double emu_min_flops) {
  if (!ctx || emu_slices < 4 || emu_slices > 8 || emu_min_flops < 0)
    return GBCC_BAD_ARG;
  ctx->c.emu_slices = emu_slices;
  ctx->c.emu_min_flops = emu_min_flops;
  return GBCC_OK;
}

gbcc_status gbcc_ctx_set_graphs(gbcc_ctx *ctx, int enable) {
  if (!ctx) return GBCC_BAD_ARG;
  ctx->c.use_graphs = enable != 0;
  return GBCC_OK;
}

gbcc_status gbcc_ctx_profile(gbcc_ctx *ctx, int enable) {
  if (!ctx) return GBCC_BAD_ARG;
  ctx->c.prof = enable != 0;
  return GBCC_OK;
}

gbcc_status gbcc_ctx_gemm_stats(gbcc_ctx *ctx, double *ms, int64_t *launches,
                                double *tc_flops, double *fp64_flops) {
  if (!ctx) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    ctx->c.prof_harvest();
    if (ms) *ms = ctx->c.prof_ms;
    if (launches) *launches = ctx->c.prof_launches;
    if (tc_flops) *tc_flops = ctx->c.prof_tc_flops;
    if (fp64_flops) *fp64_flops = ctx->c.prof_fp64_flops;
    ctx->c.prof_ms = ctx->c.prof_tc_flops = ctx->c.prof_fp64_flops = 0;
    ctx->c.prof_launches = 0;
    return GBCC_OK;
  });
}

gbcc_status gbcc_ctx_inject_fault(gbcc_ctx *ctx, int kind) {
  if (!ctx || kind < GBCC_FAULT_NONE || kind > GBCC_FAULT_DEVICE_WAIT) return GBCC_BAD_ARG;
  ctx->c.fault = kind;
  return GBCC_OK;
}

gbcc_status gbcc_ctx_gemm_records(gbcc_ctx *ctx, int64_t *mnk, double *ms, int64_t cap,
                                  int64_t *count) {
  if (!ctx || cap < 0 || (cap > 0 && (!mnk || !ms))) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    ctx->c.prof_harvest();
    auto &log = ctx->c.prof_log;
    const int64_t n = std::min<int64_t>(cap, (int64_t)log.size());
    for (int64_t i = 0; i < n; ++i) {
      mnk[3 * i] = log[i].M;
      mnk[3 * i + 1] = log[i].N;
      mnk[3 * i + 2] = log[i].K;
      ms[i] = log[i].ms;
    }
    if (count) *count = n;
    log.clear();
    return GBCC_OK;
  });
}

void gbcc_ccsd_opts_default(gbcc_ccsd_opts *o) {
  if (!o) return;
  o->mixer = 0;
  o->max_residua = 4;
  o->mixing_ratio = 1.0;
  o->max_iterations = 16;
  o->energy_convergence = 1e-6;
  o->amplitudes_convergence = 1e-5;
  o->level_shift = 0.0;
  o->distinguishable = 0;
  o->ppl = 1;
  o->integrals_slice_size = -1;
  o->integrals_slice_factor = -1.0;
  o->precision = GBCC_PREC_FP64;
  o->emu_slices = 0;
  o->formulation = 0;
  o->only_ppl = 0;
  o->emu_min_flops = -1.0;
  o->f64_split_blocks = -1;
  o->emu_max_ksplit = -1;
}

gbcc_status gbcc_ccsd_setup(gbcc_ctx *ctx, const gbcc_ccsd_in *in,
                            const gbcc_ccsd_opts *opts, gbcc_solver **out) {
  if (!ctx || !in || !out) return GBCC_BAD_ARG;
  *out = nullptr;
  return guard(ctx, [&]() {
    gbcc_ccsd_opts o;
    if (opts) o = *opts; else gbcc_ccsd_opts_default(&o);
    check_opts(o);
    apply_precision_opts(ctx->c, o);
    auto inputs = gbcc::upload_inputs(ctx->c, *in, o.precision, true, o.formulation == 1);
    auto s = std::make_unique<gbcc_solver>();
    s->ctx = ctx;
    s->opts = o;
    s->s = std::make_unique<gbcc::Ccsd>(ctx->c, std::move(inputs), o,
                                        in->init_T1, in->init_T2);
    ctx->c.check_device_errors();
    *out = s.release();
    return GBCC_OK;
  });
}

gbcc_status gbcc_ccsd_step(gbcc_solver *s, int n, double *energy,
                           int *converged) {
  if (!s) return GBCC_BAD_ARG;
  return guard(s->ctx, [&]() { return s->s->run(n, energy, converged); });
}

namespace {
// gbcc_ccsd_out of one solver (the caller synchronises the stream)
void fill_result(gbcc::Ccsd &c, gbcc::Context &ctx, gbcc_ccsd_out *out) {
  const auto &L = c.layout();
  out->energy = c.energy();
  out->direct = c.direct();
  out->exchange = c.exchange();
  out->iterations = c.iterations_done();
  out->converged = c.converged() ? 1 : 0;
  if (out->T1)
    GBCC_CUDA(cudaMemcpyAsync(out->T1, c.amplitudes(), 8 * L.n1,
                              cudaMemcpyDeviceToHost, ctx.stream));
  if (out->T2)
    GBCC_CUDA(cudaMemcpyAsync(out->T2, c.amplitudes() + L.off2, 8 * L.n2,
                              cudaMemcpyDeviceToHost, ctx.stream));
  if (out->pair_energy) {
    gbcc::DBuf pe(ctx, 8 * L.No * L.No);
    c.pair_energies(pe.as<double>());
    GBCC_CUDA(cudaMemcpyAsync(out->pair_energy, pe.as<double>(), 8 * L.No * L.No,
                              cudaMemcpyDeviceToHost, ctx.stream));
    GBCC_CUDA(cudaStreamSynchronize(ctx.stream));
  }
  if (out->energy_history) {
    const auto &h = c.history();
    if (!h.empty())
      std::memcpy(out->energy_history, h.data(), sizeof(double) * h.size());
  }
}
}  // namespace

gbcc_status gbcc_ccsd_batch_setup(gbcc_ctx *ctx, int nsys, const gbcc_ccsd_in *ins,
                                  const gbcc_ccsd_opts *opts, gbcc_batch **out) {
  if (!ctx || !ins || nsys < 1 || nsys > 64 || !out) return GBCC_BAD_ARG;
  *out = nullptr;
  return guard(ctx, [&]() {
    gbcc_ccsd_opts o;
    if (opts) o = *opts; else gbcc_ccsd_opts_default(&o);
    check_opts(o);
    apply_precision_opts(ctx->c, o);
    std::vector<std::unique_ptr<gbcc::Ccsd>> sys;
    for (int z = 0; z < nsys; ++z) {
      auto inputs = gbcc::upload_inputs(ctx->c, ins[z], o.precision, true, false);
      sys.push_back(std::make_unique<gbcc::Ccsd>(ctx->c, std::move(inputs), o, ins[z].init_T1,
                                                 ins[z].init_T2));
    }
    auto b = std::make_unique<gbcc_batch>();
    b->ctx = ctx;
    b->opts = o;
    b->b = std::make_unique<gbcc::BatchCcsd>(ctx->c, std::move(sys));
    *out = b.release();
    return GBCC_OK;
  });
}

gbcc_status gbcc_ccsd_batch_step(gbcc_batch *b, int n, gbcc_status *status) {
  if (!b) return GBCC_BAD_ARG;
  return guard(b->ctx, [&]() {
    b->b->run(n);
    if (status)
      for (int z = 0; z < b->b->size(); ++z) {
        const gbcc::Ccsd &c = b->b->system(z);
        status[z] = b->b->status(z) != GBCC_OK
                        ? b->b->status(z)
                        : (c.converged() ? GBCC_OK : GBCC_NOT_CONVERGED);
      }
    return GBCC_OK;
  });
}

gbcc_status gbcc_ccsd_batch_result(gbcc_batch *b, int z, gbcc_ccsd_out *out) {
  if (!b || !out || z < 0 || z >= b->b->size()) return GBCC_BAD_ARG;
  return guard(b->ctx, [&]() {
    fill_result(b->b->system(z), b->ctx->c, out);
    GBCC_CUDA(cudaStreamSynchronize(b->ctx->c.stream));
    return GBCC_OK;
  });
}

gbcc_status gbcc_ccsd_batch_triples(gbcc_batch *b, int z, int precision, double *e_total,
                                    double *e_t) {
  if (!b || z < 0 || z >= b->b->size()) return GBCC_BAD_ARG;
  return guard(b->ctx, [&]() {
    gbcc::Ccsd &c = b->b->system(z);
    const double *T = c.amplitudes();
    const double et = gbcc::triples_energy(b->ctx->c, c.inputs(), T, T + c.layout().off2,
                                           precision);
    if (e_t) *e_t = et;
    if (e_total) *e_total = c.energy() + et;
    return GBCC_OK;
  });
}

void gbcc_ccsd_batch_destroy(gbcc_batch *b) {
  if (!b) return;
  cudaSetDevice(b->ctx->c.device);
  b->b.reset();
  cudaStreamSynchronize(b->ctx->c.stream);
  delete b;
}

gbcc_status gbcc_ccsd_solve_batch(gbcc_ctx *ctx, int nsys, const gbcc_ccsd_in *ins,
                                  const gbcc_ccsd_opts *opts, gbcc_ccsd_out *outs,
                                  gbcc_status *status) {
  if (!ctx || !ins || nsys < 1 || !status) return GBCC_BAD_ARG;
  gbcc_ccsd_opts o;
  if (opts) o = *opts; else gbcc_ccsd_opts_default(&o);
  if (o.max_iterations < 1) {
    ctx->c.last_error = "a batch of systems needs maxIterations >= 1";
    return GBCC_BAD_ARG;
  }
  gbcc_batch *b = nullptr;
  gbcc_status st = gbcc_ccsd_batch_setup(ctx, nsys, ins, &o, &b);
  if (st != GBCC_OK) return st;
  st = gbcc_ccsd_batch_step(b, o.max_iterations, status);
  for (int z = 0; z < nsys && st == GBCC_OK && outs; ++z)
    st = gbcc_ccsd_batch_result(b, z, &outs[z]);
  gbcc_ccsd_batch_destroy(b);
  return st;
}

gbcc_status gbcc_ccsd_result(gbcc_solver *s, gbcc_ccsd_out *out) {
  if (!s || !out) return GBCC_BAD_ARG;
  return guard(s->ctx, [&]() {
    fill_result(*s->s, s->ctx->c, out);
    GBCC_CUDA(cudaStreamSynchronize(s->ctx->c.stream));
    return GBCC_OK;
  });
}

gbcc_status gbcc_ccsd_device_amplitudes(gbcc_solver *s, const double **T1,
                                        const double **T2) {
  if (!s) return GBCC_BAD_ARG;
  if (T1) *T1 = s->s->amplitudes();
  if (T2) *T2 = s->s->amplitudes() + s->s->layout().off2;
  return GBCC_OK;
}

gbcc_status gbcc_ccsd_restart(gbcc_solver *s) {
  if (!s) return GBCC_BAD_ARG;
  return guard(s->ctx, [&]() {
    s->s->restart();
    return GBCC_OK;
  });
}

void gbcc_ccsd_destroy(gbcc_solver *s) {
  if (!s) return;
  cudaSetDevice(s->ctx->c.device);
  s->s.reset();
  cudaStreamSynchronize(s->ctx->c.stream);
  delete s;
}

gbcc_status gbcc_ccsd_solve(gbcc_ctx *ctx, const gbcc_ccsd_in *in,
                            const gbcc_ccsd_opts *opts, gbcc_ccsd_out *out) {
  gbcc_solver *s = nullptr;
  gbcc_status st = gbcc_ccsd_setup(ctx, in, opts, &s);
  if (st != GBCC_OK) return st;
  double e = 0;
  int conv = 0;
  st = gbcc_ccsd_step(s, s->opts.max_iterations, &e, &conv);
  if (st == GBCC_OK && s->opts.max_iterations == 0) {
    // ClusterSinglesDoublesAlgorithm.cxx:113-119: no iteration runs; the
    // energy of the given (or zero) amplitudes is reported, without the
    // non-convergence warning
    st = guard(ctx, [&]() {
      s->s->evaluate_energy();
      return GBCC_OK;
    });
    conv = 1;
  }
  gbcc_status st2 = GBCC_OK;
  if (out) st2 = gbcc_ccsd_result(s, out);
  gbcc_ccsd_destroy(s);
  if (st != GBCC_OK) return st;
  if (st2 != GBCC_OK) return st2;
  return conv ? GBCC_OK : GBCC_NOT_CONVERGED;
}

gbcc_status gbcc_ccsd_residual(gbcc_ctx *ctx, const gbcc_ccsd_in *in,
                               const gbcc_ccsd_opts *opts, int it,
                               const double *T1, const double *T2, double *R1,
                               double *R2) {
  if (!ctx || !in || !T1 || !T2 || !R1 || !R2) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc_ccsd_opts o;
    if (opts) o = *opts; else gbcc_ccsd_opts_default(&o);
    check_opts(o);
    apply_precision_opts(ctx->c, o);
    auto inputs = gbcc::upload_inputs(ctx->c, *in, o.precision, true, o.formulation == 1);
    gbcc::Ccsd c(ctx->c, std::move(inputs), o, in->init_T1, in->init_T2);
    const auto &L = c.layout();
    gbcc::DBuf T(ctx->c, 8 * L.ntot), R(ctx->c, 8 * L.ntot);
    gbcc::fill(ctx->c, T.as<double>(), L.ntot, 0.0);
    GBCC_CUDA(cudaMemcpyAsync(T.as<double>(), T1, 8 * L.n1,
                              cudaMemcpyHostToDevice, ctx->c.stream));
    GBCC_CUDA(cudaMemcpyAsync(T.as<double>() + L.off2, T2, 8 * L.n2,
                              cudaMemcpyHostToDevice, ctx->c.stream));
    c.residual(it, T.as<double>(), R.as<double>());
    GBCC_CUDA(cudaMemcpyAsync(R1, R.as<double>(), 8 * L.n1,
                              cudaMemcpyDeviceToHost, ctx->c.stream));
    GBCC_CUDA(cudaMemcpyAsync(R2, R.as<double>() + L.off2, 8 * L.n2,
                              cudaMemcpyDeviceToHost, ctx->c.stream));
    ctx->c.check_device_errors();
    return GBCC_OK;
  });
}

gbcc_status gbcc_ccsd_solve_complex(gbcc_ctx *ctx, const gbcc_ccsd_complex_in *in,
                                    const gbcc_ccsd_opts *opts,
                                    gbcc_ccsd_complex_out *out) {
  if (!ctx || !in) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc_ccsd_opts o;
    if (opts) o = *opts; else gbcc_ccsd_opts_default(&o);
    check_opts(o);
    apply_precision_opts(ctx->c, o);
    return gbcc::complex_solve(ctx->c, *in, o, out);
  });
}

gbcc_status gbcc_ccsd_residual_complex(gbcc_ctx *ctx, const gbcc_ccsd_complex_in *in,
                                       const gbcc_ccsd_opts *opts, int it,
                                       const double *T1, const double *T2,
                                       double *R1, double *R2) {
  if (!ctx || !in || !T1 || !T2 || !R1 || !R2) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc_ccsd_opts o;
    if (opts) o = *opts; else gbcc_ccsd_opts_default(&o);
    check_opts(o);
    apply_precision_opts(ctx->c, o);
    gbcc::complex_residual(ctx->c, *in, o, it, T1, T2, R1, R2);
    ctx->c.check_device_errors();
    return GBCC_OK;
  });
}

gbcc_status gbcc_triples_complex(gbcc_ctx *ctx, const gbcc_triples_complex_in *in,
                                 int precision, double *e_total, double *e_t) {
  if (!ctx || !in) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc::require(precision == GBCC_PREC_FP64 || precision == GBCC_PREC_EMU,
                  "unknown precision");
    gbcc::complex_triples(ctx->c, *in, precision, e_total, e_t);
    return GBCC_OK;
  });
}

gbcc_status gbcc_triples(gbcc_ctx *ctx, const gbcc_triples_in *in,
                         int precision, double *e_total, double *e_t) {
  if (!ctx || !in || !in->T1 || !in->T2) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc::require(precision == GBCC_PREC_FP64 || precision == GBCC_PREC_EMU,
                  "unknown precision");
    gbcc_ccsd_in ci{};
    ci.No = in->No; ci.Nv = in->Nv; ci.NG = in->NG;
    ci.eps_h = in->eps_h; ci.eps_p = in->eps_p;
    ci.gamma = in->gamma; ci.gamma_imag = in->gamma_imag;
    ci.Vabij = in->Vabij; ci.Vijka = in->Vijka;
    auto inputs = gbcc::upload_inputs(ctx->c, ci, precision, false);
    const int64_t No = in->No, Nv = in->Nv;
    gbcc::DBuf T1(ctx->c, 8 * Nv * No), T2(ctx->c, 8 * Nv * Nv * No * No);
    GBCC_CUDA(cudaMemcpyAsync(T1.as<double>(), in->T1, 8 * Nv * No,
                              cudaMemcpyHostToDevice, ctx->c.stream));
    GBCC_CUDA(cudaMemcpyAsync(T2.as<double>(), in->T2, 8 * Nv * Nv * No * No,
                              cudaMemcpyHostToDevice, ctx->c.stream));
    const double et = gbcc::triples_energy(ctx->c, *inputs, T1.as<double>(),
                                           T2.as<double>(), precision);
    if (e_t) *e_t = et;
    if (e_total) *e_total = in->e_ccsd + et;  // CcsdPerturbativeTriples.cxx:240-247
    return GBCC_OK;
  });
}

gbcc_status gbcc_triples_from_solver(gbcc_solver *s, int precision,
                                     double *e_total, double *e_t) {
  if (!s) return GBCC_BAD_ARG;
  return guard(s->ctx, [&]() {
    gbcc::Ccsd &c = *s->s;
    const double *T = c.amplitudes();
    const double et = gbcc::triples_energy(s->ctx->c, c.inputs(), T,
                                           T + c.layout().off2, precision);
    if (e_t) *e_t = et;
    if (e_total) *e_total = c.energy() + et;
    return GBCC_OK;
  });
}

gbcc_status gbcc_coulomb_integrals(gbcc_ctx *ctx, int No, int Nv, int NG,
                                   const double *gamma, double *Vabij,
                                   double *Vaibj, double *Vijkl, double *Vijka,
                                   double *Vijab) {
  if (!ctx || !gamma) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc::require(No > 0 && Nv > 0 && NG > 0, "No, Nv, NG must be positive");
    gbcc_ccsd_in ci{};
    ci.No = No; ci.Nv = Nv; ci.NG = NG;
    std::vector<double> eh(No, 0.0), ep(Nv, 0.0);
    ci.eps_h = eh.data();
    ci.eps_p = ep.data();
    ci.gamma = gamma;
    auto I = gbcc::upload_inputs(ctx->c, ci, GBCC_PREC_FP64, true);
    cudaStream_t st = ctx->c.stream;
    const int64_t o = No, v = Nv;
    if (Vabij) GBCC_CUDA(cudaMemcpyAsync(Vabij, I->Vabij.p(), 8 * v * v * o * o, cudaMemcpyDeviceToHost, st));
    if (Vaibj) GBCC_CUDA(cudaMemcpyAsync(Vaibj, I->Vaibj.p(), 8 * v * v * o * o, cudaMemcpyDeviceToHost, st));
    if (Vijkl) GBCC_CUDA(cudaMemcpyAsync(Vijkl, I->Vijkl.p(), 8 * o * o * o * o, cudaMemcpyDeviceToHost, st));
    if (Vijka) GBCC_CUDA(cudaMemcpyAsync(Vijka, I->Vijka.p(), 8 * o * o * o * v, cudaMemcpyDeviceToHost, st));
    if (Vijab) {
      // CoulombIntegralsFromVertex.cxx:491 Vijab["ijab"] = Vabij["abij"]
      gbcc::OTen t(ctx->c, {o, o, v, v});
      gbcc::assign(ctx->c, 1.0, I->Vabij, "abij", 0.0, t, "ijab");
      GBCC_CUDA(cudaMemcpyAsync(Vijab, t.p(), 8 * v * v * o * o, cudaMemcpyDeviceToHost, st));
      GBCC_CUDA(cudaStreamSynchronize(st));
    }
    GBCC_CUDA(cudaStreamSynchronize(st));
    return GBCC_OK;
  });
}

gbcc_status gbcc_coulomb_integrals_pp(gbcc_ctx *ctx, int No, int Nv, int NG,
                                      const double *gamma, double *Vabcd, double *Vabci) {
  if (!ctx || !gamma) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc::require(No > 0 && Nv > 0 && NG > 0, "No, Nv, NG must be positive");
    gbcc_ccsd_in ci{};
    ci.No = No; ci.Nv = Nv; ci.NG = NG;
    std::vector<double> eh(No, 0.0), ep(Nv, 0.0);
    ci.eps_h = eh.data();
    ci.eps_p = ep.data();
    ci.gamma = gamma;
    auto I = gbcc::upload_inputs(ctx->c, ci, GBCC_PREC_FP64, false, true);
    cudaStream_t st = ctx->c.stream;
    const int64_t o = No, v = Nv;
    if (Vabcd) GBCC_CUDA(cudaMemcpyAsync(Vabcd, I->Vabcd.p(), 8 * v * v * v * v, cudaMemcpyDeviceToHost, st));
    if (Vabci) GBCC_CUDA(cudaMemcpyAsync(Vabci, I->Vabci.p(), 8 * v * v * v * o, cudaMemcpyDeviceToHost, st));
    GBCC_CUDA(cudaStreamSynchronize(st));
    return GBCC_OK;
  });
}

gbcc_status gbcc_coulomb_integrals_complex(gbcc_ctx *ctx, int No, int Nv, int NG,
                                           const double *gamma, double *Vabij,
                                           double *Vaijb, double *Vijab, double *Vaibj,
                                           double *Vijkl, double *Vijka, double *Vaijk) {
  if (!ctx || !gamma) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc::require(No > 0 && Nv > 0 && NG > 0, "No, Nv, NG must be positive");
    double *const out[7] = {Vabij, Vaijb, Vijab, Vaibj, Vijkl, Vijka, Vaijk};
    gbcc::complex_integrals(ctx->c, No, Nv, NG, gamma, out);
    return GBCC_OK;
  });
}

gbcc_status gbcc_dgemm(gbcc_ctx *ctx, int transA, int transB, int64_t M,
                       int64_t N, int64_t K, double alpha, const double *A,
                       int64_t lda, const double *B, int64_t ldb, double beta,
                       double *C, int64_t ldc, int precision) {
  if (!ctx) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc::require(M >= 0 && N >= 0 && K >= 0, "negative size");
    gbcc::gemm(ctx->c, transA != 0, transB != 0, M, N, K, alpha, A, lda, B,
               ldb, beta, C, ldc, 1, 0, 0, 0, precision);
    ctx->c.check_device_errors();
    return GBCC_OK;
  });
}

gbcc_status gbcc_dgemm_emu_noalloc(gbcc_ctx *ctx, int transA, int transB,
                                   int64_t M, int64_t N, int64_t K,
                                   double alpha, const double *A, int64_t lda,
                                   const double *B, int64_t ldb, double beta,
                                   double *C, int64_t ldc) {
  if (!ctx) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc::gemm_emu_noalloc(ctx->c, transA != 0, transB != 0, M, N, K, alpha, A,
                           lda, B, ldb, beta, C, ldc);
    return GBCC_OK;
  });
}

gbcc_status gbcc_energy(gbcc_ctx *ctx, int No, int Nv, const double *T1,
                        const double *T2, const double *Vabij, double *direct,
                        double *exchange) {
  if (!ctx || !T1 || !T2 || !Vabij) return GBCC_BAD_ARG;
  return guard(ctx, [&]() {
    gbcc::require(No > 0 && Nv > 0, "No and Nv must be positive");
    gbcc::Context &c = ctx->c;
    const int64_t o = No, v = Nv;
    gbcc::OTen Vx(c, {v, v, o, o});
    gbcc::assign(c, 1.0, gbcc::ten(const_cast<double *>(Vabij), {v, v, o, o}),
                 "baij", 0.0, Vx, "abij");
    const int nb = gbcc::reduction_blocks(c, v * v * o * o);
    gbcc::DBuf part(c, 8 * nb * 4), sums(c, 8 * 4);
    gbcc::energy_terms(c, T1, T2, Vabij, Vx.p(), v, o, part.as<double>(),
                       sums.as<double>());
    double h[4];
    GBCC_CUDA(cudaMemcpyAsync(h, sums.as<double>(), sizeof(h),
                              cudaMemcpyDeviceToHost, c.stream));
    GBCC_CUDA(cudaStreamSynchronize(c.stream));
    double d = 2.0 * h[0];
    d = d + 2.0 * h[1];
    double x = -1.0 * h[2];
    x = x + -1.0 * h[3];
    if (direct) *direct = d;
    if (exchange) *exchange = x;
    return GBCC_OK;
  });
}

}  // extern "C"
