// Complex (k-point) CCSD and (T) on the GPU: the programs of
// ccsd_complex.hpp run on the CUDA backend of device_backend.hpp, whose
// primitives are routines the real path already uses, applied to one real
// plane at a time.  This file holds the entry points (host code only; the
// (T) denominator kernel is in ccsd_complex_kernels.cu).  Interleaved complex
// host data become two planes through one transpose of a [2, n] view.
#include <algorithm>
#include <cmath>

#include "device_backend.hpp"

namespace gbcc {
namespace {

cx::HostIn host_in(const gbcc_ccsd_complex_in &in) {
  require(in.No > 0 && in.Nv > 0 && in.NG > 0, "No, Nv, NG must be positive");
  require(in.eps_h && in.eps_p && in.gamma, "eigenenergies and the vertex are required");
  cx::HostIn h;
  h.No = in.No;
  h.Nv = in.Nv;
  h.NG = in.NG;
  h.eps_h = in.eps_h;
  h.eps_p = in.eps_p;
  h.gamma = in.gamma;
  h.init_T1 = in.init_T1;
  h.init_T2 = in.init_T2;
  h.fock_hp = in.fock_hp;
  return h;
}

// integralsSliceSize: given, else the real path's device default (Nv / 8, at
// least 16), capped so that one complex V_xycd slice stays within 4 GiB
int64_t slice_size(const gbcc_ccsd_opts &o, int64_t Nv) {
  int64_t s;
  if (o.integrals_slice_size > 0) s = o.integrals_slice_size;
  else if (o.integrals_slice_factor >= 0) s = (int64_t)(Nv * o.integrals_slice_factor);
  else {
    const double budget = 4.0 * 1024 * 1024 * 1024 / 16.0;
    const int64_t cap = (int64_t)std::floor(std::sqrt(budget / (double)(Nv * Nv)));
    s = std::min<int64_t>(cap, std::max<int64_t>(16, Nv / 8));
  }
  return std::max<int64_t>(1, std::min<int64_t>(s, Nv));
}

}  // namespace

void complex_residual(Context &ctx, const gbcc_ccsd_complex_in &in, const gbcc_ccsd_opts &o,
                      int it, const double *T1, const double *T2, double *R1, double *R2) {
  DeviceBackend rb{ctx, o.precision};
  cx::Inputs<DeviceBackend> I;
  cx::CBuf<DeviceBackend> T;
  cx::HostIn h = host_in(in);
  h.init_T1 = T1;
  h.init_T2 = T2;
  cx::setup(rb, I, h, T);
  cx::ResidualOpts ro;
  // getResiduum's MP2 start depends on whether initial doubles were given
  ro.init_doubles = in.init_T2 != nullptr;
  ro.distinguishable = o.distinguishable != 0;
  ro.ppl = o.ppl != 0;
  ro.slice = slice_size(o, in.Nv);
  const cx::Layout L(in.Nv, in.No);
  auto R = cx::cbuf(rb, {L.ntot});
  cx::residual(rb, I, it, ro, cx::t1_of(T, L), cx::t2_of(T, L), cx::t1_of(R, L),
               cx::t2_of(R, L));
  rb.store_complex(cx::t1_of(R, L), R1);
  rb.store_complex(cx::t2_of(R, L), R2);
}

gbcc_status complex_solve(Context &ctx, const gbcc_ccsd_complex_in &in,
                          const gbcc_ccsd_opts &o, gbcc_ccsd_complex_out *out) {
  require(o.mixer == 0,
          "DiisMixer is not available for complex amplitudes: the reference's complex "
          "DIIS solve is unimplemented (src/mixers/DiisMixer.cxx:43-48)");
  DeviceBackend rb{ctx, o.precision};
  cx::Inputs<DeviceBackend> I;
  cx::CBuf<DeviceBackend> T;
  cx::SolveOpts so;
  so.res.init_doubles = cx::setup(rb, I, host_in(in), T);
  so.res.distinguishable = o.distinguishable != 0;
  so.res.ppl = o.ppl != 0;
  so.res.slice = slice_size(o, in.Nv);
  so.max_iterations = o.max_iterations;
  so.energy_convergence = o.energy_convergence;
  so.amplitudes_convergence = o.amplitudes_convergence;
  so.level_shift = o.level_shift;
  so.mixing_ratio = o.mixing_ratio;
  const cx::SolveResult r = cx::solve(rb, I, so, T);
  for (const auto &e : r.history)
    if (!std::isfinite(e.real()) || !std::isfinite(e.imag()))
      throw Error(GBCC_DIVERGED, "the complex CCSD energy is not finite");
  if (out) {
    out->energy[0] = r.energy.value.real();
    out->energy[1] = r.energy.value.imag();
    out->direct[0] = r.energy.direct.real();
    out->direct[1] = r.energy.direct.imag();
    out->exchange[0] = r.energy.exchange.real();
    out->exchange[1] = r.energy.exchange.imag();
    out->iterations = r.iterations;
    out->converged = r.converged ? 1 : 0;
    const cx::Layout L(in.Nv, in.No);
    if (out->T1) rb.store_complex(cx::t1_of(T, L), out->T1);
    if (out->T2) rb.store_complex(cx::t2_of(T, L), out->T2);
    if (out->energy_history)
      for (size_t q = 0; q < r.history.size(); ++q) {
        out->energy_history[2 * q] = r.history[q].real();
        out->energy_history[2 * q + 1] = r.history[q].imag();
      }
    if (out->pair_energy) {
      const auto p = cx::pair_energy(rb, I, cx::t1_of(T, L), cx::t2_of(T, L));
      for (size_t q = 0; q < p.size(); ++q) {
        out->pair_energy[2 * q] = p[q].real();
        out->pair_energy[2 * q + 1] = p[q].imag();
      }
    }
  }
  ctx.check_device_errors();
  return (r.converged || o.max_iterations == 0) ? GBCC_OK : GBCC_NOT_CONVERGED;
}

void complex_integrals(Context &ctx, int No, int Nv, int NG, const double *gamma,
                       double *const out[7]) {
  DeviceBackend rb{ctx, GBCC_PREC_FP64};
  cx::Inputs<DeviceBackend> I;
  cx::CBuf<DeviceBackend> T;
  gbcc_ccsd_complex_in ci{};
  ci.No = No; ci.Nv = Nv; ci.NG = NG;
  std::vector<double> eh(No, 0.0), ep(Nv, 0.0);
  ci.eps_h = eh.data();
  ci.eps_p = ep.data();
  ci.gamma = gamma;
  cx::setup(rb, I, host_in(ci), T);
  const cx::CBuf<DeviceBackend> *blocks[7] = {&I.Vabij, &I.Vaijb, &I.Vijab, &I.Vaibj,
                                              &I.Vijkl, &I.Vijka, &I.Vaijk};
  for (int q = 0; q < 7; ++q)
    if (out[q]) rb.store_complex(blocks[q]->v(), out[q]);
  ctx.check_device_errors();
}

void complex_triples(Context &ctx, const gbcc_triples_complex_in &in, int precision,
                     double *e_total, double *e_t) {
  require(in.T1 && in.T2, "CcsdSinglesAmplitudes and CcsdDoublesAmplitudes are required");
  DeviceBackend rb{ctx, precision};
  cx::Inputs<DeviceBackend> I;
  cx::CBuf<DeviceBackend> T;
  gbcc_ccsd_complex_in ci{};
  ci.No = in.No; ci.Nv = in.Nv; ci.NG = in.NG;
  ci.eps_h = in.eps_h; ci.eps_p = in.eps_p; ci.gamma = in.gamma;
  ci.init_T1 = in.T1; ci.init_T2 = in.T2;
  cx::setup(rb, I, host_in(ci), T);
  const cx::Layout L(in.Nv, in.No);
  const std::complex<double> e = cx::triples(rb, I, cx::t1_of(T, L), cx::t2_of(T, L));
  ctx.check_device_errors();
  if (e_t) {
    e_t[0] = e.real();
    e_t[1] = e.imag();
  }
  if (e_total) *e_total = in.e_ccsd + e.real();  // CcsdPerturbativeTriplesComplex.cxx:77-84
}

}  // namespace gbcc
