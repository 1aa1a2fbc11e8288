// CUDA backend of the statement programs in ccsd_complex.hpp and
// ccsd_stored.hpp: each real primitive maps onto a routine the real CCSD path
// already runs (contraction engine, permutes, elementwise kernels, the slice
// gather/scatter of the ladder, the Jacobi update and the linear mixer).
#pragma once

#include <algorithm>

#include "ccsd_complex.hpp"
#include "ccsd_kernels.hpp"

namespace gbcc {

// z = conj(z / D^{ijk}_{abc}) on the two planes of an [Nv,Nv,Nv] tensor
void conj_over_denominator(Context &ctx, double *re, double *im, const double *eh,
                           const double *ep, int64_t i0, int64_t i1, int64_t i2,
                           int64_t Nv);

inline Ten as_ten(const cx::View &v) {
  Ten t;
  t.p = v.p;
  t.order = v.order;
  t.lens = v.lens;
  return t;
}

struct DeviceBackend {
  Context &ctx;
  int precision;

  struct Buf {
    DBuf mem;
    cx::View v;
  };

  Buf alloc(std::initializer_list<int64_t> l) {
    Buf b;
    b.v = cx::view(nullptr, l);
    b.mem.alloc(ctx, sizeof(double) * (size_t)std::max<int64_t>(b.v.size(), 1));
    b.v.p = b.mem.as<double>();
    return b;
  }
  void contract(double al, const cx::View &A, const char *ia, const cx::View &B,
                const char *ib, double be, const cx::View &C, const char *ic) {
    gbcc::contract(ctx, al, as_ten(A), ia, as_ten(B), ib, be, as_ten(C), ic, precision);
  }
  void assign(double al, const cx::View &A, const char *ia, double be, const cx::View &C,
              const char *ic) {
    gbcc::assign(ctx, al, as_ten(A), ia, be, as_ten(C), ic);
  }
  void fill(const cx::View &x, double v) { gbcc::fill(ctx, x.p, x.size(), v); }
  void axpby(double a, const cx::View &x, double b, const cx::View &y) {
    require(x.size() == y.size(), "axpby: size mismatch");
    gbcc::axpby(ctx, y.size(), a, x.p, b, y.p);
  }
  void gather_slice(const cx::View &dst, const cx::View &src, int64_t x0, int64_t nx) {
    require(dst.lens[0] == src.lens[0] && dst.lens[1] == nx && dst.lens[2] == src.lens[1] &&
                x0 + nx <= src.lens[1],
            "gather_slice: bad shape");
    gbcc::gather_slice(ctx, dst.p, src.p, src.lens[0], src.lens[1], x0, nx);
  }
  void slice_add(const cx::View &R, const cx::View &Rxy, int64_t a0, int64_t b0, bool mirror) {
    require(a0 + Rxy.lens[0] <= R.lens[0] && b0 + Rxy.lens[1] <= R.lens[1],
            "slice_add: out of range");
    gbcc::slice_add(ctx, R.p, Rxy.p, R.lens[0], R.lens[2], a0, b0, Rxy.lens[0],
                    Rxy.lens[1], mirror);
  }
  void vertex_block(const cx::View &dst, const cx::View &src, int64_t p0, int64_t np,
                    int64_t q0, int64_t nq) {
    require(p0 + np <= src.lens[1] && q0 + nq <= src.lens[2], "vertex_block: out of range");
    gbcc::vertex_block(ctx, dst.p, src.p, src.lens[0], src.lens[1], p0, np, q0, nq);
  }
  void read_sums(const double *dev, double *host, int64_t n) {
    GBCC_CUDA(cudaMemcpyAsync(host, dev, sizeof(double) * n, cudaMemcpyDeviceToHost,
                              ctx.stream));
    ctx.check_device_errors();
  }
  void jacobi(const cx::Layout &L, const cx::View &eh, const cx::View &ep, const cx::View &R,
              const cx::View &T, const cx::View &est, const cx::View &dT, double shift,
              double sums[2]) {
    const FockLayout fl(L.Nv, L.No);
    require(fl.ntot == L.ntot && R.size() == L.ntot, "jacobi: layout mismatch");
    DBuf part(ctx, sizeof(double) * reduction_blocks(ctx, fl.ntot) * 2), out(ctx, 16);
    jacobi_update(ctx, fl, R.p, T.p, est.p, dT.p, eh.p, ep.p, shift, 0, nullptr,
                  part.as<double>(), out.as<double>());
    read_sums(out.as<double>(), sums, 2);
  }
  void linear_mix(const cx::View &next, const cx::View &nres, const cx::View &last,
                  const cx::View &lres, double r, double sums[2]) {
    const int64_t n = next.size();
    DBuf part(ctx, sizeof(double) * reduction_blocks(ctx, n) * 2), out(ctx, 16);
    gbcc::linear_mix(ctx, next.p, nres.p, last.p, lres.p, r, n, part.as<double>(),
                     out.as<double>());
    read_sums(out.as<double>(), sums, 2);
  }
  void conj_over_denominator(const cx::View &re, const cx::View &im, const cx::View &eh,
                             const cx::View &ep, int64_t i0, int64_t i1, int64_t i2) {
    const int64_t Nv = ep.lens[0];
    require(Nv * Nv * Nv < (int64_t(1) << 30) && re.size() == Nv * Nv * Nv &&
                im.size() == re.size() && i0 < eh.lens[0] && i1 < eh.lens[0] &&
                i2 < eh.lens[0],
            "conj_over_denominator: bad shape");
    gbcc::conj_over_denominator(ctx, re.p, im.p, eh.p, ep.p, i0, i1, i2, Nv);
  }
  void read(const cx::View &x, double *h) { read_sums(x.p, h, x.size()); }
  double scalar(const cx::View &x) {
    double h = 0.0;
    read_sums(x.p, &h, 1);
    return h;
  }
  Buf load_real(const double *h, std::initializer_list<int64_t> l) {
    Buf b = alloc(l);
    GBCC_CUDA(cudaMemcpyAsync(b.v.p, h, sizeof(double) * b.v.size(),
                              cudaMemcpyHostToDevice, ctx.stream));
    return b;
  }
  // interleaved [2, n] on the host -> [n, 2] on the device -> two planes
  void load_complex(const double *h, const cx::CView &dst) {
    const int64_t n = dst.re.size();
    DBuf a(ctx, 16 * n), b(ctx, 16 * n);
    GBCC_CUDA(cudaMemcpyAsync(a.as<double>(), h, 16 * n, cudaMemcpyHostToDevice,
                              ctx.stream));
    gbcc::assign(ctx, 1.0, ten(a.as<double>(), {2, n}), "zn", 0.0,
                 ten(b.as<double>(), {n, 2}), "nz");
    gbcc::copy(ctx, dst.re.p, b.as<double>(), n);
    gbcc::copy(ctx, dst.im.p, b.as<double>() + n, n);
  }
  void store_complex(const cx::CView &src, double *h) {
    const int64_t n = src.re.size();
    DBuf a(ctx, 16 * n), b(ctx, 16 * n);
    gbcc::copy(ctx, b.as<double>(), src.re.p, n);
    gbcc::copy(ctx, b.as<double>() + n, src.im.p, n);
    gbcc::assign(ctx, 1.0, ten(b.as<double>(), {n, 2}), "nz", 0.0,
                 ten(a.as<double>(), {2, n}), "zn");
    GBCC_CUDA(cudaMemcpyAsync(h, a.as<double>(), 16 * n, cudaMemcpyDeviceToHost,
                              ctx.stream));
    ctx.check_device_errors();
  }
};

}  // namespace gbcc
