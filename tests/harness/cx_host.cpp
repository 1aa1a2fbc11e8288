// Host backend for the complex CCSD program (test infrastructure only).
//
// Instantiates sisi4s_gb300/csrc/ccsd_complex.hpp -- the same statement
// sequence the library runs on the GPU -- with naive host loops for the real
// primitives, so that tests can compare the program with the oracle without a
// GPU.  Each primitive restates the semantics of the library kernel it stands
// for (csrc/contract.cu, csrc/ccsd_kernels.cu).  Built by the tests with g++;
// nothing in the library links it.
#include <cmath>
#include <cstring>
#include <exception>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "ccsd_complex.hpp"
#include "ccsd_stored.hpp"

namespace {

using gbcc::cx::View;

struct HostBackend {
  struct Buf {
    std::vector<double> mem;
    View v;
  };

  Buf alloc(std::initializer_list<int64_t> l) {
    Buf b;
    b.v = gbcc::cx::view(nullptr, l);
    b.mem.assign((size_t)b.v.size(), std::nan(""));  // contents undefined
    b.v.p = b.mem.data();
    return b;
  }

  static void strides(const View &t, int64_t *st) {
    int64_t s = 1;
    for (int d = 0; d < t.order; ++d) {
      st[d] = s;
      s *= t.lens[d];
    }
  }

  // C = al A.B + be C over the union of the index letters
  void contract(double al, const View &A, const char *ia, const View &B, const char *ib,
                double be, const View &C, const char *ic) {
    const std::string sa(ia), sb(ib), sc(ic);
    if ((int)sa.size() != A.order || (int)sb.size() != B.order || (int)sc.size() != C.order)
      throw std::runtime_error("contract: order mismatch " + sa + "," + sb + "->" + sc);
    std::string all;
    int64_t len[256];
    for (auto &x : len) x = -1;
    auto bind = [&](const std::string &s, const View &t) {
      for (size_t d = 0; d < s.size(); ++d) {
        const unsigned char c = (unsigned char)s[d];
        if (len[c] < 0) {
          len[c] = t.lens[d];
          all += s[d];
        } else if (len[c] != t.lens[d]) {
          throw std::runtime_error("contract: length mismatch " + sa + "," + sb + "->" + sc);
        }
      }
    };
    bind(sa, A);
    bind(sb, B);
    bind(sc, C);
    // the statements must also be acceptable to the library's contraction
    // engine (csrc/contract.cu): no batch indices, no index summed inside one
    // operand, no output that aliases an operand
    auto has = [](const std::string &s, char c) { return s.find(c) != std::string::npos; };
    for (char c : sa) {
      if (has(sb, c) && has(sc, c)) throw std::runtime_error("contract: batch index " + sa + "," + sb + "->" + sc);
      if (!has(sb, c) && !has(sc, c)) throw std::runtime_error("contract: index summed in one operand");
    }
    for (char c : sb)
      if (!has(sa, c) && !has(sc, c)) throw std::runtime_error("contract: index summed in one operand");
    for (char c : sc)
      if (!has(sa, c) && !has(sb, c))
        throw std::runtime_error("contract: output index not in an operand");
    if (C.p == A.p || C.p == B.p) throw std::runtime_error("contract: output aliases an operand");
    int64_t stA[6], stB[6], stC[6];
    strides(A, stA);
    strides(B, stB);
    strides(C, stC);
    const int n = (int)all.size();
    std::vector<int64_t> dA(n, 0), dB(n, 0), dC(n, 0), ext(n);
    for (int q = 0; q < n; ++q) {
      const char c = all[q];
      ext[q] = len[(unsigned char)c];
      size_t f;
      if ((f = sa.find(c)) != std::string::npos) dA[q] = stA[f];
      if ((f = sb.find(c)) != std::string::npos) dB[q] = stB[f];
      if ((f = sc.find(c)) != std::string::npos) dC[q] = stC[f];
    }
    const int64_t nc = C.size();
    for (int64_t e = 0; e < nc; ++e) C.p[e] = (be == 0.0) ? 0.0 : be * C.p[e];
    int64_t total = 1;
    for (int q = 0; q < n; ++q) total *= ext[q];
    std::vector<int64_t> idx(n, 0);
    for (int64_t t = 0; t < total; ++t) {
      int64_t oa = 0, ob = 0, oc = 0;
      for (int q = 0; q < n; ++q) {
        oa += idx[q] * dA[q];
        ob += idx[q] * dB[q];
        oc += idx[q] * dC[q];
      }
      C.p[oc] += al * A.p[oa] * B.p[ob];
      for (int q = 0; q < n; ++q) {
        if (++idx[q] < ext[q]) break;
        idx[q] = 0;
      }
    }
  }

  // C = al A[perm] + be C
  void assign(double al, const View &A, const char *ia, double be, const View &C,
              const char *ic) {
    const std::string sa(ia), sc(ic);
    if ((int)sa.size() != A.order || (int)sc.size() != C.order || sa.size() != sc.size())
      throw std::runtime_error("assign: bad index strings " + sa + "->" + sc);
    if (A.p == C.p) throw std::runtime_error("assign: in-place permutation");
    int64_t stA[6];
    strides(A, stA);
    const int n = C.order;
    std::vector<int64_t> dA(n);
    for (int q = 0; q < n; ++q) {
      const size_t f = sa.find(sc[q]);
      if (f == std::string::npos || A.lens[f] != C.lens[q])
        throw std::runtime_error("assign: index mismatch " + sa + "->" + sc);
      dA[q] = stA[f];
    }
    std::vector<int64_t> idx(n, 0);
    const int64_t nc = C.size();
    for (int64_t e = 0; e < nc; ++e) {
      int64_t oa = 0;
      for (int q = 0; q < n; ++q) oa += idx[q] * dA[q];
      C.p[e] = al * A.p[oa] + ((be == 0.0) ? 0.0 : be * C.p[e]);
      for (int q = 0; q < n; ++q) {
        if (++idx[q] < C.lens[q]) break;
        idx[q] = 0;
      }
    }
  }

  void fill(const View &x, double v) {
    for (int64_t e = 0; e < x.size(); ++e) x.p[e] = v;
  }

  void axpby(double a, const View &x, double b, const View &y) {
    if (x.size() != y.size()) throw std::runtime_error("axpby: size mismatch");
    for (int64_t e = 0; e < y.size(); ++e)
      y.p[e] = a * x.p[e] + ((b == 0.0) ? 0.0 : b * y.p[e]);
  }

  // gather_slice_kernel: dst[G, x, c] = src[G, x0 + x, c] of a [G, Nv, Nv] src
  void gather_slice(const View &dst, const View &src, int64_t x0, int64_t nx) {
    const int64_t G = src.lens[0], Nv = src.lens[1];
    if (dst.lens[0] != G || dst.lens[1] != nx || dst.lens[2] != Nv || x0 + nx > Nv)
      throw std::runtime_error("gather_slice: bad shape");
    for (int64_t c = 0; c < Nv; ++c)
      for (int64_t x = 0; x < nx; ++x)
        for (int64_t g = 0; g < G; ++g)
          dst.p[g + G * (x + nx * c)] = src.p[g + G * ((x0 + x) + Nv * c)];
  }

  // slice_add_kernel: R[a0+x, b0+y, i, j] += Rxy[x,y,i,j];
  // mirror: R[b0+y, a0+x, j, i] += Rxy[x,y,i,j]
  void slice_add(const View &R, const View &Rxy, int64_t a0, int64_t b0, bool mirror) {
    const int64_t Nv = R.lens[0], No = R.lens[2];
    const int64_t nx = Rxy.lens[0], ny = Rxy.lens[1];
    if (a0 + nx > Nv || b0 + ny > Nv) throw std::runtime_error("slice_add: out of range");
    for (int64_t j = 0; j < No; ++j)
      for (int64_t i = 0; i < No; ++i)
        for (int64_t y = 0; y < ny; ++y)
          for (int64_t x = 0; x < nx; ++x) {
            const double v = Rxy.p[x + nx * (y + ny * (i + No * j))];
            R.p[(a0 + x) + Nv * ((b0 + y) + Nv * (i + No * j))] += v;
            if (mirror) R.p[(b0 + y) + Nv * ((a0 + x) + Nv * (j + No * i))] += v;
          }
  }

  // vertex_block_kernel: dst[G, p, q] = src[G, p0 + p, q0 + q] of [G, Np, Np]
  void vertex_block(const View &dst, const View &src, int64_t p0, int64_t np,
                    int64_t q0, int64_t nq) {
    const int64_t G = src.lens[0], Np = src.lens[1];
    for (int64_t q = 0; q < nq; ++q)
      for (int64_t p = 0; p < np; ++p)
        for (int64_t g = 0; g < G; ++g)
          dst.p[g + G * (p + np * q)] = src.p[g + G * ((p0 + p) + Np * (q0 + q))];
  }

  // update_kernel on one plane: the D of calculateExcitationEnergies in the
  // reference's order, est = -(R - s T)/(D + s), dT = est - T, zero padding
  void jacobi(const gbcc::cx::Layout &L, const View &eh, const View &ep, const View &R,
              const View &T, const View &est, const View &dT, double s, double sums[2]) {
    sums[0] = sums[1] = 0.0;
    for (int64_t e = 0; e < L.ntot; ++e) {
      double d;
      if (e < L.n1) {
        d = ep.p[e % L.Nv] - eh.p[e / L.Nv];
      } else if (e >= L.off2 && e < L.off2 + L.n2) {
        int64_t r = e - L.off2;
        const int64_t a = r % L.Nv; r /= L.Nv;
        const int64_t b = r % L.Nv; r /= L.Nv;
        const int64_t i = r % L.No, j = r / L.No;
        d = ((ep.p[a] - eh.p[i]) + ep.p[b]) - eh.p[j];
      } else {
        est.p[e] = dT.p[e] = 0.0;
        continue;
      }
      double r = R.p[e];
      if (s != 0.0) r = r - s * T.p[e];
      est.p[e] = -r / (d + s);
      dT.p[e] = est.p[e] - T.p[e];
      sums[0] += dT.p[e] * dT.p[e];
      sums[1] += est.p[e] * est.p[e];
    }
  }

  // linear_mix_kernel: last *= 1-r; next = r next + last; likewise residua
  void linear_mix(const View &next, const View &nres, const View &last, const View &lres,
                  double r, double sums[2]) {
    sums[0] = sums[1] = 0.0;
    const double q = 1.0 - r;
    for (int64_t e = 0; e < next.size(); ++e) {
      last.p[e] = last.p[e] * q;
      next.p[e] = next.p[e] * r + last.p[e];
      lres.p[e] = lres.p[e] * q;
      nres.p[e] = nres.p[e] * r + lres.p[e];
      sums[0] += nres.p[e] * nres.p[e];
      sums[1] += next.p[e] * next.p[e];
    }
  }

  double scalar(const View &x) { return x.p[0]; }
  void read(const View &x, double *h) { std::memcpy(h, x.p, sizeof(double) * x.size()); }

  // z = conj(z / D), D = (((e_i + e_j) + e_k) - e_a) - e_b) - e_c in the
  // reference's order (CcsdPerturbativeTriplesComplex.cxx:156-161, 224-229)
  void conj_over_denominator(const View &re, const View &im, const View &eh, const View &ep,
                             int64_t i0, int64_t i1, int64_t i2) {
    const int64_t Nv = ep.lens[0];
    const double hs = (eh.p[i0] + eh.p[i1]) + eh.p[i2];
    for (int64_t c = 0; c < Nv; ++c)
      for (int64_t b = 0; b < Nv; ++b)
        for (int64_t a = 0; a < Nv; ++a) {
          const int64_t e = a + Nv * (b + Nv * c);
          const double d = ((hs - ep.p[a]) - ep.p[b]) - ep.p[c];
          re.p[e] = re.p[e] / d;
          im.p[e] = -(im.p[e] / d);
        }
  }

  Buf load_real(const double *h, std::initializer_list<int64_t> l) {
    Buf b = alloc(l);
    std::memcpy(b.v.p, h, sizeof(double) * b.v.size());
    return b;
  }
  void load_complex(const double *h, const gbcc::cx::CView &dst) {
    for (int64_t e = 0; e < dst.re.size(); ++e) {
      dst.re.p[e] = h[2 * e];
      dst.im.p[e] = h[2 * e + 1];
    }
  }
  void store_complex(const gbcc::cx::CView &src, double *h) {
    for (int64_t e = 0; e < src.re.size(); ++e) {
      h[2 * e] = src.re.p[e];
      h[2 * e + 1] = src.im.p[e];
    }
  }
};

std::string g_err;

gbcc::cx::HostIn host_in(int No, int Nv, int NG, const double *eh, const double *ep,
                         const double *gamma, const double *T1, const double *T2,
                         const double *fock = nullptr) {
  gbcc::cx::HostIn h;
  h.No = No; h.Nv = Nv; h.NG = NG;
  h.eps_h = eh; h.eps_p = ep; h.gamma = gamma;
  h.init_T1 = T1; h.init_T2 = T2;
  h.fock_hp = fock;
  return h;
}

}  // namespace

extern "C" {

const char *cx_last_error() { return g_err.c_str(); }

// R = getResiduum(it, T); complex tensors interleaved (re, im)
int cx_residual(int No, int Nv, int NG, const double *eh, const double *ep,
                const double *gamma, int it, int init_doubles, int dist, int ppl,
                int slice, const double *T1, const double *T2, double *R1, double *R2) {
  try {
    HostBackend rb;
    gbcc::cx::Inputs<HostBackend> I;
    gbcc::cx::CBuf<HostBackend> T;
    gbcc::cx::ResidualOpts o;
    gbcc::cx::setup(rb, I, host_in(No, Nv, NG, eh, ep, gamma, T1, T2), T);
    o.init_doubles = init_doubles != 0;
    o.distinguishable = dist != 0;
    o.ppl = ppl != 0;
    o.slice = slice > 0 ? slice : No;
    const gbcc::cx::Layout L(Nv, No);
    auto R = gbcc::cx::cbuf(rb, {L.ntot});
    gbcc::cx::residual(rb, I, it, o, gbcc::cx::t1_of(T, L), gbcc::cx::t2_of(T, L),
                       gbcc::cx::t1_of(R, L), gbcc::cx::t2_of(R, L));
    rb.store_complex(gbcc::cx::t1_of(R, L), R1);
    rb.store_complex(gbcc::cx::t2_of(R, L), R2);
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// run<complex> with the linear mixer; energies as (re, im) pairs
int cx_solve(int No, int Nv, int NG, const double *eh, const double *ep,
             const double *gamma, const double *T1in, const double *T2in, int max_it,
             double econv, double aconv, double shift, double ratio, int dist, int ppl,
             int slice, double *energy, int *iterations, int *converged,
             double *history, double *T1, double *T2, const double *fock) {
  try {
    HostBackend rb;
    gbcc::cx::Inputs<HostBackend> I;
    gbcc::cx::CBuf<HostBackend> T;
    gbcc::cx::SolveOpts o;
    o.res.init_doubles =
        gbcc::cx::setup(rb, I, host_in(No, Nv, NG, eh, ep, gamma, T1in, T2in, fock), T);
    o.res.distinguishable = dist != 0;
    o.res.ppl = ppl != 0;
    o.res.slice = slice > 0 ? slice : No;
    o.max_iterations = max_it;
    o.energy_convergence = econv;
    o.amplitudes_convergence = aconv;
    o.level_shift = shift;
    o.mixing_ratio = ratio;
    const auto r = gbcc::cx::solve(rb, I, o, T);
    energy[0] = r.energy.value.real();
    energy[1] = r.energy.value.imag();
    *iterations = r.iterations;
    *converged = r.converged ? 1 : 0;
    for (size_t q = 0; q < r.history.size(); ++q) {
      history[2 * q] = r.history[q].real();
      history[2 * q + 1] = r.history[q].imag();
    }
    const gbcc::cx::Layout L(Nv, No);
    rb.store_complex(gbcc::cx::t1_of(T, L), T1);
    rb.store_complex(gbcc::cx::t2_of(T, L), T2);
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// stored-integral residual (real buffers, first index fastest)
int st_residual(int No, int Nv, int it, int init_doubles, int only_ppl, const double *Vabij,
                const double *Vaibj, const double *Vijkl, const double *Vijka,
                const double *Vabcd, const double *Vabci, const double *T1, const double *T2,
                double *R1, double *R2) {
  try {
    HostBackend rb;
    auto v = [](const double *p, std::initializer_list<int64_t> l) {
      return gbcc::cx::view(const_cast<double *>(p), l);
    };
    const int64_t o = No, n = Nv;
    gbcc::st::Ints I;
    I.Vabij = v(Vabij, {n, n, o, o});
    I.Vaibj = v(Vaibj, {n, o, n, o});
    I.Vijkl = v(Vijkl, {o, o, o, o});
    I.Vijka = v(Vijka, {o, o, o, n});
    I.Vabcd = v(Vabcd, {n, n, n, n});
    I.Vabci = v(Vabci, {n, n, n, o});
    gbcc::st::Opts opts;
    opts.init_doubles = init_doubles != 0;
    opts.only_ppl = only_ppl != 0;
    gbcc::st::residual(rb, I, it, opts, v(T1, {n, o}), v(T2, {n, n, o, o}), v(R1, {n, o}),
                       v(R2, {n, n, o, o}));
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// complex pair energies [No,No] (interleaved) of the given complex amplitudes
int cx_pair_energy(int No, int Nv, int NG, const double *eh, const double *ep,
                   const double *gamma, const double *T1, const double *T2, double *pe) {
  try {
    HostBackend rb;
    gbcc::cx::Inputs<HostBackend> I;
    gbcc::cx::CBuf<HostBackend> T;
    gbcc::cx::setup(rb, I, host_in(No, Nv, NG, eh, ep, gamma, T1, T2), T);
    const gbcc::cx::Layout L(Nv, No);
    const auto p = gbcc::cx::pair_energy(rb, I, gbcc::cx::t1_of(T, L), gbcc::cx::t2_of(T, L));
    for (size_t q = 0; q < p.size(); ++q) {
      pe[2 * q] = p[q].real();
      pe[2 * q + 1] = p[q].imag();
    }
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// complex (T) energy (re, im) of the given complex amplitudes
int cx_triples(int No, int Nv, int NG, const double *eh, const double *ep,
               const double *gamma, const double *T1, const double *T2, double *et) {
  try {
    HostBackend rb;
    gbcc::cx::Inputs<HostBackend> I;
    gbcc::cx::CBuf<HostBackend> T;
    gbcc::cx::setup(rb, I, host_in(No, Nv, NG, eh, ep, gamma, T1, T2), T);
    const gbcc::cx::Layout L(Nv, No);
    const std::complex<double> e =
        gbcc::cx::triples(rb, I, gbcc::cx::t1_of(T, L), gbcc::cx::t2_of(T, L));
    et[0] = e.real();
    et[1] = e.imag();
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

}  // extern "C"
