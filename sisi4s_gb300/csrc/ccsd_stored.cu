// The stored-integral CCSD residual (CcsdEnergyFromCoulombIntegralsReference)
// inside the device solver: the program of ccsd_stored.hpp on the CUDA
// backend, on the solver's resident integrals.  The driver around it (update,
// mixers, energy, graphs) is the one of the vertex formulation.
#include "ccsd.hpp"
#include "ccsd_stored.hpp"
#include "device_backend.hpp"

namespace gbcc {

namespace {
cx::View as_view(const Ten &t) {
  cx::View v;
  v.p = t.p;
  v.order = t.order;
  v.lens = t.lens;
  return v;
}
}  // namespace

void Ccsd::residual_stored(int it, const double *Tp, double *Rp) {
  CcsdInputs &I = *in_;
  require(I.Vabcd.p() && I.Vabci.p() && I.Vaibj.p() && I.Vijkl.p(),
          "the stored formulation needs PPPP, PPPH, PHPH and HHHH integrals");
  DeviceBackend rb{ctx_, o_.precision};
  st::Ints ints;
  ints.Vabij = as_view(I.Vabij);
  ints.Vaibj = as_view(I.Vaibj);
  ints.Vijkl = as_view(I.Vijkl);
  ints.Vijka = as_view(I.Vijka);
  ints.Vabcd = as_view(I.Vabcd);
  ints.Vabci = as_view(I.Vabci);
  st::Opts so;
  so.init_doubles = init_doubles_;
  so.only_ppl = o_.only_ppl != 0;
  fill(ctx_, Rp, L_.ntot, 0.0);  // the padding between T1 and T2 included
  double *T = const_cast<double *>(Tp);
  const int64_t Nv = L_.Nv, No = L_.No;
  st::residual(rb, ints, it, so, cx::view(T, {Nv, No}), cx::view(T + L_.off2, {Nv, Nv, No, No}),
               cx::view(Rp, {Nv, No}), cx::view(Rp + L_.off2, {Nv, Nv, No, No}));
}

}  // namespace gbcc
