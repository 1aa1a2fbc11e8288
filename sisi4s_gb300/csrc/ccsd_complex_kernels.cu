// The one kernel of the complex (k-point) branch that the real path does not
// already have: the (T) denominator with its conjugation.  Every other
// device step of the complex branch runs on the real path's routines.
#include <algorithm>

#include "device_backend.hpp"

namespace gbcc {
namespace {

// z[a,b,c] = conj(z / D) with D = (((e_i + e_j) + e_k) - e_a) - e_b) - e_c
// (CcsdPerturbativeTriplesComplex.cxx:156-161, 224-229), on the two planes
__global__ void conj_over_denominator_kernel(double *__restrict__ re, double *__restrict__ im,
                                             const double *__restrict__ eh,
                                             const double *__restrict__ ep, int i0, int i1,
                                             int i2, int Nv) {
  const int n = Nv * Nv * Nv;
  const double hs = (eh[i0] + eh[i1]) + eh[i2];
  for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
    const int a = e % Nv, b = (e / Nv) % Nv, c = e / (Nv * Nv);
    const double d = ((hs - ep[a]) - ep[b]) - ep[c];
    re[e] = re[e] / d;
    im[e] = -(im[e] / d);
  }
}

}  // namespace

void conj_over_denominator(Context &ctx, double *re, double *im, const double *eh,
                           const double *ep, int64_t i0, int64_t i1, int64_t i2,
                           int64_t Nv) {
  const int64_t n = Nv * Nv * Nv;
  const int64_t cap = (int64_t)std::max(ctx.sm_count, 1) * 8;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, cap));
  conj_over_denominator_kernel<<<grid, 256, 0, ctx.stream>>>(re, im, eh, ep, (int)i0,
                                                             (int)i1, (int)i2, (int)Nv);
  GBCC_CHECK_LAUNCH(ctx);
}

}  // namespace gbcc
