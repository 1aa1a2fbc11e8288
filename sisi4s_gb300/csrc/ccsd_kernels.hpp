// Host wrappers of the CCSD bandwidth kernels (ccsd_kernels.cu).
#pragma once

#include "internal.hpp"

#define GBCC_MAX_DIIS 16

namespace gbcc {

// Layout of one Fock vector (T1 then T2) in a single buffer.
struct FockLayout {
  int64_t Nv = 0, No = 0, n1 = 0, n2 = 0, off2 = 0, ntot = 0;
  FockLayout() = default;
  FockLayout(int64_t nv, int64_t no) : Nv(nv), No(no) {
    n1 = Nv * No;
    n2 = Nv * Nv * No * No;
    off2 = (n1 + 31) / 32 * 32;
    ntot = off2 + n2;
  }
};

int reduction_blocks(const Context &ctx, int64_t n);

// X = T2 + c T1 (x) T1 for nz systems of one shape stored one after another
void outer_add(Context &ctx, double *X, const double *T2, const double *T1,
               double c, int64_t Nv, int64_t No, int64_t nz = 1);
// sums: [0] dT.dT, [1] est.est, [2+q] dT.hist[q]; partials sized
// reduction_blocks(ntot) * (2 + nhist)
void jacobi_update(Context &ctx, const FockLayout &L, const double *R,
                   const double *T, double *est, double *dT,
                   const double *eps_h, const double *eps_p, double shift,
                   int nhist, const double *const *hist, double *partials,
                   double *sums);
// sums4: [0] T2.V [1] T1T1.V [2] T2.Vx [3] T1T1.Vx
void energy_terms(Context &ctx, const double *T1, const double *T2,
                  const double *V, const double *Vx, int64_t Nv, int64_t No,
                  double *partials, double *sums4);
void pair_energy(Context &ctx, const double *T1, const double *T2,
                 const double *V, const double *Vx, int64_t Nv, int64_t No,
                 double *out);
// hist_slot: host array of the nhist history slots (passed as kernel arguments)
void diis_solve(Context &ctx, double *B, int N, int k, int count,
                const double *sums, int nhist, const int *hist_slot,
                double *weights, double *lambda, int *status);
void diis_combine(Context &ctx, int count, const double *const *src,
                  const double *w, double *out, int64_t n, double *partials,
                  double *sum);
void linear_mix(Context &ctx, double *next, double *nres, double *last,
                double *lres, double ratio, int64_t n, double *partials,
                double *sums2);
void slice_add(Context &ctx, double *R, const double *Rxy, int64_t Nv,
               int64_t No, int64_t a0, int64_t b0, int64_t nx, int64_t ny,
               bool mirror, int64_t nz = 1);
void gather_slice(Context &ctx, double *dst, const double *src, int64_t G,
                  int64_t Nv, int64_t x0, int64_t nx, int64_t nz = 1);
// nz systems' blocks of n doubles: gather dst[z n + e] = src[z][e], scatter
// dst[z][e] = src[z n + e]; src_dev / dst_dev are device arrays of nz pointers
void batch_gather(Context &ctx, const double *const *src_dev, int64_t n, int64_t nz,
                  double *dst);
void batch_scatter(Context &ctx, const double *src, int64_t n, int64_t nz,
                   double *const *dst_dev);
void vertex_block(Context &ctx, double *dst, const double *src, int64_t G,
                  int64_t Np, int64_t p0, int64_t np, int64_t q0, int64_t nq);
void any_nonzero(Context &ctx, const double *p, int64_t n, int *flag_dev);

}  // namespace gbcc
