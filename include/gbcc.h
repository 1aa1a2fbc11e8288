/*
 * gbcc.h -- C ABI of the GB300 closed-shell CCSD(T) library (libgbcc.so).
 *
 * Plain pointers and sizes only.  Every tensor crossing this boundary is a
 * float64 buffer in the reference's dense layout: first index fastest
 * (column-major), index order as in the reference's CTF index strings, e.g.
 * T2[a,b,i,j] at a + Nv*(b + Nv*(i + No*j)).  The vertex is Gamma[G,p,q] with
 * the No holes first, then the Nv particles (Np = No + Nv).
 *
 * No function throws.  Each returns a gbcc_status; gbcc_last_error() gives the
 * message of the last failure on that context.
 */
#ifndef GBCC_H
#define GBCC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GBCC_ABI_VERSION 1

typedef enum {
  GBCC_OK = 0,
  GBCC_NOT_CONVERGED = 1,    /* maxIterations reached; results are valid */
  GBCC_DIIS_SINGULAR = 2,    /* DIIS subspace matrix singular: an exact zero
                                pivot, where dsysv gives info != 0 */
  GBCC_DIVERGED = 3,         /* NaN/Inf in the energy, the amplitude norms, or
                                the DIIS overlaps and weights (overflow) */
  GBCC_OOM = 4,              /* device allocation failed / over HBM budget */
  GBCC_BAD_ARG = 5,
  GBCC_CUDA_ERROR = 6,
  GBCC_TIMEOUT = 7,          /* a bounded device wait gave up */
  GBCC_COMPLEX_UNSUPPORTED = 8, /* vertex has a non-zero imaginary part */
  GBCC_NO_DEVICE = 9
} gbcc_status;

/* arithmetic of the dense contractions */
typedef enum {
  GBCC_PREC_FP64 = 0,   /* every contraction in IEEE float64 */
  GBCC_PREC_EMU = 1     /* float64 emulated on the bf16 tensor cores (split
                           operands, exact fp32 partial sums, fp64 combine);
                           update, DIIS and energies stay float64 */
} gbcc_precision;

typedef struct gbcc_ctx gbcc_ctx;
typedef struct gbcc_solver gbcc_solver;

/* ---------------------------------------------------------------- context */
/* One context per host thread / stream.  `stream` is a cudaStream_t (NULL:
 * the context creates its own non-blocking stream). */
gbcc_status gbcc_ctx_create(int device, void *stream, gbcc_ctx **out);
void gbcc_ctx_destroy(gbcc_ctx *ctx);
const char *gbcc_last_error(const gbcc_ctx *ctx);
const char *gbcc_status_string(int status);
int gbcc_abi_version(void);
/* Largest number of bytes the library's device allocations (the device's
 * default stream-ordered memory pool) have held at once since the last reset;
 * reset != 0 restarts the count from the current use.  No counterpart in the
 * reference; it shows, e.g., that no Nv^4 tensor is ever allocated. */
gbcc_status gbcc_device_pool_high_water(int device, int reset, int64_t *bytes);
/* Number of kernels this context has launched so far (all entry points). */
uint64_t gbcc_ctx_kernel_launches(const gbcc_ctx *ctx);
/* Analytic FP64-equivalent flops issued to the contraction engine so far. */
double gbcc_ctx_flops(const gbcc_ctx *ctx);
void *gbcc_ctx_stream(const gbcc_ctx *ctx);
/* Precision-mode parameters of this context: bf16 digits per operand of the
 * emulated GEMM (4..8, default 6) and the smallest GEMM (in flops) that is
 * emulated; smaller ones run in FP64 (default 1e7). */
gbcc_status gbcc_ctx_set_emulation(gbcc_ctx *ctx, int emu_slices,
                                   double emu_min_flops);

/* (T) batching of this context: the hole triples run in batches whose
 * distinct permutation images (up to 6 per triple) share one grouped
 * tensor-core launch per W product and one epilogue launch, each image
 * holding an Nv^3 FP64 work array.  max_images bounds the images of a batch
 * (>= 6; 0, the default: a quarter of the free device memory, at most 8 GiB
 * and 192 images).  Energies do not depend on it.  No counterpart in the
 * reference, which evaluates one permutation of one triple at a time
 * (CcsdPerturbativeTriples.cxx:156-223). */
gbcc_status gbcc_ctx_set_triples_batch(gbcc_ctx *ctx, int max_images);
/* K-split policies of this context's GEMMs (see gbcc_ccsd_opts):
 * f64_blocks_per_sm >= 0, emu_max_ksplit in [1, 64].  No counterpart in the
 * reference. */
gbcc_status gbcc_ctx_set_splits(gbcc_ctx *ctx, int f64_blocks_per_sm, int emu_max_ksplit);
/* Precision mode: a solver's integrals and vertex blocks do not change
 * during the solve, so the digit panels split from them (one set per layout
 * the contractions use, at most 12 GiB per context) are kept and reused
 * (enable = 1, the default) instead of being permuted and split again in
 * every iteration.  Results are the same bits either way.  No counterpart in
 * the reference. */
gbcc_status gbcc_ctx_set_operand_cache(gbcc_ctx *ctx, int enable);

/* Replay of steady-state CCSD iterations as captured CUDA graphs (default on;
 * off runs every iteration eagerly).  Results are identical either way. */
gbcc_status gbcc_ctx_set_graphs(gbcc_ctx *ctx, int enable);
/* Timing of the tensor-core GEMM kernel: enable (1) / disable (0) CUDA-event
 * records around each of its launches on the context stream; stats returns
 * the accumulated device milliseconds, the launches, the bf16 tensor flops of
 * the emulation scheme (S(S+1)/2 products of 2MNK) and the FP64-equivalent
 * flops (2MNK), and resets the counters. */
gbcc_status gbcc_ctx_profile(gbcc_ctx *ctx, int enable);
gbcc_status gbcc_ctx_gemm_stats(gbcc_ctx *ctx, double *ms, int64_t *launches,
                                double *tc_flops, double *fp64_flops);
/* Fault injection for failure-path tests (new in this library: sisi4s has
 * none).  The next event of the chosen kind fails as if it had happened, then
 * injection switches itself off:
 *   GBCC_FAULT_DIIS_SINGULAR  the next DIIS mixing step reports a singular
 *                             matrix (the solve returns GBCC_DIIS_SINGULAR)
 *   GBCC_FAULT_NAN            the next CCSD iteration's norms read NaN
 *                             (GBCC_DIVERGED)
 *   GBCC_FAULT_OOM            the next device allocation fails (GBCC_OOM)
 *   GBCC_FAULT_DEVICE_WAIT    the next tensor-core GEMM launch first waits on
 *                             a barrier that nothing completes; the bounded
 *                             wait gives up in well under a second, every
 *                             other role of the kernel stops, and the call
 *                             returns GBCC_TIMEOUT with the context usable
 * No injected fault touches memory out of bounds or leaves a kernel hung. */
enum {
  GBCC_FAULT_NONE = 0,
  GBCC_FAULT_DIIS_SINGULAR = 1,
  GBCC_FAULT_NAN = 2,
  GBCC_FAULT_OOM = 3,
  GBCC_FAULT_DEVICE_WAIT = 4
};
gbcc_status gbcc_ctx_inject_fault(gbcc_ctx *ctx, int kind);

/* Per-launch records behind those statistics (new in this library; sisi4s
 * has per-step timers only): the M, N, K (3 values per launch, into mnk) and
 * device milliseconds (into ms) of up to cap profiled GEMM launches, oldest
 * first; *count receives the number written.  The records are cleared. */
gbcc_status gbcc_ctx_gemm_records(gbcc_ctx *ctx, int64_t *mnk, double *ms, int64_t cap,
                                  int64_t *count);

/* ------------------------------------------------------------- CCSD input */
/* Replaces ClusterSinglesDoublesAlgorithm::run<double> +
 * CcsdEnergyFromCoulombIntegrals::getResiduum (real path)
 * (src/algorithms/ClusterSinglesDoublesAlgorithm.cxx:38-128,
 *  src/algorithms/CcsdEnergyFromCoulombIntegrals.cxx:27-494).
 * Argument names and defaults are those of the reference's YAML keys
 * (ClusterSinglesDoublesAlgorithm.hpp:42-46, .cxx:48-63; LinearMixer.cxx:17;
 *  DiisMixer.cxx:55; CcsdEnergyFromCoulombIntegrals.cxx:123-124,324,375-384). */
typedef struct {
  int mixer;                     /* 0 = "LinearMixer" (default), 1 = "DiisMixer" */
  int max_residua;               /* maxResidua, default 4 */
  double mixing_ratio;           /* mixingRatio, default 1.0 */
  int max_iterations;            /* maxIterations, default 16 */
  double energy_convergence;     /* energyConvergence (relative), default 1e-6 */
  double amplitudes_convergence; /* amplitudesConvergence, default 1e-5 */
  double level_shift;            /* levelShift, default 0 */
  int distinguishable;           /* distinguishable, default 0 */
  int ppl;                       /* ppl, default 1 */
  int integrals_slice_size;      /* integralsSliceSize, default -1 (auto) */
  double integrals_slice_factor; /* integralsSliceFactor, < 0: not given */
  int precision;                 /* gbcc_precision, default GBCC_PREC_FP64 */
  int emu_slices;                /* bf16 slices per operand for GBCC_PREC_EMU
                                    (0 = library default); (T) uses one more,
                                    at most 8 */
  int formulation;               /* 0: CcsdEnergyFromCoulombIntegrals (particle
                                    ladder from the vertex, default);
                                    1: CcsdEnergyFromCoulombIntegralsReference
                                    (stored Vabcd / Vabci,
                                    CcsdEnergyFromCoulombIntegralsReference.cxx:29-292) */
  int only_ppl;                  /* onlyPPL of formulation 1, default 0 */
  /* Execution tuning (no counterpart in the reference; results do not
   * depend on them beyond rounding).  gbcc_ccsd_opts_default sets them to
   * "keep the context's setting"; a set value is applied to the context by
   * the call that takes these options. */
  double emu_min_flops;          /* > 0: smallest GEMM (flops) emulated on the
                                    tensor cores in precision mode; smaller
                                    ones run in FP64 (context default 1e7) */
  int f64_split_blocks;          /* FP64 GEMM K-split target in blocks per SM
                                    (0: no split; context default 3) */
  int emu_max_ksplit;            /* most K-splits of an emulated GEMM
                                    (1: none; context default 64) */
} gbcc_ccsd_opts;

void gbcc_ccsd_opts_default(gbcc_ccsd_opts *opts);

typedef struct {
  int No, Nv, NG;
  const double *eps_h;        /* HoleEigenEnergies [No] */
  const double *eps_p;        /* ParticleEigenEnergies [Nv] */
  const double *gamma;        /* CoulombVertex real part [NG,Np,Np] */
  const double *gamma_imag;   /* optional imaginary part; must be all zero */
  /* optional integrals; any NULL one is built on the device from gamma
   * exactly as CoulombIntegralsFromVertex does */
  const double *Vabij;        /* PPHHCoulombIntegrals [Nv,Nv,No,No] */
  const double *Vaibj;        /* PHPHCoulombIntegrals [Nv,No,Nv,No] */
  const double *Vijkl;        /* HHHHCoulombIntegrals [No,No,No,No] */
  const double *Vijka;        /* HHHPCoulombIntegrals [No,No,No,Nv] */
  const double *init_T1;      /* initialSinglesAmplitudes [Nv,No] or NULL */
  const double *init_T2;      /* initialDoublesAmplitudes [Nv,Nv,No,No] or NULL */
  const double *fock_hp;      /* HPFockMatrix f[i,a] [No,Nv] or NULL: adds the
                                 noncanonical term spins * T1_ai f_ia to every
                                 iteration's energy (getEnergy,
                                 ClusterSinglesDoublesAlgorithm.cxx:199-209).
                                 Callers zero-initialise the struct. */
  /* formulation 1 only; built from gamma when NULL (gamma may then be NULL
   * if every integral is given) */
  const double *Vabcd;        /* PPPPCoulombIntegrals [Nv,Nv,Nv,Nv] */
  const double *Vabci;        /* PPPHCoulombIntegrals [Nv,Nv,Nv,No] */
} gbcc_ccsd_in;

typedef struct {
  double energy;              /* CcsdEnergy */
  double direct, exchange;    /* last iteration's energy terms */
  int iterations;
  int converged;
  double *T1;                 /* optional caller buffer [Nv,No]  (CcsdSinglesAmplitudes) */
  double *T2;                 /* optional caller buffer [Nv,Nv,No,No] (CcsdDoublesAmplitudes) */
  double *pair_energy;        /* optional caller buffer [No,No] (PairEnergy) */
  double *energy_history;     /* optional [max_iterations]: energy of each iteration */
} gbcc_ccsd_out;

/* One-call solve from host buffers (uploads, builds integrals, iterates,
 * downloads).  Returns GBCC_NOT_CONVERGED when maxIterations was reached
 * (results still valid, as the reference only warns). */
gbcc_status gbcc_ccsd_solve(gbcc_ctx *ctx, const gbcc_ccsd_in *in,
                            const gbcc_ccsd_opts *opts, gbcc_ccsd_out *out);

/* Lockstep solve of nsys closed-shell systems of one shape: the same No, Nv
 * and NG, each with its own vertex, eigenenergies and optional starting
 * amplitudes (all or none of them starting from given doubles), one set of
 * options (DiisMixer, CcsdEnergyFromCoulombIntegrals, maxIterations >= 1).
 * Every contraction of the residual runs once for all systems, as one
 * batched product; each system keeps its own update, DIIS history and
 * convergence test, and stops where it would stop alone (its energies agree
 * with gbcc_ccsd_solve's up to the rounding of the batched products).
 * status[z] receives what gbcc_ccsd_solve would return for system z, and
 * outs[z] (if outs is not NULL) its results.  Returns GBCC_OK when the batch
 * ran, whatever the systems' statuses, else the error that stopped it.  No
 * counterpart in the reference, which solves one system per algorithm run
 * (ClusterSinglesDoublesAlgorithm.cxx:38-128). */
gbcc_status gbcc_ccsd_solve_batch(gbcc_ctx *ctx, int nsys, const gbcc_ccsd_in *ins,
                                  const gbcc_ccsd_opts *opts, gbcc_ccsd_out *outs,
                                  gbcc_status *status);

/* The same batch kept on the device (as gbcc_ccsd_setup / _step / _result do
 * for one system): setup uploads 1 to 64 systems of one shape; step runs up
 * to n more lockstep iterations and writes every system's status; result
 * reads system z back; triples runs (T) on system z's amplitudes
 * (gbcc_triples_from_solver for one member of the batch). */
typedef struct gbcc_batch gbcc_batch;
gbcc_status gbcc_ccsd_batch_setup(gbcc_ctx *ctx, int nsys, const gbcc_ccsd_in *ins,
                                  const gbcc_ccsd_opts *opts, gbcc_batch **out);
gbcc_status gbcc_ccsd_batch_step(gbcc_batch *b, int n, gbcc_status *status);
gbcc_status gbcc_ccsd_batch_result(gbcc_batch *b, int z, gbcc_ccsd_out *out);
gbcc_status gbcc_ccsd_batch_triples(gbcc_batch *b, int z, int precision, double *e_total,
                                    double *e_t);
void gbcc_ccsd_batch_destroy(gbcc_batch *b);

/* Device-resident solver: setup uploads inputs and builds integrals once;
 * step runs n more iterations (stopping early on convergence);
 * amplitudes can then be read back or handed to the (T) step. */
gbcc_status gbcc_ccsd_setup(gbcc_ctx *ctx, const gbcc_ccsd_in *in,
                            const gbcc_ccsd_opts *opts, gbcc_solver **out);
gbcc_status gbcc_ccsd_step(gbcc_solver *s, int n, double *energy,
                           int *converged);
gbcc_status gbcc_ccsd_result(gbcc_solver *s, gbcc_ccsd_out *out);
/* Device pointers of the current amplitudes (T1 then T2). */
gbcc_status gbcc_ccsd_device_amplitudes(gbcc_solver *s, const double **T1,
                                        const double **T2);
void gbcc_ccsd_destroy(gbcc_solver *s);
/* Returns the solver to its state after setup: the starting amplitudes given
 * at setup (else zero amplitudes, so the next iteration is the MP2 start),
 * no iterations done, an empty DIIS history.  The uploaded inputs, integrals,
 * buffers and captured iteration graphs are kept, so a repeated solve of the
 * same system pays none of the setup again.  No counterpart in the reference,
 * whose algorithms run once per step (ClusterSinglesDoublesAlgorithm.cxx:38-128
 * always starts from the data map's amplitudes). */
gbcc_status gbcc_ccsd_restart(gbcc_solver *s);

/* One residual evaluation R(T) for iteration index `it` (it == 0 without
 * initial doubles gives the MP2 start R2 = Vabij), for parity tests.
 * Host buffers in and out. */
gbcc_status gbcc_ccsd_residual(gbcc_ctx *ctx, const gbcc_ccsd_in *in,
                               const gbcc_ccsd_opts *opts, int it,
                               const double *T1, const double *T2,
                               double *R1, double *R2);

/* ------------------------------------------------------- complex CCSD */
/* The complex (k-point) branch of the same algorithm: ClusterSinglesDoubles
 * Algorithm::run<complex> (src/algorithms/ClusterSinglesDoublesAlgorithm.cxx:
 * 25-128) with CcsdEnergyFromCoulombIntegrals::getResiduum for complex
 * amplitudes (src/algorithms/CcsdEnergyFromCoulombIntegrals.cxx:496-891) and
 * the complex integrals of CoulombIntegralsFromVertex (:613-816).  Complex
 * tensors are interleaved (re, im) pairs in the reference's dense layout, as
 * CTF stores complex<double>.  Only the linear mixer exists for complex
 * amplitudes: the reference's complex DIIS solve is unimplemented
 * (src/mixers/DiisMixer.cxx:43-48), and DiisMixer gives GBCC_BAD_ARG. */
typedef struct {
  int No, Nv, NG;
  const double *eps_h;        /* HoleEigenEnergies [No] (real) */
  const double *eps_p;        /* ParticleEigenEnergies [Nv] (real) */
  const double *gamma;        /* CoulombVertex, complex [NG,Np,Np] */
  const double *init_T1;      /* initialSinglesAmplitudes, complex [Nv,No] or NULL */
  const double *init_T2;      /* initialDoublesAmplitudes, complex [Nv,Nv,No,No] or NULL */
  const double *fock_hp;      /* HPFockMatrix, complex [No,Nv] or NULL: adds the
                                 noncanonical spins * T1_ai f_ia (:199-209) */
} gbcc_ccsd_complex_in;

typedef struct {
  double energy[2];           /* (re, im); CcsdEnergy is the real part (:32) */
  double direct[2], exchange[2];
  int iterations;
  int converged;
  double *T1;                 /* optional caller buffer, complex [Nv,No] */
  double *T2;                 /* optional caller buffer, complex [Nv,Nv,No,No] */
  double *energy_history;     /* optional [2*max_iterations]: (re, im) per iteration */
  double *pair_energy;        /* optional caller buffer, complex [No,No] (PairEnergy) */
} gbcc_ccsd_complex_out;

gbcc_status gbcc_ccsd_solve_complex(gbcc_ctx *ctx, const gbcc_ccsd_complex_in *in,
                                    const gbcc_ccsd_opts *opts,
                                    gbcc_ccsd_complex_out *out);
/* One complex getResiduum call: R = residual(it, T), complex buffers. */
gbcc_status gbcc_ccsd_residual_complex(gbcc_ctx *ctx, const gbcc_ccsd_complex_in *in,
                                       const gbcc_ccsd_opts *opts, int it,
                                       const double *T1, const double *T2,
                                       double *R1, double *R2);

/* Replaces CcsdPerturbativeTriplesComplex::run with complex amplitudes
 * (src/algorithms/CcsdPerturbativeTriplesComplex.cxx:32-268).  e_total =
 * e_ccsd + Re E_(T) (CcsdPerturbativeTriplesComplexEnergy, :77-84); e_t =
 * E_(T) as (re, im).  The PPHH and PHHH integrals are built from gamma. */
typedef struct {
  int No, Nv, NG;
  const double *eps_h, *eps_p;  /* real [No], [Nv] */
  const double *gamma;          /* CoulombVertex, complex [NG,Np,Np] */
  const double *T1;             /* CcsdSinglesAmplitudes, complex [Nv,No] */
  const double *T2;             /* CcsdDoublesAmplitudes, complex [Nv,Nv,No,No] */
  double e_ccsd;                /* CcsdEnergy */
} gbcc_triples_complex_in;

gbcc_status gbcc_triples_complex(gbcc_ctx *ctx, const gbcc_triples_complex_in *in,
                                 int precision, double *e_total, double *e_t);

/* ---------------------------------------------------------------- (T) */
/* Replaces CcsdPerturbativeTriples::run (src/algorithms/CcsdPerturbativeTriples.cxx:119-248).
 * e_total = e_ccsd + E_(T) (the reference's CcsdPerturbativeTriplesEnergy),
 * e_t = E_(T) alone. Vabij / Vijka may be NULL (built from gamma). */
typedef struct {
  int No, Nv, NG;
  const double *eps_h, *eps_p, *gamma, *gamma_imag;
  const double *Vabij;   /* PPHHCoulombIntegrals */
  const double *Vijka;   /* HHHPCoulombIntegrals */
  const double *T1;      /* CcsdSinglesAmplitudes */
  const double *T2;      /* CcsdDoublesAmplitudes */
  double e_ccsd;         /* CcsdEnergy */
} gbcc_triples_in;

gbcc_status gbcc_triples(gbcc_ctx *ctx, const gbcc_triples_in *in,
                         int precision, double *e_total, double *e_t);
/* (T) from a device-resident CCSD solver (no amplitude round trip). */
gbcc_status gbcc_triples_from_solver(gbcc_solver *s, int precision,
                                     double *e_total, double *e_t);

/* --------------------------------------------------------------- serving */
/* Continuous admission of many CCSD(T) solves of uneven size on one device
 * (no counterpart in the reference, which runs one solve per process).
 * `slots` workers each own a host thread and a CUDA stream; requests are
 * admitted first-in first-out when a worker is free and their estimated device
 * footprint fits in the remaining `hbm_budget_bytes`, so requests that arrive
 * while others run start as slots and memory free up and their kernels run
 * concurrently.  Results are bit-identical to a solve of the same request
 * alone (every kernel is deterministic). */
typedef struct {
  int device;
  int slots;                 /* concurrent solves, default 8 */
  int64_t hbm_budget_bytes;  /* 0: 80 % of the free device memory */
  int max_batch;             /* > 1: a slot that admits a request of a small
                                shape (one whose particle-ladder block leaves
                                most SMs idle) also takes up to max_batch - 1
                                queued requests of the same shape, options and
                                (T) flag, and solves them in lockstep
                                (gbcc_ccsd_batch_*); default 8 */
} gbcc_server_opts;

typedef struct {
  int64_t id;
  int status;                /* gbcc_status of the solve */
  double e_ccsd, e_t, e_total;
  int iterations, converged;
  double t_submit, t_admit, t_start, t_done;  /* seconds, monotonic clock */
} gbcc_result;

typedef struct gbcc_server gbcc_server;
void gbcc_server_opts_default(gbcc_server_opts *opts);
gbcc_status gbcc_server_create(const gbcc_server_opts *opts, gbcc_server **out);
/* Copies the host inputs (vertex and eigenvalues only; the integrals are
 * built on the device) and queues the solve; `triples` adds (T). */
gbcc_status gbcc_server_submit(gbcc_server *s, const gbcc_ccsd_in *in,
                               const gbcc_ccsd_opts *opts, int triples,
                               int64_t *id);
gbcc_status gbcc_server_poll(gbcc_server *s, int64_t id, gbcc_result *res,
                             int *done);
gbcc_status gbcc_server_wait(gbcc_server *s, int64_t id, gbcc_result *res);
gbcc_status gbcc_server_stats(gbcc_server *s, int *pending, int *running,
                              int64_t *bytes_in_use);
/* Finishes every queued request, then stops the workers. */
void gbcc_server_destroy(gbcc_server *s);

/* ------------------------------------------------------ Coulomb integrals */
/* Replaces CoulombIntegralsFromVertex::calculateRealIntegrals for the blocks
 * the CCSD/(T) steps read (src/algorithms/CoulombIntegralsFromVertex.cxx:395-491).
 * Any NULL output is skipped.  Host buffers. */
gbcc_status gbcc_coulomb_integrals(gbcc_ctx *ctx, int No, int Nv, int NG,
                                   const double *gamma, double *Vabij,
                                   double *Vaibj, double *Vijkl, double *Vijka,
                                   double *Vijab);
/* The particle blocks the stored formulation reads
 * (CoulombIntegralsFromVertex.cxx:423-431): PPPP Vabcd [Nv,Nv,Nv,Nv] and
 * PPPH Vabci [Nv,Nv,Nv,No].  Any NULL output is skipped. */
gbcc_status gbcc_coulomb_integrals_pp(gbcc_ctx *ctx, int No, int Nv, int NG,
                                      const double *gamma, double *Vabcd, double *Vabci);
/* CoulombIntegralsFromVertex::calculateComplexIntegrals for the blocks the
 * complex CCSD / (T) read (CoulombIntegralsFromVertex.cxx:767-809): complex
 * gamma and outputs, interleaved (re, im).  Any NULL output is skipped. */
gbcc_status gbcc_coulomb_integrals_complex(gbcc_ctx *ctx, int No, int Nv, int NG,
                                           const double *gamma, double *Vabij,
                                           double *Vaijb, double *Vijab, double *Vaibj,
                                           double *Vijkl, double *Vijka, double *Vaijk);

/* ------------------------------------------------------- building blocks */
/* C[M,N] = alpha * op(A) op(B) + beta * C, column-major, device pointers,
 * stream-ordered on the context stream.  trans: 0 = N, 1 = T. */
gbcc_status gbcc_dgemm(gbcc_ctx *ctx, int transA, int transB, int64_t M,
                       int64_t N, int64_t K, double alpha, const double *A,
                       int64_t lda, const double *B, int64_t ldb, double beta,
                       double *C, int64_t ldc, int precision);

/* The emulated (GBCC_PREC_EMU) GEMM of gbcc_dgemm for callers that cannot let
 * the library allocate device memory, e.g. a serving process whose arena
 * already holds the whole HBM budget, or a host loop that must not enter the
 * CUDA allocator.  It has no counterpart in the reference.  Its scratch (digit
 * panels of both operands, exponents, error word) lives in one fixed 32 MiB
 * device array, which every GPU that runs the library's kernels holds until
 * the process exits (with CUDA's lazy module loading, from the first use on
 * that GPU); a GEMM whose scratch would exceed it (S digits x 2 bytes x
 * (M padded to 128 + N padded to 64) x K padded to 32, plus 4 bytes per row
 * and column) is rejected with GBCC_BAD_ARG.  Nothing is allocated or freed.
 * All calls on a device share the array, so calls whose work overlaps on the
 * GPU race; order them.  Each call waits for its GEMM to finish (it reads the
 * kernel's error word back) before it returns.  The first call on a device
 * looks up the array's device address and keeps it for the life of the
 * process; do not call this entry point on a device after resetting it
 * (cudaDeviceReset).  Device pointers, context stream, digits from
 * gbcc_ctx_set_emulation. */
gbcc_status gbcc_dgemm_emu_noalloc(gbcc_ctx *ctx, int transA, int transB,
                                   int64_t M, int64_t N, int64_t K,
                                   double alpha, const double *A, int64_t lda,
                                   const double *B, int64_t ldb, double beta,
                                   double *C, int64_t ldc);

/* CCSD energy terms (direct, exchange) of device amplitudes, as
 * ClusterSinglesDoublesAlgorithm::getEnergy (.cxx:131-197). Device pointers. */
gbcc_status gbcc_energy(gbcc_ctx *ctx, int No, int Nv, const double *T1,
                        const double *T2, const double *Vabij, double *direct,
                        double *exchange);

#ifdef __cplusplus
}
#endif
#endif /* GBCC_H */
