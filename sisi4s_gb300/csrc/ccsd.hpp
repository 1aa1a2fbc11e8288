// Device-resident closed-shell CCSD solver.
#pragma once

#include <memory>
#include <vector>

#include "ccsd_kernels.hpp"

namespace gbcc {

struct CcsdInputs {
  Context *ctx = nullptr;     // the integrals and vertex blocks are registered
                              // as constants of this context while alive
  ~CcsdInputs();
  int64_t No = 0, Nv = 0, NG = 0;
  OTen eps_h, eps_p;          // [No], [Nv]
  OTen Gai, Gab, Gij;         // [NG,Nv,No], [NG,Nv,Nv], [NG,No,No]
  OTen Vabij, Vx, Vaibj, Vijkl, Vijka;  // Vx[a,b,i,j] = Vabij[b,a,i,j]
  OTen fock_ai;               // HPFockMatrix as f[a,i] [Nv,No], if given
  OTen Vabcd, Vabci;          // stored formulation: [Nv,Nv,Nv,Nv], [Nv,Nv,Nv,No]
};

// Upload eps and Gamma, slice the vertex blocks, upload or build the
// integrals (CoulombIntegralsFromVertex.cxx:395-417).
std::unique_ptr<CcsdInputs> upload_inputs(Context &ctx, const gbcc_ccsd_in &in,
                                          int precision, bool need_vaibj,
                                          bool stored = false);

// One residual evaluation over nz systems of one shape (residual_program).
// With nz > 1 the input tensors, T1, T2, R1 and R2 carry a trailing system
// index (each system's block contiguous); R1 and R2 arrive zeroed.
struct ResidualArgs {
  const CcsdInputs *I = nullptr;
  const gbcc_ccsd_opts *o = nullptr;
  int64_t nz = 1;
  int64_t slice = 0;          // integralsSliceSize of the particle ladder
  bool init_doubles = false;  // initial doubles given: no MP2 start at it 0
  Ten T1, T2, R1, R2;
};
void residual_program(Context &ctx, const ResidualArgs &a, int it);

struct IterInfo {
  double energy = 0, direct = 0, exchange = 0, noncanonical = 0, dtdt = 0, tt = 0,
         lambda = 0;
  int diis_status = 0;
};

class Ccsd {
 public:
  Ccsd(Context &ctx, std::unique_ptr<CcsdInputs> in, const gbcc_ccsd_opts &o,
       const double *init_T1_host, const double *init_T2_host);
  ~Ccsd();
  Ccsd(const Ccsd &) = delete;
  Ccsd &operator=(const Ccsd &) = delete;
  // R = residual(it, T) into R_ (parity entry point uses it directly)
  void residual(int it, const double *T, double *R);
  // one full iteration; returns the host-side info
  IterInfo iterate();
  // the parts of an iteration, for a driver that evaluates the residuals of
  // several solvers at once: the graph key of the next iteration (allocating
  // its DIIS slot), the device work after the residual (which must be in
  // residual_buffer()), the host state after it, and the convergence test
  // (true: the solve stops, with an error in st or converged)
  int graph_key();
  void mix_body();
  IterInfo finish_iteration();
  bool absorb(IterInfo info, gbcc_status &st);
  double *residual_buffer() { return R_.as<double>(); }
  double *amplitude_buffer() { return T_.as<double>(); }
  bool has_initial_doubles() const { return init_doubles_; }
  const gbcc_ccsd_opts &options() const { return o_; }
  // runs up to n iterations; returns status
  gbcc_status run(int n, double *energy, int *converged);
  const double *amplitudes() const { return T_.as<double>(); }
  const FockLayout &layout() const { return L_; }
  CcsdInputs &inputs() { return *in_; }
  Context &ctx() { return ctx_; }
  int iterations_done() const { return it_; }
  bool converged() const { return converged_; }
  double energy() const { return e_; }
  double direct() const { return dir_; }
  double exchange() const { return exc_; }
  const std::vector<double> &history() const { return hist_; }
  void pair_energies(double *dev_out);
  int64_t slice_size() const { return slice_; }
  // energy of the current amplitudes without iterating (maxIterations 0)
  void evaluate_energy();
  // back to the state after construction (the given starting amplitudes, or
  // zero amplitudes and the MP2 start), keeping the resident integrals, the
  // buffers and the captured iteration graphs
  void restart();

 private:
  Context &ctx_;
  std::unique_ptr<CcsdInputs> in_;
  gbcc_ccsd_opts o_;
  FockLayout L_;
  bool init_doubles_ = false;
  int64_t slice_ = 0;
  DBuf T_, R_;                 // current amplitudes, residual
  DBuf T0_;                    // given starting amplitudes (restart), if any
  DBuf E_, D_, Lres_;          // linear mixer: estimate, change, last change
  std::vector<DBuf> slotA_, slotD_;  // DIIS history
  DBuf B_, w_, scal_, partials_, hist_slot_;
  int next_ = 0, count_ = 0;
  bool have_last_ = false;
  int it_ = 0;
  bool converged_ = false;
  double e_ = 0, prev_ = 0, dir_ = 0, exc_ = 0;
  std::vector<double> hist_;
  double *pinned_ = nullptr;
  // steady-state iterations replayed as CUDA graphs, one per starting state
  // (DIIS ring position, or linear-mixer buffer parity)
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    uint64_t launches = 0;
    double flops = 0;
  };
  std::vector<Graph> graphs_;
  uint64_t swaps_ = 0;
  void iteration_body();
  void residual_stored(int it, const double *T, double *R);
  void energy_sums(const double *amp);
  void energy_from_sums(const double *h, IterInfo &info) const;
};

}  // namespace gbcc
