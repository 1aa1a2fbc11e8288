// Lockstep CCSD over several closed-shell systems of one shape.
#pragma once

#include <map>
#include <memory>
#include <utility>
#include <vector>

#include "ccsd.hpp"

namespace gbcc {

// Systems with the same No, Nv and NG (each with its own vertex,
// eigenenergies and starting amplitudes) iterate together: one residual
// program evaluates every system's residual, with each contraction one
// batched product over the systems (one grouped tensor-core launch in
// precision mode, one batched FP64 GEMM otherwise).  The update, the DIIS
// mixer and the energy sums stay per system, on each system's own solver
// (ClusterSinglesDoublesAlgorithm.cxx:89-113 for each).  A system that
// converges or fails is frozen at that iteration while the others go on, so
// its result is the one it reaches alone, up to the rounding of the batched
// products; the stacked inputs then shrink to the systems still running, so
// that a stopped system costs nothing.  Steady-state iterations replay
// captured CUDA graphs, one per DIIS ring position and set of running
// systems.
class BatchCcsd {
 public:
  BatchCcsd(Context &ctx, std::vector<std::unique_ptr<Ccsd>> systems);
  ~BatchCcsd();
  BatchCcsd(const BatchCcsd &) = delete;
  BatchCcsd &operator=(const BatchCcsd &) = delete;
  // runs up to n more iterations of every system still running
  void run(int n);
  int size() const { return (int)sys_.size(); }
  Ccsd &system(int z) { return *sys_[z]; }
  // GBCC_OK while running or converged, else the error that stopped it
  gbcc_status status(int z) const { return st_[z]; }
  bool running(int z) const { return active_[z] != 0; }
  int64_t slice_size() const { return slice_; }

 private:
  Context &ctx_;
  std::vector<std::unique_ptr<Ccsd>> sys_;
  std::vector<gbcc_status> st_;
  std::vector<char> active_;
  gbcc_ccsd_opts o_;
  FockLayout L_;
  int64_t nz_ = 0, slice_ = 0;
  int it_ = 0;
  CcsdInputs in_;              // residual inputs with the trailing system index
  DBuf T1b_, T2b_, R1b_, R2b_;
  DBuf ptrs_;                  // device pointers: T1, T2, R1, R2 of each running system
  std::vector<int> run_;       // the running systems, in stacked order
  void upload_pointers();
  void compact(uint64_t mask);
  struct Graph {
    cudaGraphExec_t exec = nullptr;
    uint64_t launches = 0;
    double flops = 0;
  };
  std::map<std::pair<int, uint64_t>, Graph> graphs_;
  void body();
};

}  // namespace gbcc
