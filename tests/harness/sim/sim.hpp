// Host simulation of the device side of libgbcc, for tests on machines
// without a GPU.  The library's host code (C ABI, CCSD driver, contraction
// engine, complex and stored programs, serving) is compiled unchanged and
// linked against
//   - sim_runtime.cpp: the CUDA runtime calls it makes, with "device" memory
//     in host memory and CUDA stream capture emulated (work submitted to a
//     capturing stream is recorded and runs at every launch of the graph);
//   - sim_kernels.cpp: host models of the kernel launchers, each following
//     the arithmetic of its kernel in FP64 (the emulated GEMMs are modelled
//     by plain FP64 products).
// Test infrastructure only: nothing in the library loads it.
#pragma once

#include <cuda_runtime.h>

#include <functional>

namespace sim {

using Op = std::function<void()>;

// Run op on stream s now, or record it if s is being captured.
void submit(cudaStream_t s, Op op);
bool capturing(cudaStream_t s);

}  // namespace sim
