// placeholder, replaced by the emulated FP64 GEMM
#include "internal.hpp"
namespace gbcc {
void gemm_emu(Context &, bool, bool, int64_t, int64_t, int64_t, double,
              const double *, int64_t, const double *, int64_t, double,
              double *, int64_t, int64_t, int64_t, int64_t, int64_t) {
  throw Error(GBCC_BAD_ARG, "GBCC_PREC_EMU is not available in this build");
}
}  // namespace gbcc
