// Split-precision GEMMs: placeholder until the tcgen05 kernels land.
#include "split.h"

namespace gi {
gi_status split_gemm_dipole(Ctx* c, const double*, int, double*, int, size_t, int) {
  c->err = "split precision not available in this build";
  return GI_ERR_ARG;
}
gi_status split_gemm_final(Ctx* c, const double*, int, int, const double*, int, int, double*, int) {
  c->err = "split precision not available in this build";
  return GI_ERR_ARG;
}
gi_status split_prepare(Ctx*) { return GI_OK; }
void split_invalidate(Ctx*) {}
void split_release(Ctx*) {}
}  // namespace gi
