// Mixed-precision (tcgen05) path of the SBE right-hand side.
#include "sbe_ctx.cuh"

namespace sbe {

void mixed_free(SbeCtx* c) { (void)c; }

int rhs_mixed(SbeCtx* c, const double2* P, const double2* C, const double2* D, double2* dP,
              double2* dC, double2* dD, cudaStream_t s) {
  (void)c; (void)P; (void)C; (void)D; (void)dP; (void)dC; (void)dD; (void)s;
  return fail(SBE_ERR_UNSUPPORTED, "mixed precision path not built");
}

int rk4_mixed(SbeCtx* c, double2* P, double2* C, double2* D, const double2* Ek0,
              const double2* dEk, double dt, double2* src, cudaStream_t s) {
  (void)c; (void)P; (void)C; (void)D; (void)Ek0; (void)dEk; (void)dt; (void)src; (void)s;
  return fail(SBE_ERR_UNSUPPORTED, "mixed precision path not built");
}

}  // namespace sbe
