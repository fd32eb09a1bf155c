// gbdx_backsolve_d32h64.cu -- BacksolveAdjoint backward instantiations for
// state dim 32, hidden width 64.
#include <initializer_list>

#include "gbdx_backsolve_impl.cuh"

namespace gbdx {
BsEntry find_backsolve_entry_d32h64(int solver, bool precise) {
  if (precise)
    return backsolve_entry<32, 64, true, GBDX_EULER, GBDX_HEUN, GBDX_DOPRI5, GBDX_TSIT5>(solver);
  return backsolve_entry<32, 64, false, GBDX_EULER, GBDX_HEUN, GBDX_DOPRI5, GBDX_TSIT5>(solver);
}
}  // namespace gbdx
