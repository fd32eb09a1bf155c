// gbdx_backsolve_d64h256.cu -- BacksolveAdjoint backward instantiations for
// state dim 64, hidden width 256.
#include <initializer_list>

#include "gbdx_backsolve_impl.cuh"

namespace gbdx {
BsEntry find_backsolve_entry_d64h256(int solver, bool precise) {
  if (precise) return backsolve_entry<64, 256, true, GBDX_TSIT5>(solver);
  return backsolve_entry<64, 256, false, GBDX_TSIT5, GBDX_DOPRI5>(solver);
}
}  // namespace gbdx
