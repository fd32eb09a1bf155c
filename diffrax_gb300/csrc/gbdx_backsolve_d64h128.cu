// gbdx_backsolve_d64h128.cu -- BacksolveAdjoint backward instantiations for
// state dim 64, hidden width 128.
#include <initializer_list>

#include "gbdx_backsolve_impl.cuh"

namespace gbdx {
BsEntry find_backsolve_entry_d64h128(int solver, bool precise) {
  if (precise) return backsolve_entry<64, 128, true, GBDX_TSIT5>(solver);
  return backsolve_entry<64, 128, false, GBDX_TSIT5>(solver);
}
}  // namespace gbdx
