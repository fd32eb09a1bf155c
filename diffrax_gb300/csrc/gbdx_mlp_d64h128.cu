// gbdx_mlp_d64h128.cu -- MLP-field integrator instantiations for state dim 64,
// hidden width 128.
#include "gbdx_mlp_impl.cuh"

namespace gbdx {
OdeEntry find_mlp_entry_d64h128(int solver, bool precise, bool sde) {
  return mlp_entry<64, 128, false, false>(solver, precise, sde);
}
}  // namespace gbdx
