// gbdx_mlp_d64h256.cu -- MLP-field integrator instantiations for state dim 64,
// hidden width 256.
#include "gbdx_mlp_impl.cuh"

namespace gbdx {
OdeEntry find_mlp_entry_d64h256(int solver, bool precise, bool sde) {
  return mlp_entry<64, 256, false, false>(solver, precise, sde);
}
}  // namespace gbdx
