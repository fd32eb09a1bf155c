// gbdx_mlp_d32h64.cu -- MLP-field integrator instantiations for state dim 32,
// hidden width 64.
#include "gbdx_mlp_impl.cuh"

namespace gbdx {
OdeEntry find_mlp_entry_d32h64(int solver, bool precise, bool sde) {
  return mlp_entry<32, 64, true, false>(solver, precise, sde);
}
}  // namespace gbdx
