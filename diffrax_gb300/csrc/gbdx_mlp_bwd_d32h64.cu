// gbdx_mlp_bwd_d32h64.cu -- MLP-field backward instantiations for state dim 32,
// hidden width 64.
#include "gbdx_mlp_bwd_impl.cuh"

namespace gbdx {
BwdEntry find_mlp_bwd_entry_d32h64(int solver, bool precise, bool sde) {
  return mlp_bwd_entry<32, 64, true>(solver, precise, sde);
}
}  // namespace gbdx
