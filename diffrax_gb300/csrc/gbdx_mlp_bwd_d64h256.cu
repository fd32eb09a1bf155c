// gbdx_mlp_bwd_d64h256.cu -- MLP-field backward instantiations for state dim 64,
// hidden width 256.
#include "gbdx_mlp_bwd_impl.cuh"

namespace gbdx {
BwdEntry find_mlp_bwd_entry_d64h256(int solver, bool precise, bool sde) {
  return mlp_bwd_entry<64, 256, false>(solver, precise, sde);
}
}  // namespace gbdx
