// gbdx_mlp_xo_d64h256.cu -- extended-output MLP-field integrator instantiations
// (SaveAt(steps=n), SaveAt(dense=True), the clip controller, events) for state
// dim 64, hidden width 256.
#include "gbdx_mlp_impl.cuh"

namespace gbdx {
OdeEntry find_mlp_xo_entry_d64h256(int solver, bool precise, bool sde) {
  return mlp_entry<64, 256, false, true>(solver, precise, sde);
}
}  // namespace gbdx
