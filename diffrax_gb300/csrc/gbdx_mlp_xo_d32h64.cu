// gbdx_mlp_xo_d32h64.cu -- extended-output MLP-field integrator instantiations
// (SaveAt(steps=n), SaveAt(dense=True), the clip controller, events) for state
// dim 32, hidden width 64.
#include "gbdx_mlp_impl.cuh"

namespace gbdx {
OdeEntry find_mlp_xo_entry_d32h64(int solver, bool precise, bool sde) {
  return mlp_entry<32, 64, true, true>(solver, precise, sde);
}
}  // namespace gbdx
