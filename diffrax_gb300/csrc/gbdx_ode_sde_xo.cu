// gbdx_ode_sde_xo.cu -- the Ornstein-Uhlenbeck SDE with the extended outputs
// (SaveAt(steps=n), SaveAt(dense=True), ClipStepSizeController, events), on
// the W-only and the space-time Levy area trees (own translation unit so the
// instantiations compile in parallel).
#include "gbdx_ode_impl.cuh"

namespace gbdx {
OdeEntry find_ode_sde_entry_f32_xo(int solver, int dim) {
  return find_ode_sde_entry_t<false, true>(solver, dim);
}
OdeEntry find_ode_sde_levy_entry_f32_xo(int solver, int dim) {
  return find_ode_sde_entry_t<true, true>(solver, dim);
}
}  // namespace gbdx
