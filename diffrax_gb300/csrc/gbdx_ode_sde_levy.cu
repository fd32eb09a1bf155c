// gbdx_ode_sde_levy.cu -- the Ornstein-Uhlenbeck SDE driven by the virtual
// Brownian tree with space-time Levy area, and ShARK (own translation unit so
// the instantiations compile in parallel).
#include "gbdx_ode_impl.cuh"

namespace gbdx {
OdeEntry find_ode_sde_levy_entry_f32(int solver, int dim) {
  return find_ode_sde_entry_t<true>(solver, dim);
}
}  // namespace gbdx
