// gbdx_ode_sde.cu -- the Ornstein-Uhlenbeck SDE on the analytic-field kernels
// (own translation unit so the instantiations compile in parallel).
#include "gbdx_ode_impl.cuh"

namespace gbdx {
OdeEntry find_ode_sde_entry_f32(int solver, int dim) {
  return find_ode_sde_entry_t<false>(solver, dim);
}
}  // namespace gbdx
