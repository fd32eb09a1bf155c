// gbdx_ode_f32.cu -- FP32-state instantiations of the analytic-field kernels.
#include "gbdx_ode_impl.cuh"

namespace gbdx {
OdeEntry find_ode_entry_f32(int solver, int field, int dim) {
  return find_ode_entry_t<float, false>(solver, field, dim);
}
}  // namespace gbdx
