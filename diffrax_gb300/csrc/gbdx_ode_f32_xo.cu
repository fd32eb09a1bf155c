// gbdx_ode_f32_xo.cu -- FP32-state analytic-field kernels with the extended
// outputs SaveAt(steps=n) and SaveAt(dense=True) (own translation unit so the
// instantiations compile in parallel).
#include "gbdx_ode_impl.cuh"

namespace gbdx {
OdeEntry find_ode_entry_f32_xo(int solver, int field, int dim) {
  return find_ode_entry_t<float, true>(solver, field, dim);
}
}  // namespace gbdx
