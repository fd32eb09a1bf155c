// gbdx_ode_f64_xo.cu -- FP64-state analytic-field kernels with the extended
// outputs SaveAt(steps=n) and SaveAt(dense=True) (own translation unit so the
// instantiations compile in parallel).
#include "gbdx_ode_impl.cuh"

namespace gbdx {
OdeEntry find_ode_entry_f64_xo(int solver, int field, int dim) {
  return find_ode_entry_t<double, true>(solver, field, dim);
}
}  // namespace gbdx
