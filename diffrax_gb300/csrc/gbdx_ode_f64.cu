// gbdx_ode_f64.cu -- FP64-state instantiations of the analytic-field kernels.
#include "gbdx_ode_impl.cuh"

namespace gbdx {
OdeEntry find_ode_entry_f64(int solver, int field, int dim) {
  return find_ode_entry_t<double, false>(solver, field, dim);
}
}  // namespace gbdx
