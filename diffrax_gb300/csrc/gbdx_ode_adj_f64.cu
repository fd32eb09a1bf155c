// gbdx_ode_adj_f64.cu -- analytic-field adjoints, FP64 state: the parity mode,
// compiled without FMA contraction like the other FP64 kernels.
#include "gbdx_ode_adj_impl.cuh"

namespace gbdx {
AdjEntry find_ode_adj_entry_f64(int solver, int field, int dim) {
  return find_ode_adj_entry_t<double>(solver, field, dim, false);
}
cudaError_t launch_reduce_arg_rows_f64(const void *rows, int64_t batch, int n_args, void *out,
                                       cudaStream_t s) {
  return launch_reduce_arg_rows_t<double>(rows, batch, n_args, out, s);
}
}  // namespace gbdx
