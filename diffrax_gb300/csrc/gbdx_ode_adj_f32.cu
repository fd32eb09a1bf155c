// gbdx_ode_adj_f32.cu -- analytic-field adjoints, FP32 state (FP64 t/dt).
#include "gbdx_ode_adj_impl.cuh"

namespace gbdx {
AdjEntry find_ode_adj_entry_f32(int solver, int field, int dim, bool sde) {
  return find_ode_adj_entry_t<float>(solver, field, dim, sde);
}
cudaError_t launch_reduce_arg_rows_f32(const void *rows, int64_t batch, int n_args, void *out,
                                       cudaStream_t s) {
  return launch_reduce_arg_rows_t<float>(rows, batch, n_args, out, s);
}
}  // namespace gbdx
