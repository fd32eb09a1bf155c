// gbdx_ode_adj_impl.cuh -- launchers of the analytic-field adjoints for one
// state dtype: the forward with the full gradient tape (K0/K1 on a Taped
// field), the RecursiveCheckpointAdjoint backward and the BacksolveAdjoint
// backward.  Included once per dtype translation unit.
#pragma once

#include "gbdx_launch.h"
#include "gbdx_ode_adj.cuh"
#include "gbdx_ode_impl.cuh"

namespace gbdx {

template <int SOLVER, class F, class T>
cudaError_t launch_ode_rc_bwd(const SolveParams &P, const AdjParams &Q, cudaStream_t s) {
  if (P.batch <= 0) return cudaSuccess;
  ode_rc_bwd_kernel<SOLVER, F, T><<<unsigned((P.batch + 127) / 128), 128, 0, s>>>(P, Q);
  return cudaGetLastError();
}

template <int SOLVER, class F, class T>
cudaError_t launch_ode_bs(const SolveParams &P, const AdjParams &Q, cudaStream_t s) {
  if (P.batch <= 0) return cudaSuccess;
  ode_bs_kernel<SOLVER, F, T><<<unsigned((P.batch + 127) / 128), 128, 0, s>>>(P, Q);
  return cudaGetLastError();
}

template <int SOLVER, class F, class T>
AdjEntry adj_entry() {
  AdjEntry e;
  e.fwd = OdeEntry{&launch_ode<SOLVER, Taped<F>, T, false>,
                   &occupancy_ode<SOLVER, Taped<F>, T, false>};
  e.rc_bwd = &launch_ode_rc_bwd<SOLVER, F, T>;
  if constexpr (F::SDE)
    e.bs_bwd = nullptr;  // BacksolveAdjoint is offered for ODEs
  else
    e.bs_bwd = &launch_ode_bs<SOLVER, F, T>;
  e.n_args = F::NARGS;
  return e;
}

// Euler, Heun, Dopri5 and Tsit5 on Lotka-Volterra, Van der Pol and the
// Ornstein-Uhlenbeck drift (dim 1, 2, 4); with sde, the Ornstein-Uhlenbeck
// SDE (dim 2, 4; FP32 state) with Euler or Heun.
template <class T>
AdjEntry find_ode_adj_entry_t(int solver, int field, int dim, bool sde) {
#define GBDX_ADJ_SOLVERS(F)                                          \
  switch (solver) {                                                  \
    case GBDX_EULER: return adj_entry<GBDX_EULER, F, T>();           \
    case GBDX_HEUN: return adj_entry<GBDX_HEUN, F, T>();             \
    case GBDX_DOPRI5: return adj_entry<GBDX_DOPRI5, F, T>();         \
    case GBDX_TSIT5: return adj_entry<GBDX_TSIT5, F, T>();           \
    default: break;                                                  \
  }
  if (sde) {
    if constexpr (sizeof(T) == 4) {
      using S2 = OrnsteinUhlenbeckSDE<float, 2>;
      using S4 = OrnsteinUhlenbeckSDE<float, 4>;
      if (field == GBDX_ORNSTEIN_UHLENBECK && (solver == GBDX_EULER || solver == GBDX_HEUN)) {
        if (dim == 2) return solver == GBDX_EULER ? adj_entry<GBDX_EULER, S2, T>()
                                                  : adj_entry<GBDX_HEUN, S2, T>();
        if (dim == 4) return solver == GBDX_EULER ? adj_entry<GBDX_EULER, S4, T>()
                                                  : adj_entry<GBDX_HEUN, S4, T>();
      }
    }
    return AdjEntry{};
  }
  if (field == GBDX_LOTKA_VOLTERRA && dim == 2) { GBDX_ADJ_SOLVERS(LotkaVolterra<T>) }
  if (field == GBDX_VAN_DER_POL && dim == 2) { GBDX_ADJ_SOLVERS(VanDerPol<T>) }
  if (field == GBDX_ORNSTEIN_UHLENBECK) {
    using OU1 = OrnsteinUhlenbeck<T, 1>;
    using OU2 = OrnsteinUhlenbeck<T, 2>;
    using OU4 = OrnsteinUhlenbeck<T, 4>;
    if (dim == 1) { GBDX_ADJ_SOLVERS(OU1) }
    if (dim == 2) { GBDX_ADJ_SOLVERS(OU2) }
    if (dim == 4) { GBDX_ADJ_SOLVERS(OU4) }
  }
#undef GBDX_ADJ_SOLVERS
  return AdjEntry{};
}

// out[p] = sum over the batch of rows[b][p] (compensated), one warp per
// argument.
template <class T>
__global__ void reduce_arg_rows_kernel(const T *rows, int64_t batch, int n_args, T *out) {
  const int p = blockIdx.x;
  T s = T(0), c = T(0);
  for (int64_t b = threadIdx.x; b < batch; b += blockDim.x)
    kahan_add_t(s, c, rows[b * n_args + p]);
  s -= c;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (threadIdx.x == 0) out[p] = s;
}

template <class T>
cudaError_t launch_reduce_arg_rows_t(const void *rows, int64_t batch, int n_args, void *out,
                                     cudaStream_t s) {
  if (n_args <= 0) return cudaSuccess;
  reduce_arg_rows_kernel<T><<<unsigned(n_args), 32, 0, s>>>(static_cast<const T *>(rows), batch,
                                                            n_args, static_cast<T *>(out));
  return cudaGetLastError();
}

}  // namespace gbdx
