// gbdx_ode_impl.cuh -- launchers of the analytic-field kernels (K0 plain,
// K1 fused) for one state dtype.  Included once per dtype translation unit so
// the instantiations compile in parallel.
#pragma once

#include "gbdx_launch.h"
#include "gbdx_traj.cuh"

namespace gbdx {

// XO selects the extended-output kernels (SaveAt(steps=n), SaveAt(dense=True)).
template <int SOLVER, class FIELD, class T, bool XO>
cudaError_t launch_ode(const SolveParams &P, const LaunchCfg &cfg, cudaStream_t s) {
  if (P.batch <= 0) return cudaSuccess;
  if (cfg.kernel == GBDX_KERNEL_PLAIN) {
    const int64_t blocks = (P.batch + 127) / 128;
    plain_kernel<SOLVER, FIELD, T, XO><<<(unsigned)blocks, 128, 0, s>>>(P);
  } else {
    fused_kernel<SOLVER, FIELD, T, XO><<<cfg.grid, cfg.block, 0, s>>>(P);
  }
  return cudaGetLastError();
}

template <int SOLVER, class FIELD, class T, bool XO>
cudaError_t occupancy_ode(int block, int *ctas_per_sm) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(
      ctas_per_sm, fused_kernel<SOLVER, FIELD, T, XO>, block, 0);
}

template <class T, bool XO>
OdeEntry find_ode_entry_t(int solver, int field, int dim) {
#define GBDX_ENTRY(S, F) \
  OdeEntry { &launch_ode<S, F, T, XO>, &occupancy_ode<S, F, T, XO> }
#define GBDX_SOLVERS(F)                                        \
  switch (solver) {                                            \
    case GBDX_EULER: return GBDX_ENTRY(GBDX_EULER, F);         \
    case GBDX_HEUN: return GBDX_ENTRY(GBDX_HEUN, F);           \
    case GBDX_DOPRI5: return GBDX_ENTRY(GBDX_DOPRI5, F);       \
    case GBDX_TSIT5: return GBDX_ENTRY(GBDX_TSIT5, F);         \
    case GBDX_DOPRI8: return GBDX_ENTRY(GBDX_DOPRI8, F);       \
    default: return OdeEntry{nullptr, nullptr};                \
  }
  if (field == GBDX_LOTKA_VOLTERRA && dim == 2) { GBDX_SOLVERS(LotkaVolterra<T>) }
  if (field == GBDX_VAN_DER_POL && dim == 2) { GBDX_SOLVERS(VanDerPol<T>) }
  using OU1 = OrnsteinUhlenbeck<T, 1>;
  using OU2 = OrnsteinUhlenbeck<T, 2>;
  using OU4 = OrnsteinUhlenbeck<T, 4>;
  if (field == GBDX_ORNSTEIN_UHLENBECK) {
    if (dim == 1) { GBDX_SOLVERS(OU1) }
    if (dim == 2) { GBDX_SOLVERS(OU2) }
    if (dim == 4) { GBDX_SOLVERS(OU4) }
  }
#undef GBDX_SOLVERS
#undef GBDX_ENTRY
  return OdeEntry{nullptr, nullptr};
}

// The Ornstein-Uhlenbeck SDE (FP32 state: the tree's values are FP32).
template <bool LEVY, bool XO = false>
inline OdeEntry find_ode_sde_entry_t(int solver, int dim) {
#define GBDX_ENTRY(S, F) \
  OdeEntry { &launch_ode<S, F, float, XO>, &occupancy_ode<S, F, float, XO> }
#define GBDX_SOLVERS(F)                                        \
  switch (solver) {                                            \
    case GBDX_EULER: return GBDX_ENTRY(GBDX_EULER, F);         \
    case GBDX_HEUN: return GBDX_ENTRY(GBDX_HEUN, F);           \
    case GBDX_DOPRI5: return GBDX_ENTRY(GBDX_DOPRI5, F);       \
    case GBDX_TSIT5: return GBDX_ENTRY(GBDX_TSIT5, F);         \
    case GBDX_SHARK:                                           \
      if constexpr (LEVY) return GBDX_ENTRY(GBDX_SHARK, F);    \
      return OdeEntry{nullptr, nullptr};                       \
    case GBDX_SRA1:                                            \
      if constexpr (LEVY) return GBDX_ENTRY(GBDX_SRA1, F);     \
      return OdeEntry{nullptr, nullptr};                       \
    case GBDX_SEA:                                             \
      if constexpr (LEVY) return GBDX_ENTRY(GBDX_SEA, F);      \
      return OdeEntry{nullptr, nullptr};                       \
    default: return OdeEntry{nullptr, nullptr};                \
  }
  using OU2 = OrnsteinUhlenbeckSDE<float, 2, LEVY>;
  using OU4 = OrnsteinUhlenbeckSDE<float, 4, LEVY>;
  if (dim == 2) { GBDX_SOLVERS(OU2) }
  if (dim == 4) { GBDX_SOLVERS(OU4) }
#undef GBDX_SOLVERS
#undef GBDX_ENTRY
  return OdeEntry{nullptr, nullptr};
}

}  // namespace gbdx
