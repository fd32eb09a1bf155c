// gbdx_mlp_impl.cuh -- launchers of the MLP-field integrator for one (D, H)
// shape; included by one translation unit per shape so they compile in
// parallel.
#pragma once

#include "gbdx_launch.h"
#include "gbdx_mlp.cuh"

namespace gbdx {

template <int SOLVER, int D, int H, bool PRECISE, bool SDE>
cudaError_t launch_mlp(const SolveParams &P, const LaunchCfg &cfg, cudaStream_t s) {
  using Sm = typename MlpField<MlpShape<D, H>, PRECISE, SDE>::Sm;
  auto k = mlp_fused_kernel<SOLVER, D, H, PRECISE, SDE>;
  cudaError_t e =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sm));
  if (e != cudaSuccess) return e;
  if (P.batch <= 0) return cudaSuccess;
  k<<<cfg.grid, 256, sizeof(Sm), s>>>(P);
  return cudaGetLastError();
}

template <int SOLVER, int D, int H, bool PRECISE, bool SDE>
cudaError_t occupancy_mlp(int block, int *ctas) {
  (void)block;
  using Sm = typename MlpField<MlpShape<D, H>, PRECISE, SDE>::Sm;
  auto k = mlp_fused_kernel<SOLVER, D, H, PRECISE, SDE>;
  cudaError_t e =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sm));
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k, 256, sizeof(Sm));
}

template <int D, int H, bool PRECISE, bool SDE>
OdeEntry mlp_entry_for_solver(int solver) {
#define GBDX_MLP_ENTRY(S) \
  OdeEntry { &launch_mlp<S, D, H, PRECISE, SDE>, &occupancy_mlp<S, D, H, PRECISE, SDE> }
  switch (solver) {
    case GBDX_EULER: return GBDX_MLP_ENTRY(GBDX_EULER);
    case GBDX_HEUN: return GBDX_MLP_ENTRY(GBDX_HEUN);
    case GBDX_DOPRI5:
      if constexpr (!SDE) return GBDX_MLP_ENTRY(GBDX_DOPRI5);
      break;
    case GBDX_TSIT5:
      if constexpr (!SDE) return GBDX_MLP_ENTRY(GBDX_TSIT5);
      break;
    default: break;
  }
#undef GBDX_MLP_ENTRY
  return OdeEntry{nullptr, nullptr};
}

template <int D, int H, bool WITH_SDE>
OdeEntry mlp_entry(int solver, bool precise, bool sde) {
  if (sde) {
    if constexpr (WITH_SDE) {
      return precise ? mlp_entry_for_solver<D, H, true, true>(solver)
                     : mlp_entry_for_solver<D, H, false, true>(solver);
    } else {
      return OdeEntry{nullptr, nullptr};
    }
  }
  return precise ? mlp_entry_for_solver<D, H, true, false>(solver)
                 : mlp_entry_for_solver<D, H, false, false>(solver);
}

}  // namespace gbdx
