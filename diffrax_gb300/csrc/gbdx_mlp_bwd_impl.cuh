// gbdx_mlp_bwd_impl.cuh -- launchers of the MLP-field backward for one shape.
#pragma once

#include "gbdx_launch.h"
#include "gbdx_mlp_bwd.cuh"

namespace gbdx {

template <int SOLVER, int D, int H, bool PRECISE, bool SDE>
cudaError_t launch_mlp_bwd(const SolveParams &P, const BwdParams &Q, int grid, cudaStream_t s) {
  using Sm = typename MlpVjp<MlpShape<D, H>, PRECISE, SDE>::Sm;
  auto k = mlp_bwd_kernel<SOLVER, D, H, PRECISE, SDE>;
  cudaError_t e =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sm));
  if (e != cudaSuccess) return e;
  if (P.batch <= 0) return cudaSuccess;
  k<<<grid, 256, sizeof(Sm), s>>>(P, Q);
  return cudaGetLastError();
}

template <int SOLVER, int D, int H, bool PRECISE, bool SDE>
cudaError_t occupancy_mlp_bwd(int *ctas) {
  using Sm = typename MlpVjp<MlpShape<D, H>, PRECISE, SDE>::Sm;
  auto k = mlp_bwd_kernel<SOLVER, D, H, PRECISE, SDE>;
  cudaError_t e =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sm));
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k, 256, sizeof(Sm));
}

template <int D, int H, bool PRECISE, bool SDE>
BwdEntry mlp_bwd_entry_for_solver(int solver) {
#define GBDX_BWD_ENTRY(S) \
  BwdEntry { &launch_mlp_bwd<S, D, H, PRECISE, SDE>, &occupancy_mlp_bwd<S, D, H, PRECISE, SDE> }
  switch (solver) {
    case GBDX_EULER: return GBDX_BWD_ENTRY(GBDX_EULER);
    case GBDX_HEUN: return GBDX_BWD_ENTRY(GBDX_HEUN);
    case GBDX_DOPRI5:
      if constexpr (!SDE) return GBDX_BWD_ENTRY(GBDX_DOPRI5);
      break;
    case GBDX_TSIT5:
      if constexpr (!SDE) return GBDX_BWD_ENTRY(GBDX_TSIT5);
      break;
    default: break;
  }
#undef GBDX_BWD_ENTRY
  return BwdEntry{nullptr, nullptr};
}

template <int D, int H, bool WITH_SDE>
BwdEntry mlp_bwd_entry(int solver, bool precise, bool sde) {
  if (sde) {
    if constexpr (WITH_SDE) {
      return precise ? mlp_bwd_entry_for_solver<D, H, true, true>(solver)
                     : mlp_bwd_entry_for_solver<D, H, false, true>(solver);
    } else {
      return BwdEntry{nullptr, nullptr};
    }
  }
  return precise ? mlp_bwd_entry_for_solver<D, H, true, false>(solver)
                 : mlp_bwd_entry_for_solver<D, H, false, false>(solver);
}

}  // namespace gbdx
