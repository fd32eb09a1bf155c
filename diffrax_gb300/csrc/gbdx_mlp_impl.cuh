// gbdx_mlp_impl.cuh -- launchers of the MLP-field integrator for one (D, H)
// shape; included by one translation unit per shape so they compile in
// parallel.
#pragma once

#include "gbdx_launch.h"
#include "gbdx_mlp.cuh"

namespace gbdx {

// Dynamic shared memory of one CTA: the field and row state, and (XO) the
// event state after it.
template <int D, int H, bool PRECISE, bool SDE, bool XO>
constexpr size_t mlp_smem_bytes() {
  using Sm = typename MlpField<MlpShape<D, H>, PRECISE, SDE>::Sm;
  return XO ? mlp_events_offset<Sm>() + sizeof(RowEvents<MlpShape<D, H>::M>) : sizeof(Sm);
}

template <int SOLVER, int D, int H, bool PRECISE, bool SDE, bool XO>
cudaError_t launch_mlp(const SolveParams &P, const LaunchCfg &cfg, cudaStream_t s) {
  constexpr size_t bytes = mlp_smem_bytes<D, H, PRECISE, SDE, XO>();
  static_assert(bytes <= 227 * 1024, "shared memory of one CTA");
  auto k = mlp_fused_kernel<SOLVER, D, H, PRECISE, SDE, XO>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  if (P.batch <= 0) return cudaSuccess;
  k<<<cfg.grid, 256, bytes, s>>>(P);
  return cudaGetLastError();
}

template <int SOLVER, int D, int H, bool PRECISE, bool SDE, bool XO>
cudaError_t occupancy_mlp(int block, int *ctas) {
  (void)block;
  constexpr size_t bytes = mlp_smem_bytes<D, H, PRECISE, SDE, XO>();
  auto k = mlp_fused_kernel<SOLVER, D, H, PRECISE, SDE, XO>;
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k, 256, bytes);
}

template <int D, int H, bool PRECISE, bool SDE, bool XO>
OdeEntry mlp_entry_for_solver(int solver) {
#define GBDX_MLP_ENTRY(S)                                   \
  OdeEntry {                                                \
    &launch_mlp<S, D, H, PRECISE, SDE, XO>, &occupancy_mlp<S, D, H, PRECISE, SDE, XO> \
  }
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

template <int D, int H, bool WITH_SDE, bool XO>
OdeEntry mlp_entry(int solver, bool precise, bool sde) {
  if (sde) {
    if constexpr (WITH_SDE) {
      return precise ? mlp_entry_for_solver<D, H, true, true, XO>(solver)
                     : mlp_entry_for_solver<D, H, false, true, XO>(solver);
    } else {
      return OdeEntry{nullptr, nullptr};
    }
  }
  return precise ? mlp_entry_for_solver<D, H, true, false, XO>(solver)
                 : mlp_entry_for_solver<D, H, false, false, XO>(solver);
}

}  // namespace gbdx
