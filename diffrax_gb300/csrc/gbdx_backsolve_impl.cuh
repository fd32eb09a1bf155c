// gbdx_backsolve_impl.cuh -- launchers of the MLP-field BacksolveAdjoint
// backward for one shape.
#pragma once

#include "gbdx_backsolve.cuh"
#include "gbdx_launch.h"

namespace gbdx {

template <int SOLVER, int D, int H, bool PRECISE>
cudaError_t launch_backsolve(const SolveParams &P, const BsParams &Q, int grid, cudaStream_t s) {
  using Sm = typename BsField<BsShape<D, H>, PRECISE>::Sm;
  auto k = mlp_backsolve_kernel<SOLVER, D, H, PRECISE>;
  cudaError_t e =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sm));
  if (e != cudaSuccess) return e;
  if (P.batch <= 0 || grid <= 0) return cudaSuccess;
  k<<<grid, 256, sizeof(Sm), s>>>(P, Q);
  return cudaGetLastError();
}

template <int SOLVER, int D, int H, bool PRECISE>
cudaError_t occupancy_backsolve(int *ctas) {
  using Sm = typename BsField<BsShape<D, H>, PRECISE>::Sm;
  auto k = mlp_backsolve_kernel<SOLVER, D, H, PRECISE>;
  cudaError_t e =
      cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sizeof(Sm));
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, k, 256, sizeof(Sm));
}

template <int D, int H, bool PRECISE, int... SOLVERS>
BsEntry backsolve_entry(int solver) {
  BsEntry out{nullptr, nullptr, 0, 0, 0, 0};
  (void)std::initializer_list<int>{
      (solver == SOLVERS
           ? (out = BsEntry{&launch_backsolve<SOLVERS, D, H, PRECISE>,
                            &occupancy_backsolve<SOLVERS, D, H, PRECISE>, BsShape<D, H>::M,
                            Tab<SOLVERS>::S, BsShape<D, H>::REC, BsShape<D, H>::GFRAG ? 1 : 0},
              0)
           : 0)...};
  return out;
}

}  // namespace gbdx
