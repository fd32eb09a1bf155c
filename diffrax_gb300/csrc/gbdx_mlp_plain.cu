// gbdx_mlp_plain.cu -- the plain form of the MLP-field solve: one trajectory
// per thread (K0), the MLP evaluated with FP32 dot products on the CUDA cores,
// weights read through the cache hierarchy.  It shares Traj (gbdx_traj.cuh)
// with the analytic fields and is the baseline the row-tile tensor-core
// integrator is compared against.
#include "gbdx_launch.h"
#include "gbdx_mlp_plain.cuh"
#include "gbdx_traj.cuh"

namespace gbdx {

template <int SOLVER, class FIELD>
cudaError_t launch_mlp_plain(const SolveParams &P, const LaunchCfg &cfg, cudaStream_t s) {
  (void)cfg;
  if (P.batch <= 0) return cudaSuccess;
  const int64_t blocks = (P.batch + 127) / 128;
  plain_kernel<SOLVER, FIELD, float><<<(unsigned)blocks, 128, 0, s>>>(P);
  return cudaGetLastError();
}

template <int SOLVER, class FIELD>
cudaError_t occupancy_mlp_plain(int block, int *ctas) {
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(ctas, plain_kernel<SOLVER, FIELD, float>,
                                                       block, 0);
}

// The shapes of the neural-ODE/SDE workloads.
OdeEntry find_mlp_plain_entry(int solver, int D, int H, bool sde) {
  using C3 = MlpPlainField<64, 128, false>;
  using C4 = MlpPlainField<64, 256, false>;
  using C5 = MlpPlainField<32, 64, true>;
  if (!sde && D == 64 && H == 128 && solver == GBDX_TSIT5)
    return OdeEntry{&launch_mlp_plain<GBDX_TSIT5, C3>, &occupancy_mlp_plain<GBDX_TSIT5, C3>};
  if (!sde && D == 64 && H == 256 && solver == GBDX_TSIT5)
    return OdeEntry{&launch_mlp_plain<GBDX_TSIT5, C4>, &occupancy_mlp_plain<GBDX_TSIT5, C4>};
  if (sde && D == 32 && H == 64 && solver == GBDX_HEUN)
    return OdeEntry{&launch_mlp_plain<GBDX_HEUN, C5>, &occupancy_mlp_plain<GBDX_HEUN, C5>};
  return OdeEntry{nullptr, nullptr};
}

}  // namespace gbdx
