// gbdx_launch.h -- host-side launch table shared by the ABI and the kernel
// translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "gbdx_common.cuh"

namespace gbdx {

struct LaunchCfg {
  int kernel;  // GBDX_KERNEL_PLAIN or GBDX_KERNEL_FUSED
  int block;   // threads per CTA (fused)
  int grid;    // CTAs (fused)
};

using OdeLaunchFn = cudaError_t (*)(const SolveParams &, const LaunchCfg &, cudaStream_t);
using OdeOccFn = cudaError_t (*)(int block, int *ctas_per_sm);

struct OdeEntry {
  OdeLaunchFn launch;
  OdeOccFn occupancy;
};

OdeEntry find_ode_entry_f32(int solver, int field, int dim);
OdeEntry find_ode_entry_f64(int solver, int field, int dim);
OdeEntry find_mlp_entry_d64h128(int solver, bool precise, bool sde);
OdeEntry find_mlp_entry_d64h256(int solver, bool precise, bool sde);
OdeEntry find_mlp_entry_d32h64(int solver, bool precise, bool sde);

}  // namespace gbdx
