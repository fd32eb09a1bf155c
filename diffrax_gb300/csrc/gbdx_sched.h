// gbdx_sched.h -- work ordering for the persistent kernels.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace gbdx {

constexpr int kScheduleBuckets = 1024;

inline size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Workspace bytes needed by build_longest_first_order for n trajectories.
size_t schedule_workspace_bytes(int64_t n);

// Writes into `ws` a permutation of [0, n) ordered by decreasing |t1 - t0|
// (t0, t1 are per-trajectory device arrays) and returns it in *order_out.
cudaError_t build_longest_first_order(const double *t0, const double *t1, int64_t n,
                                      void *ws, int32_t **order_out, cudaStream_t s);

}  // namespace gbdx
