// gbdx_noalloc.cu -- a forward solve for callers that cannot allocate.
//
// Some hosts cannot call cudaMalloc at solve time: real-time or embedded
// callers that reserve all device memory at start-up, and plugin hosts that
// hand the solver only its input and output buffers.  For them
// gbdx_solve_fwd_noalloc runs the same
// forward solve as gbdx_solve_fwd but takes its scratch (the work counter and
// the longest-first work order of the fused kernels) from a fixed array that
// this library places in device memory when it is loaded.
//
// The array is kNoAllocScratchBytes (4 MiB) per GPU that loads the library and
// is held until the process exits.  A host-side reference to its symbol is not
// a device address, so the device address is looked up once per device with
// cudaGetSymbolAddress, with that device current, on the first call made on it.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/gbdx.h"

namespace gbdx {
int set_last_error(int code, const char *msg);
}

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
constexpr int kMaxDevices = 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_scratch_mu;
void *g_scratch_ptr[kMaxDevices];

// Device address of the scratch array on the current device (set-up on the
// first call per device).
int scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gbdx::set_last_error(GBDX_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return gbdx::set_last_error(GBDX_ERR_CUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p)
      return gbdx::set_last_error(GBDX_ERR_CUDA, e != cudaSuccess ? cudaGetErrorString(e)
                                                                 : "null scratch address");
    g_scratch_ptr[dev] = p;
  }
  *out = g_scratch_ptr[dev];
  return GBDX_OK;
}

}  // namespace

extern "C" int gbdx_solve_fwd_noalloc(const gbdx_problem *problem, int64_t batch,
                                      const double *t0, const double *t1, const double *dt0,
                                      int64_t time_stride, const void *y0, const void *args,
                                      int64_t args_stride, const void *params,
                                      const double *save_ts, void *ys_out, double *ts_out,
                                      int32_t *result_out, int32_t *stats_out, void *stream) {
  if (!problem) return gbdx::set_last_error(GBDX_ERR_INVALID, "null problem");
  const size_t need = gbdx_workspace_size(problem, batch);
  if (need > kNoAllocScratchBytes)
    return gbdx::set_last_error(
        GBDX_ERR_WORKSPACE,
        "gbdx_solve_fwd_noalloc: this batch needs more scratch than the library's fixed "
        "4 MiB array (more than 1047360 trajectories on the fused kernels); use "
        "gbdx_solve_fwd with a caller workspace");
  void *scratch = nullptr;
  const int rc = scratch_address(&scratch);
  if (rc != GBDX_OK) return rc;
  // gbdx_solve_fwd clears the work counter and rebuilds the work order on the
  // stream before every launch, so the array's previous contents never matter.
  return gbdx_solve_fwd(problem, batch, t0, t1, dt0, time_stride, y0, args, args_stride,
                        params, save_ts, ys_out, ts_out, result_out, stats_out, scratch,
                        kNoAllocScratchBytes, stream);
}
