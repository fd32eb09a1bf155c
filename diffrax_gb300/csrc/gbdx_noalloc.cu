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
// a device address, so the device address is looked up with
// cudaGetSymbolAddress, with the device current, on the first call made on it.
// The address belongs to the device's CUDA context: it is kept together with
// that context's identity and looked up again when the context changes (after
// cudaDeviceReset, for one).
#include <cuda.h>
#include <cuda_runtime.h>

#include <stdio.h>

#include <mutex>

#include "../../include/gbdx.h"

namespace gbdx {
int set_last_error(int code, const char *msg);
int problem_adjoint(const gbdx_problem *p);
}

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(4) << 20;
constexpr int kMaxDevices = 256;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct ScratchSlot {
  void *ptr;                // device address of g_noalloc_scratch
  unsigned long long ctx;   // id of the context it was looked up in (0: unknown)
};

std::mutex g_scratch_mu;
ScratchSlot g_scratch[kMaxDevices];

using CtxGetCurrentFn = CUresult (*)(CUcontext *);
using CtxGetIdFn = CUresult (*)(CUcontext, unsigned long long *);

// Id of the calling thread's current CUDA context, through the driver entry
// points the runtime exposes (no link against libcuda).  False when there is
// no current context or the driver does not provide the calls.
bool current_context_id(unsigned long long *id) {
  static CtxGetCurrentFn get_current = nullptr;
  static CtxGetIdFn get_id = nullptr;
  static bool looked_up = false;
  if (!looked_up) {
    looked_up = true;
    void *f = nullptr, *g = nullptr;
    cudaDriverEntryPointQueryResult q1, q2;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault,
                                         &q1) == cudaSuccess &&
        q1 == cudaDriverEntryPointSuccess &&
        cudaGetDriverEntryPointByVersion("cuCtxGetId", &g, 12000, cudaEnableDefault, &q2) ==
            cudaSuccess &&
        q2 == cudaDriverEntryPointSuccess) {
      get_current = reinterpret_cast<CtxGetCurrentFn>(f);
      get_id = reinterpret_cast<CtxGetIdFn>(g);
    }
  }
  if (!get_current || !get_id) return false;
  CUcontext c = nullptr;
  if (get_current(&c) != CUDA_SUCCESS || !c) return false;
  return get_id(c, id) == CUDA_SUCCESS && *id != 0;
}

// Device address of the scratch array on the current device: looked up on
// the first call per device and again whenever the device's context changed.
int scratch_address(void **out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gbdx::set_last_error(GBDX_ERR_CUDA, cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return gbdx::set_last_error(GBDX_ERR_CUDA, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  unsigned long long ctx = 0;
  bool known = current_context_id(&ctx);
  ScratchSlot &slot = g_scratch[dev];
  if (known && slot.ptr && slot.ctx == ctx) {
    *out = slot.ptr;
    return GBDX_OK;
  }
  void *p = nullptr;
  e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p)
    return gbdx::set_last_error(GBDX_ERR_CUDA, e != cudaSuccess ? cudaGetErrorString(e)
                                                               : "null scratch address");
  // the lookup made the device's context current on this thread
  if (!known) known = current_context_id(&ctx);
  slot.ptr = p;
  slot.ctx = known ? ctx : 0;  // unknown: looked up again on the next call
  *out = p;
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
  // A problem created for a gradient records its tape in the workspace, where
  // gbdx_solve_bwd reads it back; a tape in the shared array could not be
  // handed to the backward, so such problems take a caller workspace.
  if (gbdx::problem_adjoint(problem) != GBDX_ADJ_NONE)
    return gbdx::set_last_error(
        GBDX_ERR_UNSUPPORTED,
        "gbdx_solve_fwd_noalloc solves forward-only problems; this problem was created with "
        "an adjoint, whose tape must live in a caller workspace that the backward reads: use "
        "gbdx_solve_fwd");
  const size_t need = gbdx_workspace_size(problem, batch);
  if (need > kNoAllocScratchBytes) {
    char msg[320];
    snprintf(msg, sizeof msg,
             "gbdx_solve_fwd_noalloc: this batch of %lld trajectories needs %zu bytes of "
             "scratch, more than the library's fixed 4 MiB (%zu-byte) array (about 4 bytes "
             "per trajectory: at most 1047360 trajectories on the fused kernels); use "
             "gbdx_solve_fwd with a caller workspace",
             (long long)batch, need, kNoAllocScratchBytes);
    return gbdx::set_last_error(GBDX_ERR_WORKSPACE, msg);
  }
  void *scratch = nullptr;
  const int rc = scratch_address(&scratch);
  if (rc != GBDX_OK) return rc;
  // gbdx_solve_fwd clears the work counter and rebuilds the work order on the
  // stream before every launch, so the array's previous contents never matter.
  return gbdx_solve_fwd(problem, batch, t0, t1, dt0, time_stride, y0, args, args_stride,
                        params, save_ts, ys_out, ts_out, result_out, stats_out, scratch,
                        kNoAllocScratchBytes, stream);
}
