// gbdx_reduce.cu -- compensated reduction of per-CTA parameter-gradient partials.
#include "gbdx_launch.h"

namespace gbdx {

namespace {
// grad[p] = sum over CTAs of (sum - comp)[cta][p], Kahan-compensated, in a
// fixed CTA order.
__global__ void reduce_partials_kernel(const float *psum, const float *pcomp, int n_cta,
                                       int n_params, float *out) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n_params) return;
  float s = 0.f, c = 0.f;
  for (int k = 0; k < n_cta; k++) {
    const float x = psum[size_t(k) * n_params + p] - pcomp[size_t(k) * n_params + p];
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  out[p] = s;
}
}  // namespace

cudaError_t launch_reduce_partials(const float *psum, const float *pcomp, int n_cta,
                                   int n_params, float *out, cudaStream_t s) {
  if (n_params <= 0) return cudaSuccess;
  reduce_partials_kernel<<<(n_params + 255) / 256, 256, 0, s>>>(psum, pcomp, n_cta, n_params,
                                                                out);
  return cudaGetLastError();
}

}  // namespace gbdx
