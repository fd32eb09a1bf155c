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
// The same reduction for partials whose weight blocks are in mma-fragment
// order (tile t of a [no][ni] block holds its 128 values at 128 t + 4 lane + q,
// q indexing (g, 2c), (g, 2c + 1), (g + 8, 2c), (g + 8, 2c + 1)): thread p' of
// the fragment order writes the flat position of its value.  With
// `diffusion`, the neural SDE's [D][D] diffusion weights and D biases follow
// the drift's parameters.
__global__ void reduce_partials_frag_kernel(const float *psum, const float *pcomp, int n_cta,
                                            int D, int H, int diffusion, float *out) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  const int ow0 = 0, ob0 = H * D, ow1 = ob0 + H, ob1 = ow1 + H * H, ow2 = ob1 + H,
            ob2 = ow2 + D * H, ows = ob2 + D, obs = ows + D * D,
            np = diffusion ? obs + D : ows;
  if (q >= np) return;
  int woff = -1, ni = 0;
  if (q < ob0) { woff = ow0; ni = D; }
  else if (q >= ow1 && q < ob1) { woff = ow1; ni = H; }
  else if (q >= ow2 && q < ob2) { woff = ow2; ni = H; }
  else if (diffusion && q >= ows && q < obs) { woff = ows; ni = D; }
  int p = q;
  if (woff >= 0) {
    const int e = q - woff, t = e >> 7, lane = (e & 127) >> 2, k = e & 3;
    const int og = (t / (ni / 8)) * 16 + (lane >> 2) + ((k >> 1) << 3);
    const int ic = (t % (ni / 8)) * 8 + 2 * (lane & 3) + (k & 1);
    p = woff + og * ni + ic;
  }
  float s = 0.f, c = 0.f;
  for (int m = 0; m < n_cta; m++) {
    const float x = psum[size_t(m) * np + q] - pcomp[size_t(m) * np + q];
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  out[p] = s;
}
}  // namespace

cudaError_t launch_reduce_partials_frag(const float *psum, const float *pcomp, int n_cta, int D,
                                        int H, int diffusion, float *out, cudaStream_t s) {
  const int np = H * D + H + H * H + H + D * H + D + (diffusion ? D * D + D : 0);
  reduce_partials_frag_kernel<<<(np + 255) / 256, 256, 0, s>>>(psum, pcomp, n_cta, D, H,
                                                               diffusion, out);
  return cudaGetLastError();
}

cudaError_t launch_reduce_partials(const float *psum, const float *pcomp, int n_cta,
                                   int n_params, float *out, cudaStream_t s) {
  if (n_params <= 0) return cudaSuccess;
  reduce_partials_kernel<<<(n_params + 255) / 256, 256, 0, s>>>(psum, pcomp, n_cta, n_params,
                                                                out);
  return cudaGetLastError();
}

}  // namespace gbdx
