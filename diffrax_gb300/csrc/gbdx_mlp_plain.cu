// gbdx_mlp_plain.cu -- the plain form of the MLP-field solve: one trajectory
// per thread (K0), the MLP evaluated with FP32 dot products on the CUDA cores,
// weights read through the cache hierarchy.  It shares Traj (gbdx_traj.cuh)
// with the analytic fields and is the baseline the row-tile tensor-core
// integrator is compared against.
#include "gbdx_launch.h"
#include "gbdx_traj.cuh"

namespace gbdx {

template <int D_, int H, bool DIFF>
struct MlpPlainField {
  static constexpr int D = D_, NARGS = 0;
  static constexpr bool SDE = DIFF;
  // flat layout: W0 [H][D], b0, W1 [H][H], b1, W2 [D][H], b2, Ws [D][D], bs
  __device__ static void vf(const SolveParams &P, const float *, const float *y, float *o) {
    const float *W0 = P.mlp, *b0 = W0 + H * D, *W1 = b0 + H, *b1 = W1 + H * H, *W2 = b1 + H,
                *b2 = W2 + D * H;
    float h1[H], h2[H];
#pragma unroll 1
    for (int n = 0; n < H; n++) {
      float a = __ldg(b0 + n);
      for (int k = 0; k < D; k++) a = fmaf(__ldg(W0 + n * D + k), y[k], a);
      h1[n] = tanhf(a);
    }
#pragma unroll 1
    for (int n = 0; n < H; n++) {
      float a = __ldg(b1 + n);
      for (int k = 0; k < H; k++) a = fmaf(__ldg(W1 + n * H + k), h1[k], a);
      h2[n] = tanhf(a);
    }
#pragma unroll 1
    for (int n = 0; n < D; n++) {
      float a = __ldg(b2 + n);
      for (int k = 0; k < H; k++) a = fmaf(__ldg(W2 + n * H + k), h2[k], a);
      o[n] = a;
    }
  }
  __device__ static void sigma(const SolveParams &P, const float *, const float *y, float *s) {
    const float *Ws = P.mlp + (H * D + H + H * H + H + D * H + D), *bs = Ws + D * D;
#pragma unroll 1
    for (int n = 0; n < D; n++) {
      float a = __ldg(bs + n);
      for (int k = 0; k < D; k++) a = fmaf(__ldg(Ws + n * D + k), y[k], a);
      s[n] = 0.1f * tanhf(a);
    }
  }
};

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
