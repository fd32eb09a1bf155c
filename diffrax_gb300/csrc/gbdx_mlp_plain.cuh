// gbdx_mlp_plain.cuh -- the MLP field of the plain form (one trajectory per
// thread): FP32 dot products on the CUDA cores, weights read through the cache
// hierarchy, and its VJP for the plain backward.
#pragma once

#include "gbdx_common.cuh"

namespace gbdx {

template <int D_, int H, bool DIFF>
struct MlpPlainField {
  static constexpr int D = D_, NARGS = 0;
  static constexpr bool SDE = DIFF;
  static constexpr bool TAPE = true;  // records the full gradient tape when asked
  // flat layout: W0 [H][D], b0, W1 [H][H], b1, W2 [D][H], b2, Ws [D][D], bs
  static constexpr int OW0 = 0, OB0 = H * D, OW1 = OB0 + H, OB1 = OW1 + H * H, OW2 = OB1 + H,
                       OB2 = OW2 + D * H, OWS = OB2 + D, OBS = OWS + D * D;
  static constexpr int NP = OWS + (DIFF ? D * D + D : 0);

  __device__ static void hidden(const float *W, const float *y, float (&h1)[H], float (&h2)[H]) {
#pragma unroll 1
    for (int n = 0; n < H; n++) {
      float a = __ldg(W + OB0 + n);
      for (int k = 0; k < D; k++) a = fmaf(__ldg(W + OW0 + n * D + k), y[k], a);
      h1[n] = tanhf(a);
    }
#pragma unroll 1
    for (int n = 0; n < H; n++) {
      float a = __ldg(W + OB1 + n);
      for (int k = 0; k < H; k++) a = fmaf(__ldg(W + OW1 + n * H + k), h1[k], a);
      h2[n] = tanhf(a);
    }
  }

  __device__ static void vf(const SolveParams &P, const float *, const float *y, float *o) {
    float h1[H], h2[H];
    hidden(P.mlp, y, h1, h2);
#pragma unroll 1
    for (int n = 0; n < D; n++) {
      float a = __ldg(P.mlp + OB2 + n);
      for (int k = 0; k < H; k++) a = fmaf(__ldg(P.mlp + OW2 + n * H + k), h2[k], a);
      o[n] = a;
    }
  }

  __device__ static void sigma(const SolveParams &P, const float *, const float *y, float *s) {
#pragma unroll 1
    for (int n = 0; n < D; n++) {
      float a = __ldg(P.mlp + OBS + n);
      for (int k = 0; k < D; k++) a = fmaf(__ldg(P.mlp + OWS + n * D + k), y[k], a);
      s[n] = 0.1f * tanhf(a);
    }
  }

  // gy += (df/dy)^T g + (d sigma/dy)^T (gs); every parameter cotangent v_p
  // (each parameter once) is handed to add(p, v_p).
  template <class ADD>
  __device__ static void vjp_with(const float *W, const float *y, const float *g, const float *gs,
                                  float *gy, ADD add) {
    float h1[H], h2[H], dz[H], dz0[H];
    hidden(W, y, h1, h2);
#pragma unroll 1
    for (int o = 0; o < D; o++) {
      const float go = g[o];
      add(OB2 + o, go);
      for (int k = 0; k < H; k++) add(OW2 + o * H + k, go * h2[k]);
    }
#pragma unroll 1
    for (int k = 0; k < H; k++) {
      float a = 0.f;
      for (int o = 0; o < D; o++) a = fmaf(__ldg(W + OW2 + o * H + k), g[o], a);
      dz[k] = a * (1.f - h2[k] * h2[k]);
    }
#pragma unroll 1
    for (int n = 0; n < H; n++) {
      add(OB1 + n, dz[n]);
      for (int k = 0; k < H; k++) add(OW1 + n * H + k, dz[n] * h1[k]);
    }
#pragma unroll 1
    for (int k = 0; k < H; k++) {
      float a = 0.f;
      for (int n = 0; n < H; n++) a = fmaf(__ldg(W + OW1 + n * H + k), dz[n], a);
      dz0[k] = a * (1.f - h1[k] * h1[k]);
    }
#pragma unroll 1
    for (int n = 0; n < H; n++) {
      add(OB0 + n, dz0[n]);
      for (int k = 0; k < D; k++) add(OW0 + n * D + k, dz0[n] * y[k]);
    }
#pragma unroll 1
    for (int k = 0; k < D; k++) {
      float a = 0.f;
      for (int n = 0; n < H; n++) a = fmaf(__ldg(W + OW0 + n * D + k), dz0[n], a);
      gy[k] += a;
    }
    if constexpr (DIFF) {
      // sigma = 0.1 tanh(Ws y + bs): d sigma / dz = 0.1 (1 - tanh^2)
      float gz[D];
#pragma unroll 1
      for (int n = 0; n < D; n++) {
        float a = __ldg(W + OBS + n);
        for (int k = 0; k < D; k++) a = fmaf(__ldg(W + OWS + n * D + k), y[k], a);
        const float th = tanhf(a);
        gz[n] = gs[n] * 0.1f * (1.f - th * th);
        add(OBS + n, gz[n]);
        for (int k = 0; k < D; k++) add(OWS + n * D + k, gz[n] * y[k]);
      }
#pragma unroll 1
      for (int k = 0; k < D; k++) {
        float a = 0.f;
        for (int n = 0; n < D; n++) a = fmaf(__ldg(W + OWS + n * D + k), gz[n], a);
        gy[k] += a;
      }
    }
  }

  // The parameter cotangents added to this trajectory's column of dP
  // ([NP][stride] layout, coalesced across the threads of a warp).
  __device__ static void vjp(const float *W, const float *y, const float *g, const float *gs,
                             float *gy, float *dP, int64_t stride) {
    vjp_with(W, y, g, gs, gy, [&](int p, float v) { dP[p * stride] += v; });
  }
};

}  // namespace gbdx
