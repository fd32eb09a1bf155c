// gbdx_vbt.cuh -- device virtual Brownian tree (BrownianIncrement).
//
// W(t) on [vbt_t0, vbt_t0 + T] by binary bridge descent from a counter-based
// generator, as VirtualBrownianTree._evaluate_leaf (diffrax/_brownian/
// tree.py:366-448, 607-621) with the midpoint rule of _brownian_arch
// (:752-768).  Jax's threefry key splitting is replaced by Philox4x32-10
// counters (trajectory, tree node, draw kind, dimension quad): every node has
// its own independent normals, as in the reference.  The FP64 oracle uses the
// same integer stream.
#pragma once

#include <stdint.h>

#include "gbdx_common.cuh"

namespace gbdx {

__device__ __forceinline__ void philox4x32_10(uint32_t (&c)[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const uint32_t lo0 = 0xD2511F53u * c[0], hi0 = __umulhi(0xD2511F53u, c[0]);
    const uint32_t lo1 = 0xCD9E8D57u * c[2], hi1 = __umulhi(0xCD9E8D57u, c[2]);
    const uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
}

enum { kVbtRoot = 0, kVbtMid = 1, kVbtLeaf = 2 };

// Normals of dimensions (col, col + 1), col even, for one tree node.
__device__ __forceinline__ float2 vbt_normal_pair(uint64_t seed, uint32_t traj, uint32_t node,
                                                  uint32_t kind, int col) {
  uint32_t c[4] = {traj, node, (kind << 24) | uint32_t(col >> 2), 0x5EEDu};
  philox4x32_10(c, uint32_t(seed), uint32_t(seed >> 32));
  const int p = (col >> 1) & 1;  // which Box-Muller pair of the quad
  const float u = (float(c[2 * p] >> 8) + 0.5f) * (1.0f / 16777216.0f);
  const float v = (float(c[2 * p + 1] >> 8) + 0.5f) * (1.0f / 16777216.0f);
  const float rad = sqrtf(-2.0f * logf(u));
  float s, co;
  sincospif(2.0f * v, &s, &co);
  return make_float2(rad * co, rad * s);
}

// sqrt(T) W_unit(r) for dimensions (col, col + 1) of trajectory `traj` at time t.
static __device__ __noinline__ float2 vbt_w_pair(const SolveParams &P, int64_t traj, double t,
                                          int col) {
  const float r = float((t - P.vbt_t0) / P.vbt_len);
  const float tol = float(P.vbt_tol_unit);
  const uint32_t tj = uint32_t(traj);
  float2 z = vbt_normal_pair(P.seed, tj, 0u, kVbtRoot, col);
  float ws0 = 0.f, ws1 = 0.f, wsu0 = z.x, wsu1 = z.y;
  float s = 0.f, su = 1.f;
  uint32_t node = 1;
  // while 2^-level > tol (tree.py:406-409)
  while (su > tol) {
    const float st = 0.5f * su, t_mid = s + st;
    z = vbt_normal_pair(P.seed, tj, node, kVbtMid, col);
    const float a = 0.5f * sqrtf(su);
    const float m0 = 0.5f * wsu0, m1 = 0.5f * wsu1;
    const float st0 = m0 + a * z.x, st1 = m1 + a * z.y;  // W_{s,t}
    const float tu0 = m0 - a * z.x, tu1 = m1 - a * z.y;  // W_{t,u}
    const bool right = r > t_mid;
    if (right) {
      ws0 += st0;
      ws1 += st1;
      wsu0 = tu0;
      wsu1 = tu1;
      s = t_mid;
    } else {
      wsu0 = st0;
      wsu1 = st1;
    }
    node = 2 * node + (right ? 1u : 0u);
    su = st;
  }
  const float sr = fmaxf(r - s, 0.f), ru = fmaxf(su - sr, 0.f);
  z = vbt_normal_pair(P.seed, tj, node, kVbtLeaf, col);
  const float bb = sqrtf(sr * ru / su), f = sr / su;
  const float sq = float(sqrt(P.vbt_len));
  return make_float2(sq * (ws0 + f * wsu0 + bb * z.x), sq * (ws1 + f * wsu1 + bb * z.y));
}

}  // namespace gbdx
