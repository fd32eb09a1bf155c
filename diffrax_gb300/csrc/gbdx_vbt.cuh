// gbdx_vbt.cuh -- device virtual Brownian tree (BrownianIncrement, and
// SpaceTimeLevyArea in vbt_levy_pair).
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

enum { kVbtRoot = 0, kVbtMid = 1, kVbtLeaf = 2, kVbtRootH = 3, kVbtMidH = 4, kVbtLeafH = 5 };

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
  const float r = float((t - P.vbt_t0) * P.vbt_inv_len);
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
  const float sq = P.vbt_sqrt_len;
  return make_float2(sq * (ws0 + f * wsu0 + bb * z.x), sq * (ws1 + f * wsu1 + bb * z.y));
}

// Normals of the quad of dimensions 4 quad .. 4 quad + 3 for one tree node:
// both Box-Muller pairs of one Philox block (vbt_normal_pair returns one).
__device__ __forceinline__ float4 vbt_normal_quad(uint64_t seed, uint32_t traj, uint32_t node,
                                                  uint32_t kind, int quad) {
  uint32_t c[4] = {traj, node, (kind << 24) | uint32_t(quad), 0x5EEDu};
  philox4x32_10(c, uint32_t(seed), uint32_t(seed >> 32));
  float out[4];
#pragma unroll
  for (int p = 0; p < 2; p++) {
    const float u = (float(c[2 * p] >> 8) + 0.5f) * (1.0f / 16777216.0f);
    const float v = (float(c[2 * p + 1] >> 8) + 0.5f) * (1.0f / 16777216.0f);
    const float rad = sqrtf(-2.0f * logf(u));
    float sn, co;
    sincospif(2.0f * v, &sn, &co);
    out[2 * p] = rad * co;
    out[2 * p + 1] = rad * sn;
  }
  return make_float4(out[0], out[1], out[2], out[3]);
}

// The bridge state of one descent path for a quad of dimensions: W at the
// start of each level's dyadic interval and the increment across it.
// Consecutive evaluations of a solve lie close together, so their paths share
// the upper levels; an evaluation re-descends only below the deepest level
// whose interval also contains the new time.
constexpr int kVbtCacheLevels = 24;
struct VbtQuadCache {
  float ws[kVbtCacheLevels + 1][4], wsu[kVbtCacheLevels + 1][4];
  uint32_t node;  // heap index of the cached path's leaf interval
  long long traj; // trajectory of the cached path (-1: none)
};

// sqrt(T) W_unit(r) for the quad of dimensions of trajectory `traj` at time t:
// the values of vbt_w_pair, descending from the cached path.
static __device__ __noinline__ float4 vbt_w_quad(const SolveParams &P, int64_t traj, double t, int quad,
                                          VbtQuadCache &C) {
  const float r = float((t - P.vbt_t0) * P.vbt_inv_len);
  const float tol = float(P.vbt_tol_unit);
  const uint32_t tj = uint32_t(traj);
  // the new path: levels and leaf node, by the comparisons of vbt_w_pair
  float s = 0.f, su = 1.f;
  uint32_t node = 1;
  int L = 0;
  while (su > tol) {
    const float st = 0.5f * su, tm = s + st;
    const bool right = r > tm;
    if (right) s = tm;
    node = 2 * node + (right ? 1u : 0u);
    su = st;
    L++;
  }
  int d = 0;
  if (L <= kVbtCacheLevels && C.traj == (long long)traj) {
    const uint32_t x = node ^ C.node;
    d = x == 0 ? L : L - 1 - (31 - __clz(x));  // levels shared with the cached path
  } else {
    const float4 z = vbt_normal_quad(P.seed, tj, 0u, kVbtRoot, quad);
    if (L <= kVbtCacheLevels) {
      C.traj = (long long)traj;
#pragma unroll
      for (int q = 0; q < 4; q++) C.ws[0][q] = 0.f;
      C.wsu[0][0] = z.x;
      C.wsu[0][1] = z.y;
      C.wsu[0][2] = z.z;
      C.wsu[0][3] = z.w;
    }
  }
  float ws[4], wsu[4];
  if (L <= kVbtCacheLevels) {
#pragma unroll
    for (int q = 0; q < 4; q++) {
      ws[q] = C.ws[d][q];
      wsu[q] = C.wsu[d][q];
    }
  } else {  // deeper than the cache: plain descent from the root
    const float4 z = vbt_normal_quad(P.seed, tj, 0u, kVbtRoot, quad);
    ws[0] = ws[1] = ws[2] = ws[3] = 0.f;
    wsu[0] = z.x;
    wsu[1] = z.y;
    wsu[2] = z.z;
    wsu[3] = z.w;
  }
  // replay the first d decisions for the interval at level d
  s = 0.f;
  su = 1.f;
  for (int l = 0; l < d; l++) {
    const float st = 0.5f * su, tm = s + st;
    if (r > tm) s = tm;
    su = st;
  }
  for (int l = d; l < L; l++) {
    const float st = 0.5f * su, tm = s + st;
    const float4 z = vbt_normal_quad(P.seed, tj, node >> (L - l), kVbtMid, quad);
    const float a = 0.5f * sqrtf(su);
    const float zz[4] = {z.x, z.y, z.z, z.w};
    const bool right = r > tm;
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const float m = 0.5f * wsu[q];
      const float wst = m + a * zz[q], wtu = m - a * zz[q];
      if (right) {
        ws[q] += wst;
        wsu[q] = wtu;
      } else {
        wsu[q] = wst;
      }
    }
    if (right) s = tm;
    su = st;
    if (l + 1 <= kVbtCacheLevels) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        C.ws[l + 1][q] = ws[q];
        C.wsu[l + 1][q] = wsu[q];
      }
    }
  }
  C.node = node;
  const float sr = fmaxf(r - s, 0.f), ru = fmaxf(su - sr, 0.f);
  const float4 z = vbt_normal_quad(P.seed, tj, node, kVbtLeaf, quad);
  const float bb = sqrtf(sr * ru / su), f = sr / su;
  const float sq = P.vbt_sqrt_len;
  return make_float4(sq * (ws[0] + f * wsu[0] + bb * z.x), sq * (ws[1] + f * wsu[1] + bb * z.y),
                     sq * (ws[2] + f * wsu[2] + bb * z.z), sq * (ws[3] + f * wsu[3] + bb * z.w));
}

// The tree with space-time Levy area: W_unit(r) and bar H_unit(r) = r H_{0,r}
// at unit time r for dimensions (col, col + 1), col even, unscaled (the caller
// combines two points by Chen's relation and scales by sqrt(T)).  The descent
// carries W and bar H of each dyadic interval: root W_1 ~ N(0, 1), bar H_1 ~
// N(0, 1/12) (tree.py:389-394); midpoint rule tree.py:727-750; final bridge
// tree.py:562-603.  The kVbt*H draws feed bar H, the others W, as in the
// FP64 oracle.
static __device__ __noinline__ void vbt_levy_pair(const SolveParams &P, int64_t traj, float r, int col,
                                                  float2 &w_r, float2 &bhh_r) {
  const float tol = float(P.vbt_tol_unit);
  const uint32_t tj = uint32_t(traj);
  const float2 z0 = vbt_normal_pair(P.seed, tj, 0u, kVbtRoot, col);
  const float2 n0 = vbt_normal_pair(P.seed, tj, 0u, kVbtRootH, col);
  float ws[2] = {0.f, 0.f}, wsu[2] = {z0.x, z0.y};
  float hs[2] = {0.f, 0.f};
  const float inv_sqrt12 = 0.28867513459481287f;
  float hsu[2] = {n0.x * inv_sqrt12, n0.y * inv_sqrt12};
  float s = 0.f, su = 1.f;
  uint32_t node = 1;
  while (su > tol) {  // while 2^-level > tol (tree.py:406-409)
    const float st = 0.5f * su, t_mid = s + st;
    const float2 z1 = vbt_normal_pair(P.seed, tj, node, kVbtMid, col);
    const float2 z2 = vbt_normal_pair(P.seed, tj, node, kVbtMidH, col);
    const float zs = 0.25f * sqrtf(su), ns = sqrtf(su * (1.0f / 12.0f));
    const float c3 = 1.5f / su, q = 0.25f * su;
    const bool right = r > t_mid;
    const float zz1[2] = {z1.x, z1.y}, zz2[2] = {z2.x, z2.y};
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const float z = zz1[i] * zs, n = zz2[i] * ns;
      const float wt1 = 0.5f * wsu[i], wt2 = c3 * hsu[i] + z;
      const float ht1 = 0.125f * hsu[i] - q * z, ht2 = q * n;
      if (right) {
        const float w_t = ws[i] + (wt1 + wt2);
        hs[i] = hs[i] + (ht1 + ht2) + 0.5f * (t_mid * ws[i] - s * w_t);
        ws[i] = w_t;
        wsu[i] = wt1 - wt2;
        hsu[i] = ht1 - ht2;
      } else {
        wsu[i] = wt1 + wt2;
        hsu[i] = ht1 + ht2;
      }
    }
    if (right) s = t_mid;
    node = 2 * node + (right ? 1u : 0u);
    su = st;
  }
  const float sr = fmaxf(r - s, 0.f), ru = fmaxf(su - sr, 0.f);
  const float2 x1 = vbt_normal_pair(P.seed, tj, node, kVbtLeaf, col);
  const float2 x2 = vbt_normal_pair(P.seed, tj, node, kVbtLeafH, col);
  const float sr3 = sr * sr * sr, ru3 = ru * ru * ru, su3 = su * su * su;
  const float dd = sqrtf(sr3 + ru3);
  const float sr_ru_half = sqrtf(sr * ru);
  const float d_prime = 1.0f / (2.0f * su * dd);
  const float a = d_prime * sr3 * sr_ru_half, b = d_prime * ru3 * sr_ru_half;
  const float c = sqrtf(3.0f * sr3 * ru3) / (6.0f * dd);
  const float fw = sr / su, fh = 6.0f * sr * ru / su3, fx = 2.0f * (a + b) / su, fb = sr3 / su3;
  const float xx1[2] = {x1.x, x1.y}, xx2[2] = {x2.x, x2.y};
  float wo[2], ho[2];
#pragma unroll
  for (int i = 0; i < 2; i++) {
    const float w_sr = fw * wsu[i] + fh * hsu[i] + fx * xx1[i];
    wo[i] = ws[i] + w_sr;
    const float bhh_sr = fb * hsu[i] - a * xx1[i] + c * xx2[i];
    ho[i] = hs[i] + bhh_sr + 0.5f * (r * ws[i] - s * wo[i]);
  }
  w_r = make_float2(wo[0], wo[1]);
  bhh_r = make_float2(ho[0], ho[1]);
}

}  // namespace gbdx
