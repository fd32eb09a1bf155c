// gbdx_mlp_bwd.cuh -- RecursiveCheckpointAdjoint backward for MLP fields.
//
// The reference differentiates the discrete solve (diffrax/_adjoint.py:179-312):
// rejected steps get zero cotangent through where(keep, ...) (_integrate.py:
// 422-424) and the controller is under stop_gradient (pid.py:374, 499-501,
// 529-530), so the gradient is the VJP of the chain of accepted steps on the
// realised time grid.  Checkpointing changes only what is recomputed.
//
// The forward kernel records that grid (FP64, every accepted step) and the
// state at checkpoints (every accepted step while the slots last, then every
// 2nd, 4th, ... step).  Here a CTA of 8 warps walks a tile of M trajectories
// backwards in lockstep.  One iteration of a row is either
//   * BWD: recompute the stages of accepted step n from y_n, then the exact VJP
//     of the step -- interpolant VJP of the saves inside it, the reverse stage
//     loop with the MLP backprop on the tensor cores (transposed ldmatrix
//     operands) and, for SDEs, the diffusion VJP; or
//   * FWD: recompute one step forward inside a checkpoint segment, storing the
//     state in a per-trajectory scratch (only when the checkpoint stride > 1).
// Parameter gradients accumulate per CTA in FP32 with Kahan compensation; a
// final kernel sums the CTA partials, again compensated.
#pragma once

#include "gbdx_mlp.cuh"

namespace gbdx {

__device__ __forceinline__ void kahan_add(float *sum, float *comp, float x) {
  const float y = x - *comp;
  const float t = *sum + y;
  *comp = (t - *sum) - y;
  *sum = t;
}

// Interpolant as a linear map of (y0, y1, k_j): out = ay0 y0 + ay1 y1 +
// sum_j g_j k_j (tsit5.py:119-150, _local_interpolation.py:29-139).
template <int SOLVER>
__device__ __forceinline__ void interp_coeffs(float th, float &ay0, float &ay1, float (&g)[7]) {
#pragma unroll
  for (int j = 0; j < 7; j++) g[j] = 0.f;
  const float t2 = th * th, t3 = t2 * th, t4 = t3 * th;
  if constexpr (SOLVER == GBDX_TSIT5) {
    ay0 = 1.f;
    ay1 = 0.f;
#pragma unroll
    for (int j = 0; j < 7; j++) g[j] = tsit5_w<float>(j, th);
  } else if constexpr (SOLVER == GBDX_DOPRI5) {
    const float Mm = 16.f * t4 - 32.f * t3 + 16.f * t2;
    ay0 = -8.f * t4 + 18.f * t3 - 11.f * t2 + 1.f + Mm;
    ay1 = -8.f * t4 + 14.f * t3 - 5.f * t2;
#pragma unroll
    for (int j = 0; j < 7; j++) g[j] = Mm * float(Tab<GBDX_DOPRI5>::cmid(j));
    g[0] += -2.f * t4 + 5.f * t3 - 4.f * t2 + th;
    g[6] += 2.f * t4 - 3.f * t3 + t2;
  } else if constexpr (SOLVER == GBDX_HEUN) {
    ay0 = 2.f * t3 - 3.f * t2 + 1.f;
    ay1 = -2.f * t3 + 3.f * t2;
    g[0] = t3 - 2.f * t2 + th;
    g[1] = t3 - t2;
  } else {
    ay0 = 1.f - th;
    ay1 = th;
  }
}

template <int M>
struct BwdRows {
  double t_lo[M], t_hi[M];
  long long idx[M];
  float h[M], theta[M];
  int active[M], loaded[M], fin[M], dir[M], mode[M], n[M], m[M], N[M], s[M], cs[M];
  int k_lo[M], k_hi[M], sflag[M], sslot[M], ld_kind[M], ld_slot[M], live[M];
  // SDE: the time whose Brownian value W the row's threads carry from the
  // row's previous iteration (NaN: none), and which ends of this iteration's
  // step still need a tree evaluation
  double wt[M];
  int w_lo[M], w_hi[M];
};
enum { kModeBwd = 0, kModeFwd = 1 };
enum { kLoadNone = 0, kLoadCheckpoint = 1, kLoadScratch = 2 };

template <class SH, bool PRECISE, bool SDE>
struct BwdSmem;

// The cotangents are held as three BF16 pieces like the forward's
// activations (24 significant bits), so the gradient keeps the accuracy of an
// FP32 evaluation with the same BF16 weights.  The layer-0 cotangent G1 is
// written into the storage of the layer-1 activations A2 (all three pieces),
// which are dead once dW2 has been accumulated.
template <class SH, bool SDE>
struct BwdSmem<SH, false, SDE> {
  static_assert(SH::NP == 3 && !SH::GFRAG,
                "three-piece operands, weights in shared memory");
  MlpSmem<SH, false, SDE> f;  // weights, biases, X, A1, A2 (forward recompute)
  __nv_bfloat16 G3[SH::M][SH::PD], G3l[SH::M][SH::PD], G3l2[SH::M][SH::PD];
  __nv_bfloat16 Gs[SDE ? SH::M : 1][SH::PD], Gsl[SDE ? SH::M : 1][SH::PD],
      Gsl2[SDE ? SH::M : 1][SH::PD];
  __nv_bfloat16 G2[SH::M][SH::PH], G2l[SH::M][SH::PH], G2l2[SH::M][SH::PH];
  float db0[SH::H], db1[SH::H], db2[SH::D], dbs[SH::D];
  BwdRows<SH::M> rows;
};

template <class SH, bool SDE>
struct BwdSmem<SH, true, SDE> {
  MlpSmem<SH, true, SDE> f;
  float G3[SH::M][SH::D + 1];
  float Gs[SDE ? SH::M : 1][SH::D + 1];
  float G2[SH::M][SH::H + 1];
  float G1[SH::M][SH::H + 1];
  float db0[SH::H], db1[SH::H], db2[SH::D], dbs[SH::D];
  BwdRows<SH::M> rows;
};

// dW[o][n] (the [O][N] block at offset `off`) += G^T S over the tile's rows,
// with G and S held as three BF16 pieces each (warp_tile_gemm_tt3),
// accumulated into this CTA's Kahan partials.  The partials of a weight block
// are in mma-fragment order: m16n8 tile t = (o / 16) (N / 8) + n / 8 holds its
// 128 values at off + 128 t + 4 lane + q, q indexing the accumulator elements
// (g, 2c), (g, 2c + 1), (g + 8, 2c), (g + 8, 2c + 1), so a lane's four values
// are one 16-byte load and store (the final reduction restores the flat
// order).
template <class SH, int O, int N>
__device__ __forceinline__ void dw_tiles(const __nv_bfloat16 *const (&G)[3], int ldg,
                                         const __nv_bfloat16 *const (&S)[3], int lds, int off,
                                         float *psum, float *pcomp, int warp, int lane) {
  constexpr int TILES = (O / 16) * (N / 8);
  static_assert(TILES % SH::WARPS == 0, "weight-gradient tile split");
  constexpr int T = TILES / SH::WARPS;
  constexpr int CH = T < 8 ? T : 8;
  static_assert((N / 8) % CH == 0 && T % CH == 0, "weight-gradient chunk split");
  const int g = lane >> 2, c = lane & 3;
#pragma unroll 1
  for (int ch = 0; ch < T / CH; ch++) {
    const int t = warp * T + ch * CH;
    const int ot = t / (N / 8), nt0 = t % (N / 8);
    // the partials this chunk updates are loaded before its products, so the
    // L2 latency overlaps the tensor-core work
    float4 ps[CH], pc[CH];
#pragma unroll
    for (int j = 0; j < CH; j++) {
      const int p = off + (t + j) * 128 + lane * 4;
      ps[j] = *reinterpret_cast<const float4 *>(psum + p);
      pc[j] = *reinterpret_cast<const float4 *>(pcomp + p);
    }
    float acc[CH][4];
#pragma unroll
    for (int j = 0; j < CH; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
    warp_tile_gemm_tt3<SH::M, CH>(acc, G, ldg, ot * 16, S, lds, nt0 * 8, lane);
#pragma unroll
    for (int j = 0; j < CH; j++) {
      float sv[4] = {ps[j].x, ps[j].y, ps[j].z, ps[j].w};
      float cv[4] = {pc[j].x, pc[j].y, pc[j].z, pc[j].w};
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const float y = acc[j][q] - cv[q];
        const float tq = sv[q] + y;
        cv[q] = (tq - sv[q]) - y;
        sv[q] = tq;
      }
      const int p = off + (t + j) * 128 + lane * 4;
      *reinterpret_cast<float4 *>(psum + p) = make_float4(sv[0], sv[1], sv[2], sv[3]);
      *reinterpret_cast<float4 *>(pcomp + p) = make_float4(cv[0], cv[1], cv[2], cv[3]);
    }
  }
}

template <class SH, bool PRECISE, bool SDE>
struct MlpVjp {
  using Sm = BwdSmem<SH, PRECISE, SDE>;
  static constexpr int D = SH::D, H = SH::H, M = SH::M, NE = SH::NE;

  // Given the forward recompute of one stage (X, A1, A2 in smem; sig in
  // registers) and the cotangents of its output F (G3) and of its diffusion
  // sigma (Gsig, SDE), return gY = d<G3, F> / dY + d<Gsig, sigma> / dY in the
  // owned layout and accumulate the parameter gradients.
  __device__ static void run(Sm &sm, const float *P, const float (&G3r)[NE],
                             const float (&Gsr)[NE], const float (&sig)[NE], float (&gY)[NE],
                             float *psum, float *pcomp, int tid, int warp, int lane) {
    // 1. output cotangents to smem, bias gradients of the last layer
#pragma unroll
    for (int e = 0; e < NE; e++) {
      int row, col;
      elem_rc<SH>(e, warp, lane, row, col);
      // sigma = 0.1 tanh(z): d sigma / dz = 0.1 (1 - (sigma / 0.1)^2)
      const float gz = SDE ? Gsr[e] * 0.1f * (1.f - 100.f * sig[e] * sig[e]) : 0.f;
      if constexpr (PRECISE) {
        sm.G3[row][col] = G3r[e];
        if constexpr (SDE) sm.Gs[row][col] = gz;
      } else {
        if ((e & 1) == 0)
          store_split3x2(G3r[e], G3r[e + 1], &sm.G3[row][col], &sm.G3l[row][col],
                         &sm.G3l2[row][col]);
        if constexpr (SDE) split_store3(gz, &sm.Gs[row][col], &sm.Gsl[row][col], &sm.Gsl2[row][col]);
      }
      if (G3r[e] != 0.f) atomicAdd(&sm.db2[col], G3r[e]);
      if (SDE && gz != 0.f) atomicAdd(&sm.dbs[col], gz);
    }
    __syncthreads();
    if constexpr (PRECISE) {
      const float *W0 = P + SH::OW0, *W1 = P + SH::OW1, *W2 = P + SH::OW2, *Ws = P + SH::OWS;
      // 2. G2 = (G3 W2) * (1 - A2^2); dW2 += G3^T A2
      for (int i = tid; i < M * H; i += SH::THREADS) {
        const int r = i / H, hh = i % H;
        float a = 0.f;
        for (int d = 0; d < D; d++) a = fmaf(sm.G3[r][d], __ldg(W2 + d * H + hh), a);
        const float ah = sm.f.A2[r][hh];
        const float v = a * (1.f - ah * ah);
        sm.G2[r][hh] = v;
        if (v != 0.f) atomicAdd(&sm.db1[hh], v);
      }
      for (int i = tid; i < D * H; i += SH::THREADS) {
        const int d = i / H, hh = i % H;
        float a = 0.f;
        for (int r = 0; r < M; r++) a = fmaf(sm.G3[r][d], sm.f.A2[r][hh], a);
        kahan_add(psum + SH::OW2 + i, pcomp + SH::OW2 + i, a);
      }
      __syncthreads();
      // 3. G1 = (G2 W1) * (1 - A1^2); dW1 += G2^T A1
      for (int i = tid; i < M * H; i += SH::THREADS) {
        const int r = i / H, hh = i % H;
        float a = 0.f;
        for (int o = 0; o < H; o++) a = fmaf(sm.G2[r][o], __ldg(W1 + o * H + hh), a);
        const float ah = sm.f.A1[r][hh];
        const float v = a * (1.f - ah * ah);
        sm.G1[r][hh] = v;
        if (v != 0.f) atomicAdd(&sm.db0[hh], v);
      }
      for (int i = tid; i < H * H; i += SH::THREADS) {
        const int o = i / H, hh = i % H;
        float a = 0.f;
        for (int r = 0; r < M; r++) a = fmaf(sm.G2[r][o], sm.f.A1[r][hh], a);
        kahan_add(psum + SH::OW1 + i, pcomp + SH::OW1 + i, a);
      }
      __syncthreads();
      // 4. gY = G1 W0 (+ Gs Ws); dW0 += G1^T X (dWs += Gs^T X)
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        float a = 0.f;
        for (int o = 0; o < H; o++) a = fmaf(sm.G1[row][o], __ldg(W0 + o * D + col), a);
        if constexpr (SDE)
          for (int o = 0; o < D; o++) a = fmaf(sm.Gs[row][o], __ldg(Ws + o * D + col), a);
        gY[e] = a;
      }
      for (int i = tid; i < H * D; i += SH::THREADS) {
        const int o = i / D, d = i % D;
        float a = 0.f;
        for (int r = 0; r < M; r++) a = fmaf(sm.G1[r][o], sm.f.X[r][d], a);
        kahan_add(psum + SH::OW0 + i, pcomp + SH::OW0 + i, a);
      }
      if constexpr (SDE)
        for (int i = tid; i < D * D; i += SH::THREADS) {
          const int o = i / D, d = i % D;
          float a = 0.f;
          for (int r = 0; r < M; r++) a = fmaf(sm.Gs[r][o], sm.f.X[r][d], a);
          kahan_add(psum + SH::OWS + i, pcomp + SH::OWS + i, a);
        }
    } else {
      const int g = lane >> 2, c = lane & 3;
      const __nv_bfloat16 *const G3p[3] = {&sm.G3[0][0], &sm.G3l[0][0], &sm.G3l2[0][0]};
      const __nv_bfloat16 *const G2p[3] = {&sm.G2[0][0], &sm.G2l[0][0], &sm.G2l2[0][0]};
      {  // 2. G2 = (G3 W2) * (1 - A2^2), hidden-tile layout
        const int t0 = warp * SH::TPWH, mt = t0 / SH::NTH, nt0 = t0 % SH::NTH;
        float acc[SH::TPWH][4];
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        warp_tile_gemm_bt3<D, SH::TPWH>(acc, &sm.G3[mt * 16][0], &sm.G3l[mt * 16][0],
                                        &sm.G3l2[mt * 16][0], SH::PD, &sm.f.W2[0][0], SH::PH,
                                        nt0 * 8, lane);
        auto A2 = sm.f.a2();
        auto A2l = sm.f.a2l();
        auto A2l2 = sm.f.a2l2();
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++)
#pragma unroll
          for (int hr = 0; hr < 2; hr++) {
            const int row = mt * 16 + g + hr * 8, col = (nt0 + j) * 8 + 2 * c;
            const float a0 = __bfloat162float(A2[row][col]) + __bfloat162float(A2l[row][col]) +
                             __bfloat162float(A2l2[row][col]);
            const float a1 = __bfloat162float(A2[row][col + 1]) +
                             __bfloat162float(A2l[row][col + 1]) +
                             __bfloat162float(A2l2[row][col + 1]);
            const float v0 = acc[j][2 * hr] * (1.f - a0 * a0);
            const float v1 = acc[j][2 * hr + 1] * (1.f - a1 * a1);
            store_split3x2(v0, v1, &sm.G2[row][col], &sm.G2l[row][col], &sm.G2l2[row][col]);
            if (v0 != 0.f) atomicAdd(&sm.db1[col], v0);
            if (v1 != 0.f) atomicAdd(&sm.db1[col + 1], v1);
          }
      }
      {
        const __nv_bfloat16 *const A2p[3] = {&sm.f.a2()[0][0], &sm.f.a2l()[0][0],
                                             &sm.f.a2l2()[0][0]};
        dw_tiles<SH, D, H>(G3p, SH::PD, A2p, SH::PH, SH::OW2, psum, pcomp, warp, lane);
      }
      __syncthreads();
      // A2 is dead from here: G1 (three pieces) takes its storage
      __nv_bfloat16(*G1)[SH::PH] = sm.f.a2();
      __nv_bfloat16(*G1l)[SH::PH] = sm.f.a2l();
      __nv_bfloat16(*G1l2)[SH::PH] = sm.f.a2l2();
      {  // 3. G1 = (G2 W1) * (1 - A1^2)
        const int t0 = warp * SH::TPWH, mt = t0 / SH::NTH, nt0 = t0 % SH::NTH;
        float acc[SH::TPWH][4];
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        warp_tile_gemm_bt3<H, SH::TPWH>(acc, &sm.G2[mt * 16][0], &sm.G2l[mt * 16][0],
                                        &sm.G2l2[mt * 16][0], SH::PH, &sm.f.W1[0][0], SH::PH,
                                        nt0 * 8, lane);
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++)
#pragma unroll
          for (int hr = 0; hr < 2; hr++) {
            const int row = mt * 16 + g + hr * 8, col = (nt0 + j) * 8 + 2 * c;
            const float a0 = __bfloat162float(sm.f.A1[row][col]) +
                             __bfloat162float(sm.f.A1l[row][col]) +
                             __bfloat162float(sm.f.A1l2[row][col]);
            const float a1 = __bfloat162float(sm.f.A1[row][col + 1]) +
                             __bfloat162float(sm.f.A1l[row][col + 1]) +
                             __bfloat162float(sm.f.A1l2[row][col + 1]);
            const float v0 = acc[j][2 * hr] * (1.f - a0 * a0);
            const float v1 = acc[j][2 * hr + 1] * (1.f - a1 * a1);
            store_split3x2(v0, v1, &G1[row][col], &G1l[row][col], &G1l2[row][col]);
            if (v0 != 0.f) atomicAdd(&sm.db0[col], v0);
            if (v1 != 0.f) atomicAdd(&sm.db0[col + 1], v1);
          }
      }
      {
        const __nv_bfloat16 *const A1p[3] = {&sm.f.A1[0][0], &sm.f.A1l[0][0],
                                             &sm.f.A1l2[0][0]};
        dw_tiles<SH, H, H>(G2p, SH::PH, A1p, SH::PH, SH::OW1, psum, pcomp, warp, lane);
      }
      __syncthreads();
      {  // 4. gY = G1 W0 (+ Gs Ws), owned layout
        const int t0 = warp * SH::TPW, mt = t0 / SH::NT, nt0 = t0 % SH::NT;
        float acc[SH::TPW][4];
#pragma unroll
        for (int j = 0; j < SH::TPW; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        warp_tile_gemm_bt3<H, SH::TPW>(acc, &G1[mt * 16][0], &G1l[mt * 16][0],
                                       &G1l2[mt * 16][0], SH::PH, &sm.f.W0[0][0], SH::PW0,
                                       nt0 * 8, lane);
        if constexpr (SDE)
          warp_tile_gemm_bt3<D, SH::TPW>(acc, &sm.Gs[mt * 16][0], &sm.Gsl[mt * 16][0],
                                         &sm.Gsl2[mt * 16][0], SH::PD, &sm.f.Ws[0][0], SH::PD,
                                         nt0 * 8, lane);
#pragma unroll
        for (int e = 0; e < NE; e++) gY[e] = acc[e >> 2][e & 3];
      }
      const __nv_bfloat16 *const Xp[3] = {&sm.f.X[0][0], &sm.f.Xl[0][0], &sm.f.Xl2[0][0]};
      {
        const __nv_bfloat16 *const G1p[3] = {&G1[0][0], &G1l[0][0], &G1l2[0][0]};
        dw_tiles<SH, H, D>(G1p, SH::PH, Xp, SH::PD, SH::OW0, psum, pcomp, warp, lane);
      }
      if constexpr (SDE) {
        const __nv_bfloat16 *const Gsp[3] = {&sm.Gs[0][0], &sm.Gsl[0][0], &sm.Gsl2[0][0]};
        dw_tiles<SH, D, D>(Gsp, SH::PD, Xp, SH::PD, SH::OWS, psum, pcomp, warp, lane);
      }
    }
  }
};

// Row set-up for the backward of trajectory i.
template <class SH>
__device__ void bwd_row_init(BwdRows<SH::M> &R, int r, int64_t i, const SolveParams &P) {
  const int N = P.tape_n[i];
  const int s = P.tape_stride[i];
  const int64_t ti = i * P.time_stride;
  const int dir = (P.t0[ti] < P.t1[ti]) ? 1 : -1;
  R.idx[r] = i;
  R.dir[r] = dir;
  R.N[r] = N;
  R.s[r] = s;
  R.active[r] = 1;
  R.fin[r] = 0;
  R.wt[r] = __longlong_as_double(0x7ff8000000000000LL);  // no carried W
  // number of ts saved: those <= t_N (all of them unless max_steps stopped it)
  const double tN = *GBDX_AT(P, P.tape_t, i * (P.max_steps + 1) + N, 1,
                             P.batch * (P.max_steps + 1), GBDX_SITE_TAPE_T);
  int k = 0;
  while (k < P.n_ts && dir * P.save_ts[k] <= tN) k++;
  R.k_hi[r] = k;
  R.k_lo[r] = k;
  if (N == 0) {
    R.n[r] = -1;
    R.mode[r] = kModeBwd;
    R.ld_kind[r] = kLoadNone;
  } else {
    const int n = N - 1;
    R.n[r] = n;
    if (n % s == 0) {
      R.mode[r] = kModeBwd;
      R.cs[r] = n;
      R.ld_kind[r] = kLoadCheckpoint;
      R.ld_slot[r] = n / s;
    } else {
      const int cs = (n / s) * s;
      R.cs[r] = cs;
      R.m[r] = cs;
      R.mode[r] = kModeFwd;
      R.ld_kind[r] = kLoadCheckpoint;
      R.ld_slot[r] = cs / s;
    }
  }
}

template <int SOLVER, int D, int H, bool PRECISE, bool SDE>
__global__ void __launch_bounds__(256) mlp_bwd_kernel(SolveParams P, BwdParams Q) {
  using SH = MlpShape<D, H>;
  using FLD = MlpField<SH, PRECISE, SDE>;
  using VJP = MlpVjp<SH, PRECISE, SDE>;
  using Sm = typename VJP::Sm;
  using TB = Tab<SOLVER>;
  constexpr int S = TB::S, NE = SH::NE, M = SH::M;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Sm &sm = *reinterpret_cast<Sm *>(smem_raw);
  BwdRows<M> &R = sm.rows;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float *W = P.mlp;
  float *psum = Q.part_sum + size_t(blockIdx.x) * Q.n_params;
  float *pcomp = Q.part_comp + size_t(blockIdx.x) * Q.n_params;
  const int n_save = P.n_save;

  FLD::stage(sm.f, P, tid);
  for (int i = tid; i < H; i += SH::THREADS) sm.db0[i] = sm.db1[i] = 0.f;
  for (int i = tid; i < D; i += SH::THREADS) sm.db2[i] = sm.dbs[i] = 0.f;
  if (tid < M) {
    const unsigned long long q = atomicAdd(P.queue, 1ull);
    if (q < (unsigned long long)P.batch) {
      bwd_row_init<SH>(R, tid, P.order ? (int64_t)P.order[q] : (int64_t)q, P);
      R.loaded[tid] = 1;
    } else {
      R.active[tid] = 0;
      R.loaded[tid] = 0;
      R.ld_kind[tid] = kLoadNone;
    }
  }
  __syncthreads();

  float Y[NE], GY[NE];
  // Newly loaded rows: the cotangent of the final state (the t1 save and,
  // when t0 == t1, every ts save), and y at the step the row starts from.
  auto load_rows = [&]() {
#pragma unroll
    for (int e = 0; e < NE; e++) {
      int row, col;
      elem_rc<SH>(e, warp, lane, row, col);
      if (R.loaded[row]) {
        const int64_t i = R.idx[row];
        const float *gys = Q.grad_ys + i * n_save * D + col;
        float g = 0.f;
        int slot = (P.save_t0 ? 1 : 0) + R.k_hi[row];
        if (R.N[row] == 0) {
          for (int m2 = 0; m2 < P.n_ts; m2++)
            g += *GBDX_AT(P, gys, (slot + m2) * D, 1, (n_save - 1) * D + 1, GBDX_SITE_GRAD_YS);
          slot += P.n_ts;
        }
        if (P.save_t1)
          g += *GBDX_AT(P, gys, slot * D, 1, (n_save - 1) * D + 1, GBDX_SITE_GRAD_YS);
        GY[e] = g;
        Y[e] = 0.f;
      }
      if (R.ld_kind[row] == kLoadCheckpoint)
        Y[e] = *GBDX_AT(P, P.tape_y, (R.idx[row] * P.checkpoints + R.ld_slot[row]) * D + col, 1,
                        P.batch * P.checkpoints * D, GBDX_SITE_TAPE_Y);
      else if (R.ld_kind[row] == kLoadScratch)
        Y[e] = *GBDX_AT(P, Q.scratch, (R.idx[row] * Q.seg_max + R.ld_slot[row]) * D + col, 1,
                        P.batch * Q.seg_max * D, GBDX_SITE_SCRATCH);
    }
  };
#pragma unroll
  for (int e = 0; e < NE; e++) Y[e] = GY[e] = 0.f;
  load_rows();
  __syncthreads();
  if (tid < M) {
    R.loaded[tid] = 0;
    R.ld_kind[tid] = kLoadNone;
  }

  float K[S][NE], F[NE], sig[NE], dW[NE];
  float Wc[SDE ? NE : 1];  // the carried Brownian values of the owned elements
#pragma unroll
  for (int e = 0; e < (SDE ? NE : 1); e++) Wc[e] = 0.f;
  VbtQuadCache vc;  // this lane's tree path (SDE)
  vc.traj = -1;
  vc.node = 0;
  while (true) {
    // ---- A. row set-up: the step this row works on -----------------------
    if (tid < M) {
      R.h[tid] = 0.f;
      R.fin[tid] = 0;
      R.live[tid] = 0;
      if (R.active[tid] && (R.mode[tid] == kModeFwd || R.n[tid] >= 0)) {
        R.live[tid] = 1;
        const int j = R.mode[tid] == kModeBwd ? R.n[tid] : R.m[tid];
        const double *tt = GBDX_AT(P, P.tape_t, R.idx[tid] * (P.max_steps + 1) + j, 2,
                                   P.batch * (P.max_steps + 1), GBDX_SITE_TAPE_T) - j;
        R.t_lo[tid] = tt[j];
        R.t_hi[tid] = tt[j + 1];
        const double dt = tt[j + 1] - tt[j];
        R.h[tid] = float(R.dir[tid] > 0 ? dt : -dt);
        if (R.mode[tid] == kModeBwd) {
          int k = R.k_hi[tid];
          while (k > 0 && (j == 0 || R.dir[tid] * P.save_ts[k - 1] > tt[j])) k--;
          R.k_lo[tid] = k;
        } else {
          R.k_lo[tid] = R.k_hi[tid];
        }
      }
      if constexpr (SDE) {
        R.w_lo[tid] = R.live[tid] && !(R.wt[tid] == R.t_lo[tid]);
        R.w_hi[tid] = R.live[tid] && !(R.wt[tid] == R.t_hi[tid]);
      }
    }
    __syncthreads();
    float hrow[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) {
      int row, col;
      elem_rc<SH>(e, warp, lane, row, col);
      hrow[e] = R.h[row];
    }
    if constexpr (SDE) {
      // W at both ends of the step.  A row's consecutive iterations share an
      // end (a recompute step's t_hi is the next one's t_lo; a backpropagated
      // step's t_lo is the previous step's t_hi), whose value its threads
      // carry: W(t) is a function of (seed, trajectory, t), so the carried
      // value is the one a fresh evaluation gives.  The other ends come from
      // the lane's cached tree path (consecutive evaluations lie within a
      // step or two).
      float wa[NE], wb[NE];
      vbt_owned<SH>(P, R, R.w_lo, R.t_lo, vc, wa, warp, lane);
      vbt_owned<SH>(P, R, R.w_hi, R.t_hi, vc, wb, warp, lane);
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        if (R.live[row]) {
          if (!R.w_lo[row]) wa[e] = Wc[e];
          if (!R.w_hi[row]) wb[e] = Wc[e];
          Wc[e] = R.mode[row] == kModeFwd ? wb[e] : wa[e];
        }
        dW[e] = wb[e] - wa[e];
      }
      if (tid < M && R.live[tid]) R.wt[tid] = R.mode[tid] == kModeFwd ? R.t_hi[tid] : R.t_lo[tid];
    }
    // ---- B. forward stages of the step ----------------------------------
    float Yi[NE];
#pragma unroll
    for (int i = 0; i < S; i++) {
#pragma unroll
      for (int e = 0; e < NE; e++) {
        float a = Y[e];
#pragma unroll
        for (int j = 0; j < i; j++)
          if (TB::a(i, j) != 0.0) a = fmaf(float(TB::a(i, j)), K[j][e], a);
        Yi[e] = a;
      }
      __syncthreads();
      FLD::put_x(sm.f, Yi, warp, lane);
      __syncthreads();
      FLD::eval(sm.f, W, F, sig, tid, warp, lane);
#pragma unroll
      for (int e = 0; e < NE; e++)
        K[i][e] = SDE ? F[e] * hrow[e] + sig[e] * dW[e] : F[e] * hrow[e];
    }
    float Y1[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) {
      if constexpr (TB::SSAL) {
        Y1[e] = Yi[e];
      } else {
        float a = Y[e];
#pragma unroll
        for (int j = 0; j < S; j++) a = fmaf(float(TB::b(j)), K[j][e], a);
        Y1[e] = a;
      }
    }
    // ---- C. FWD rows: store the recomputed state -------------------------
    // ---- D. BWD rows: cotangents of the saves inside the step ------------
    float KB[S][NE], GY0[NE], GY1[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) {
      int row, col;
      elem_rc<SH>(e, warp, lane, row, col);
#pragma unroll
      for (int j = 0; j < S; j++) KB[j][e] = 0.f;
      GY0[e] = 0.f;
      GY1[e] = 0.f;
      if (R.live[row] && R.mode[row] == kModeFwd) {
        *GBDX_AT(P, Q.scratch, (R.idx[row] * Q.seg_max + (R.m[row] - R.cs[row])) * D + col, 1,
                 P.batch * Q.seg_max * D, GBDX_SITE_SCRATCH) = Y1[e];
      } else if (R.live[row]) {
        GY1[e] = GY[e];
      }
    }
    while (true) {
      int fl = 0;
      if (tid < M) {
        R.sflag[tid] = 0;
        if (R.live[tid] && R.mode[tid] == kModeBwd && R.k_lo[tid] < R.k_hi[tid]) {
          const int k = R.k_hi[tid] - 1;
          const double tsd = R.dir[tid] * P.save_ts[k];
          const double tp = R.t_lo[tid], tn = R.t_hi[tid];
          R.theta[tid] = float(tp == tn ? 0.0 : (tsd - tp) / (tn - tp));
          R.sslot[tid] = (P.save_t0 ? 1 : 0) + k;
          R.k_hi[tid] = k;
          R.sflag[tid] = 1;
          fl = 1;
        }
      }
      if (!__syncthreads_or(fl)) break;
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        if (R.sflag[row]) {
          const float gb = *GBDX_AT(P, Q.grad_ys, (R.idx[row] * n_save + R.sslot[row]) * D + col,
                                    1, P.batch * n_save * D, GBDX_SITE_GRAD_YS);
          float ay0, ay1, gg[7];
          interp_coeffs<SOLVER>(R.theta[row], ay0, ay1, gg);
          GY0[e] = fmaf(ay0, gb, GY0[e]);
          GY1[e] = fmaf(ay1, gb, GY1[e]);
#pragma unroll
          for (int j = 0; j < S; j++) KB[j][e] = fmaf(gg[j], gb, KB[j][e]);
        }
      }
      __syncthreads();
    }
    // y1 = last stage input (SSAL) or y0 + sum b_j k_j
    float YB[NE];  // cotangent of the current stage input
#pragma unroll
    for (int e = 0; e < NE; e++) {
      if constexpr (TB::SSAL) {
        YB[e] = GY1[e];
      } else {
        GY0[e] += GY1[e];
#pragma unroll
        for (int j = 0; j < S; j++) KB[j][e] = fmaf(float(TB::b(j)), GY1[e], KB[j][e]);
        YB[e] = 0.f;
      }
    }
    // ---- E. reverse stage loop -------------------------------------------
#pragma unroll
    for (int i = S - 1; i >= 0; i--) {
#pragma unroll
      for (int e = 0; e < NE; e++) {
        float a = Y[e];
#pragma unroll
        for (int j = 0; j < i; j++)
          if (TB::a(i, j) != 0.0) a = fmaf(float(TB::a(i, j)), K[j][e], a);
        Yi[e] = a;
      }
      __syncthreads();
      FLD::put_x(sm.f, Yi, warp, lane);
      __syncthreads();
      FLD::eval(sm.f, W, F, sig, tid, warp, lane);  // recompute A1, A2 (and sigma)
      float G3r[NE], Gsr[NE], gY[NE];
#pragma unroll
      for (int e = 0; e < NE; e++) {
        G3r[e] = KB[i][e] * hrow[e];
        Gsr[e] = SDE ? KB[i][e] * dW[e] : 0.f;
      }
      __syncthreads();
      VJP::run(sm, W, G3r, Gsr, sig, gY, psum, pcomp, tid, warp, lane);
#pragma unroll
      for (int e = 0; e < NE; e++) {
        const float gyi = gY[e] + (i == S - 1 ? YB[e] : 0.f);
        GY0[e] += gyi;
#pragma unroll
        for (int j = 0; j < i; j++)
          if (TB::a(i, j) != 0.0) KB[j][e] = fmaf(float(TB::a(i, j)), gyi, KB[j][e]);
      }
    }
    __syncthreads();
    // flush this iteration's bias gradients into the CTA partials
    for (int i = tid; i < H; i += SH::THREADS) {
      kahan_add(psum + SH::OB0 + i, pcomp + SH::OB0 + i, sm.db0[i]);
      kahan_add(psum + SH::OB1 + i, pcomp + SH::OB1 + i, sm.db1[i]);
      sm.db0[i] = sm.db1[i] = 0.f;
    }
    for (int i = tid; i < D; i += SH::THREADS) {
      kahan_add(psum + SH::OB2 + i, pcomp + SH::OB2 + i, sm.db2[i]);
      sm.db2[i] = 0.f;
      if (SDE) {
        kahan_add(psum + SH::OBS + i, pcomp + SH::OBS + i, sm.dbs[i]);
        sm.dbs[i] = 0.f;
      }
    }
    // ---- F. advance the rows ---------------------------------------------
#pragma unroll
    for (int e = 0; e < NE; e++) {
      int row, col;
      elem_rc<SH>(e, warp, lane, row, col);
      if (R.live[row]) {
        if (R.mode[row] == kModeFwd)
          Y[e] = Y1[e];
        else
          GY[e] = GY0[e];
      }
    }
    __syncthreads();
    int fin = 0;
    if (tid < M) {
      R.ld_kind[tid] = kLoadNone;
      if (R.active[tid]) {
        if (R.mode[tid] == kModeFwd) {
          R.m[tid]++;
          if (R.m[tid] == R.n[tid]) R.mode[tid] = kModeBwd;
        } else {
          const int n = R.n[tid] - 1;
          R.n[tid] = n;
          const int s = R.s[tid];
          if (n < 0) {
            R.fin[tid] = 1;
            fin = 1;
          } else if (n % s == 0) {
            R.ld_kind[tid] = kLoadCheckpoint;
            R.ld_slot[tid] = n / s;
            R.cs[tid] = n;
          } else if (n > R.cs[tid]) {
            R.ld_kind[tid] = kLoadScratch;
            R.ld_slot[tid] = n - R.cs[tid] - 1;
          } else {
            const int cs = (n / s) * s;
            R.cs[tid] = cs;
            R.m[tid] = cs;
            R.mode[tid] = kModeFwd;
            R.ld_kind[tid] = kLoadCheckpoint;
            R.ld_slot[tid] = cs / s;
          }
        }
      }
    }
    if (__syncthreads_or(fin)) {
      // finished rows: dL/dy0 (plus the t0 save's cotangent)
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        if (R.fin[row]) {
          const int64_t i = R.idx[row];
          float g = GY[e];
          if (P.save_t0) g += Q.grad_ys[(i * n_save) * D + col];
          Q.grad_y0[i * D + col] = g;
        }
      }
      __syncthreads();
      if (tid < M && R.fin[tid]) {
        const unsigned long long q = atomicAdd(P.queue, 1ull);
        if (q < (unsigned long long)P.batch) {
          bwd_row_init<SH>(R, tid, P.order ? (int64_t)P.order[q] : (int64_t)q, P);
          R.loaded[tid] = 1;
        } else {
          R.active[tid] = 0;
        }
      }
    }
    __syncthreads();
    load_rows();
    __syncthreads();
    if (tid < M) R.loaded[tid] = 0;
    if (!__syncthreads_or(tid < M && R.active[tid])) break;
  }
}

}  // namespace gbdx
