// gbdx_mlp.cuh -- fused integrator for MLP vector fields (neural ODEs/SDEs).
//
// One CTA of 8 warps integrates a tile of M trajectories ("rows") in lockstep;
// rows finish independently and are refilled from the work counter.  Per RK
// stage the tile evaluates the field as a chain of tensor-core products,
//   F = W2 tanh(W1 tanh(W0 Y + b0) + b1) + b2        (eqx.nn.MLP semantics)
// with the weights resident in shared memory as BF16 and FP32 accumulation.
// The weights are the model's BF16 values (FP32 inputs are rounded to BF16);
// the operands they multiply -- stage inputs, hidden activations -- are held
// as sums of three BF16 pieces (24 significant bits), so every product is
// exact up to the FP32 accumulation and the field is as accurate as an FP32
// evaluation with the same weights.
// The RK state of every (row, component) -- y, the stage increments k_i, the
// FSAL vector and the error estimate -- lives in registers in the layout of
// the last product's accumulator fragments, so all stage arithmetic is
// register-local.  Per-row scalars (FP64 t and dt, PID history, counters) live
// in shared memory and are advanced by one thread per row.
//
// Semantics follow the analytic-field kernels (gbdx_traj.cuh), which in turn
// follow diffrax/_integrate.py:302-885 and the files cited there.  The SDE
// variant is Heun/Euler on MultiTerm(ODETerm(MLP), ControlTerm(diag
// 0.1 tanh(Ws y + bs), VirtualBrownianTree)) (_term.py:666-731, 271-555,
// _brownian/tree.py:325-354, 366-448, 607-621, 752-768).
#pragma once

#include <cuda_bf16.h>

#include "gbdx_common.cuh"
#include "gbdx_mma.cuh"
#include "gbdx_traj.cuh"
#include "gbdx_vbt.cuh"

namespace gbdx {

template <int D_, int H_>
struct MlpShape {
  static constexpr int D = D_, H = H_;
  static constexpr int M = (H_ >= 256) ? 16 : 32;  // rows per CTA
  static constexpr int THREADS = 256, WARPS = 8;
  // Width 256: W0 and W2 are read as pre-arranged BF16 mma B fragments from
  // global memory (L2-resident, 32 KB each), so that W1 and the three-piece
  // activations fit the 227 KB of shared memory.
  static constexpr bool GFRAG = H_ >= 256;
  static constexpr int PD = D + 8, PH = H + 8;      // padded smem row strides (bf16)
  static constexpr int PW0 = D + 8;                 // row stride of W0
  static constexpr int MT = M / 16, NT = D / 8, NTH = H / 8;
  static constexpr int TPW = MT * NT / WARPS;       // output tiles per warp
  static constexpr int TPWH = MT * NTH / WARPS;     // hidden tiles per warp
  static constexpr int NE = 4 * TPW;                // owned elements per thread
  // BF16 pieces of each activation operand (24 significant bits)
  static constexpr int NP = 3;
  static_assert(MT * NT % WARPS == 0 && TPW >= 1, "tile split");
  static_assert(MT * NTH % WARPS == 0 && NTH % TPWH == 0, "hidden tile split");
  static_assert(NT % TPW == 0, "output tile split");
  static_assert(NT <= 8, "error-norm partials: at most 8 column tiles");
  // flat parameter offsets (FP32, row-major [out][in])
  static constexpr int OW0 = 0, OB0 = OW0 + H * D, OW1 = OB0 + H, OB1 = OW1 + H * H,
                       OW2 = OB1 + H, OB2 = OW2 + D * H, OWS = OB2 + D, OBS = OWS + D * D;
};

template <int M>
struct RowState {
  double tprev[M], tnext[M], t1[M], floor1[M], dtc[M], tp_old[M], tn_old[M], t0s[M], t1s[M];
  long long idx[M];
  float h[M], hist1[M], hist2[M], acc[M], theta[M];
  int active[M], first[M], keep[M], anynan[M], dir[M], save_index[M], ts_index[M];
  int nsteps[M], nacc[M], nrej[M], result[M], sflag[M], sslot[M], fin[M], nfill[M];
  int loaded[M], sc[M], nc[M], cpstride[M], cpslot[M], cpcompact[M], at_dtmin[M], live[M];
  double ginv[M];  // RN(1 / nc), for the grid fraction
  int sdown[M], stslot[M];  // SaveAt(steps=n): steps to the next save; this step's slot
  int sidx[M], jidx[M];     // ClipStepSizeController: search hints into step_ts / jump_ts
  // the error norm's partial sums per 8-column output tile, added in a fixed
  // order (results do not depend on warp timing)
  float part[M][8];
};

// Events (registered conditions) of the extended-output integrator, in the
// dynamic shared memory after the kernel's own: the conditions' last values,
// the one that fired (-1: none), the event time, the latest time a save may
// take (the event time once a root was found), the root's theta in its step
// (-1: no root); components 0..3 of y0, y1 and the stage increments for the
// root find; the steady-state norms' per-tile partials (f.f, y.y).
template <int M>
struct RowEvents {
  double evv[M][GBDX_MAX_EVENTS], tfin[M], tsave[M];
  int evi[M];
  float thfin[M];
  float ey0[M][4], ey1[M][4], ek[M][7][4];
  float pf[M][8], py[M][8];
};

template <class SH, bool PRECISE, bool SDE>
struct MlpSmem;

template <class SH, bool SDE>
struct MlpSmem<SH, false, SDE> {
  static constexpr int M3 = SH::NP == 3 ? SH::M : 1;
  __nv_bfloat16 W0[SH::GFRAG ? 1 : SH::H][SH::PW0];  // (global fragments at width 256)
  __nv_bfloat16 W1[SH::H][SH::PH];
  __nv_bfloat16 W2[SH::GFRAG ? 1 : SH::D][SH::PH];
  const uint2 *w0f, *w2f;                            // the fragments (width 256)
  __nv_bfloat16 Ws[SDE ? SH::D : 1][SH::PD];
  float b0[SH::H], b1[SH::H], b2[SH::D], bs[SH::D];
  // stage input and hidden activations as BF16 pieces (the third piece only
  // with NP == 3)
  __nv_bfloat16 X[SH::M][SH::PD], Xl[SH::M][SH::PD], Xl2[M3][SH::PD];
  __nv_bfloat16 A1[SH::M][SH::PH], A1l[SH::M][SH::PH], A1l2[M3][SH::PH];
  __nv_bfloat16 A2s[SH::M][SH::PH], A2ls[SH::M][SH::PH], A2l2s[M3][SH::PH];
  RowState<SH::M> rows;
  __device__ __nv_bfloat16 (*a2())[SH::PH] { return A2s; }
  __device__ __nv_bfloat16 (*a2l())[SH::PH] { return A2ls; }
  __device__ __nv_bfloat16 (*a2l2())[SH::PH] { return A2l2s; }
  // the third pieces' rows (null with two pieces)
  __device__ __nv_bfloat16 *xl2(int r) { return SH::NP == 3 ? &Xl2[r][0] : nullptr; }
  __device__ __nv_bfloat16 *a1l2(int r) { return SH::NP == 3 ? &A1l2[r][0] : nullptr; }
  __device__ __nv_bfloat16 *a2l2r(int r) { return SH::NP == 3 ? &a2l2()[r][0] : nullptr; }
};

template <class SH, bool SDE>
struct MlpSmem<SH, true, SDE> {
  float b0[SH::H], b1[SH::H], b2[SH::D], bs[SH::D];
  float X[SH::M][SH::D + 1];
  float A1[SH::M][SH::H + 1];
  float A2[SH::M][SH::H + 1];
  RowState<SH::M> rows;
};

// (row, col) of owned element e of this thread in the output-tile layout.
template <class SH>
__device__ __forceinline__ void elem_rc(int e, int warp, int lane, int &row, int &col) {
  const int j = e >> 2, q = e & 3;
  const int t = warp * SH::TPW + j;
  const int mt = t / SH::NT, nt = t % SH::NT;
  row = mt * 16 + (lane >> 2) + ((q >> 1) << 3);
  col = nt * 8 + 2 * (lane & 3) + (q & 1);
}

template <class SH, bool PRECISE, bool SDE>
struct MlpField {
  using Sm = MlpSmem<SH, PRECISE, SDE>;
  static constexpr int D = SH::D, H = SH::H, M = SH::M, NE = SH::NE;

  // Stage the weights (BF16 mode) and biases into shared memory (at width 256
  // only W1: W0 and W2 are the global fragments S.w0f, S.w2f).
  __device__ static void stage(Sm &sm, const SolveParams &S, int tid) {
    const float *P = S.mlp;
    for (int i = tid; i < H; i += SH::THREADS) {
      sm.b0[i] = P[SH::OB0 + i];
      sm.b1[i] = P[SH::OB1 + i];
    }
    for (int i = tid; i < D; i += SH::THREADS) {
      sm.b2[i] = P[SH::OB2 + i];
      if (SDE) sm.bs[i] = P[SH::OBS + i];
    }
    if constexpr (!PRECISE) {
      // the model's BF16 weights
      if constexpr (SH::GFRAG) {
        if (tid == 0) {
          sm.w0f = S.w0f;
          sm.w2f = S.w2f;
        }
      } else {
        for (int i = tid; i < H * D; i += SH::THREADS)
          sm.W0[i / D][i % D] = __float2bfloat16_rn(P[SH::OW0 + i]);
        for (int i = tid; i < D * H; i += SH::THREADS)
          sm.W2[i / H][i % H] = __float2bfloat16_rn(P[SH::OW2 + i]);
      }
      for (int i = tid; i < H * H; i += SH::THREADS)
        sm.W1[i / H][i % H] = __float2bfloat16_rn(P[SH::OW1 + i]);
      if constexpr (SDE)
        for (int i = tid; i < D * D; i += SH::THREADS)
          sm.Ws[i / D][i % D] = __float2bfloat16_rn(P[SH::OWS + i]);
    }
  }

  // Write the stage input Y (owned elements) as the first product's operand.
  __device__ static void put_x(Sm &sm, const float (&Y)[NE], int warp, int lane) {
#pragma unroll
    for (int e = 0; e < NE; e += 2) {
      int row, col;
      elem_rc<SH>(e, warp, lane, row, col);
      if constexpr (PRECISE) {
        sm.X[row][col] = Y[e];
        sm.X[row][col + 1] = Y[e + 1];
      } else {
        __nv_bfloat16 *x2 = sm.xl2(row);
        store_split3x2(Y[e], Y[e + 1], &sm.X[row][col], &sm.Xl[row][col],
                       x2 ? x2 + col : nullptr);
      }
    }
  }

  // acc += (A0 + A1 [+ A2])[rows, K] W[n, K]^T: one BF16 tensor-core product
  // per activation piece against the BF16 weights.
  template <int K, int NTW>
  __device__ static __forceinline__ void split_gemm(float (&acc)[NTW][4], const __nv_bfloat16 *A0,
                                                    const __nv_bfloat16 *A1,
                                                    const __nv_bfloat16 *A2, int lda,
                                                    const __nv_bfloat16 *W, int ldw, int lane) {
    warp_tile_gemm_p<K, NTW, SH::NP>(acc, A0, A1, A2, lda, W, ldw, lane);
  }

  // F = MLP(X) and (SDE) sigma = 0.1 tanh(Ws X + bs), both in the owned layout.
  // X must have been written and synchronised.  Ends synchronised so that X,
  // A1 and A2 may be rewritten by the caller after its next barrier.
  __device__ static void eval(Sm &sm, const float *P, float (&F)[NE], float (&sig)[NE],
                              int tid, int warp, int lane) {
    if constexpr (PRECISE) {
      const float *W0 = P + SH::OW0, *W1 = P + SH::OW1, *W2 = P + SH::OW2, *Ws = P + SH::OWS;
      for (int i = tid; i < M * H; i += SH::THREADS) {
        const int r = i / H, n = i % H;
        float a = sm.b0[n];
        for (int k = 0; k < D; k++) a = fmaf(sm.X[r][k], __ldg(W0 + n * D + k), a);
        sm.A1[r][n] = tanhf(a);
      }
      if constexpr (SDE) {
#pragma unroll
        for (int e = 0; e < NE; e++) {
          int row, col;
          elem_rc<SH>(e, warp, lane, row, col);
          float a = sm.bs[col];
          for (int k = 0; k < D; k++) a = fmaf(sm.X[row][k], __ldg(Ws + col * D + k), a);
          sig[e] = 0.1f * tanhf(a);
        }
      }
      __syncthreads();
      for (int i = tid; i < M * H; i += SH::THREADS) {
        const int r = i / H, n = i % H;
        float a = sm.b1[n];
        for (int k = 0; k < H; k++) a = fmaf(sm.A1[r][k], __ldg(W1 + n * H + k), a);
        sm.A2[r][n] = tanhf(a);
      }
      __syncthreads();
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        float a = sm.b2[col];
        for (int k = 0; k < H; k++) a = fmaf(sm.A2[row][k], __ldg(W2 + col * H + k), a);
        F[e] = a;
      }
    } else {
      const int g = lane >> 2, c = lane & 3;
      {  // layer 0: A1 = tanh(X W0^T + b0)
        const int t0 = warp * SH::TPWH, mt = t0 / SH::NTH, nt0 = t0 % SH::NTH;
        float acc[SH::TPWH][4];
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        if constexpr (SH::GFRAG)
          gemm_gfrag_p<D, SH::TPWH, SH::NP>(acc, &sm.X[mt * 16][0], &sm.Xl[mt * 16][0],
                                            sm.xl2(mt * 16), SH::PD, sm.w0f, nt0, lane);
        else
          split_gemm<D, SH::TPWH>(acc, &sm.X[mt * 16][0], &sm.Xl[mt * 16][0], sm.xl2(mt * 16),
                                  SH::PD, &sm.W0[nt0 * 8][0], SH::PW0, lane);
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) {
          const int col = (nt0 + j) * 8 + 2 * c, r0 = mt * 16 + g;
          const float bb0 = sm.b0[col], bb1 = sm.b0[col + 1];
          __nv_bfloat16 *p2a = sm.a1l2(r0), *p2b = sm.a1l2(r0 + 8);
          store_split3x2(tanhf(acc[j][0] + bb0), tanhf(acc[j][1] + bb1), &sm.A1[r0][col],
                         &sm.A1l[r0][col], p2a ? p2a + col : nullptr);
          store_split3x2(tanhf(acc[j][2] + bb0), tanhf(acc[j][3] + bb1), &sm.A1[r0 + 8][col],
                         &sm.A1l[r0 + 8][col], p2b ? p2b + col : nullptr);
        }
      }
      if constexpr (SDE) {  // diffusion product on the same operand
        const int t0 = warp * SH::TPW, mt = t0 / SH::NT, nt0 = t0 % SH::NT;
        float acc[SH::TPW][4];
#pragma unroll
        for (int j = 0; j < SH::TPW; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        split_gemm<D, SH::TPW>(acc, &sm.X[mt * 16][0], &sm.Xl[mt * 16][0], sm.xl2(mt * 16),
                               SH::PD, &sm.Ws[nt0 * 8][0], SH::PD, lane);
#pragma unroll
        for (int e = 0; e < NE; e++) {
          int row, col;
          elem_rc<SH>(e, warp, lane, row, col);
          sig[e] = 0.1f * tanhf(acc[e >> 2][e & 3] + sm.bs[col]);
        }
      }
      __syncthreads();
      {  // layer 1: A2 = tanh(A1 W1^T + b1)
        const int t0 = warp * SH::TPWH, mt = t0 / SH::NTH, nt0 = t0 % SH::NTH;
        float acc[SH::TPWH][4];
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        split_gemm<H, SH::TPWH>(acc, &sm.A1[mt * 16][0], &sm.A1l[mt * 16][0], sm.a1l2(mt * 16),
                                SH::PH, &sm.W1[nt0 * 8][0], SH::PH, lane);
        auto A2 = sm.a2();
        auto A2l = sm.a2l();
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) {
          const int col = (nt0 + j) * 8 + 2 * c, r0 = mt * 16 + g;
          const float bb0 = sm.b1[col], bb1 = sm.b1[col + 1];
          __nv_bfloat16 *p2a = sm.a2l2r(r0), *p2b = sm.a2l2r(r0 + 8);
          store_split3x2(tanhf(acc[j][0] + bb0), tanhf(acc[j][1] + bb1), &A2[r0][col],
                         &A2l[r0][col], p2a ? p2a + col : nullptr);
          store_split3x2(tanhf(acc[j][2] + bb0), tanhf(acc[j][3] + bb1), &A2[r0 + 8][col],
                         &A2l[r0 + 8][col], p2b ? p2b + col : nullptr);
        }
      }
      __syncthreads();
      {  // layer 2: F = A2 W2^T + b2, straight into the owned layout
        const int t0 = warp * SH::TPW, mt = t0 / SH::NT, nt0 = t0 % SH::NT;
        float acc[SH::TPW][4];
#pragma unroll
        for (int j = 0; j < SH::TPW; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        if constexpr (SH::GFRAG)
          gemm_gfrag_p<H, SH::TPW, SH::NP>(acc, &sm.a2()[mt * 16][0], &sm.a2l()[mt * 16][0],
                                           sm.a2l2r(mt * 16), SH::PH, sm.w2f, nt0, lane);
        else
          split_gemm<H, SH::TPW>(acc, &sm.a2()[mt * 16][0], &sm.a2l()[mt * 16][0],
                                 sm.a2l2r(mt * 16), SH::PH, &sm.W2[nt0 * 8][0], SH::PH, lane);
#pragma unroll
        for (int e = 0; e < NE; e++) {
          int row, col;
          elem_rc<SH>(e, warp, lane, row, col);
          F[e] = acc[e >> 2][e & 3] + sm.b2[col];
        }
      }
    }
  }
};

// ---------------------------------------------------------------------------
// Per-row controller (one thread per row).  The FP32-state rules of
// Traj::step: log-domain PID, integer-key time comparisons, carried dt.
// ---------------------------------------------------------------------------
template <int M>
__device__ __forceinline__ bool row_running(const RowState<M> &R, int r, int max_steps) {
  return R.active[r] && order_key(R.tprev[r]) < order_key(R.t1[r]) &&
         R.result[r] == GBDX_SUCCESSFUL && R.nsteps[r] < max_steps;
}

template <int M, bool XO>
__device__ void row_init(RowState<M> &R, RowEvents<M> *EV, int r, int64_t i,
                         const SolveParams &P, int D, bool fsal) {
  const int64_t ti = i * P.time_stride;
  double a = P.t0[ti], b = P.t1[ti];
  const int dir = (a < b) ? 1 : -1;
  a *= dir;
  b *= dir;
  R.idx[r] = i;
  R.dir[r] = dir;
  R.t1[r] = b;
  double tn;
  if (P.controller == GBDX_PID) {
    double h = P.dt0 ? P.dt0[ti] * dir : 0.01;
    if (P.has_dtmax) h = fmin(h, P.dtmax);
    if (P.has_dtmin) h = fmax(h, P.dtmin);
    tn = a + h;
    if constexpr (XO) {
      if (P.n_step_ts > 0 || P.n_jump_ts > 0)
        tn = clip_start(P, dir, R.sidx[r], R.jidx[r], a, tn);
    }
    R.hist1[r] = 0.f;
    R.hist2[r] = 0.f;
  } else {
    const double h = P.dt0[ti] * dir;
    R.sc[r] = 1;
    R.nc[r] = (int)ceil((b - a) / next_up(h));
    R.t0s[r] = a;
    R.t1s[r] = b;
    tn = a + h;
  }
  R.tnext[r] = fmin(tn, b);
  R.dtc[r] = R.tnext[r] - a;
  R.tprev[r] = a;
  R.floor1[r] = t1_clip_floor(b);
  R.first[r] = 1;
  R.save_index[r] = 0;
  R.ts_index[r] = 0;
  R.nsteps[r] = R.nacc[r] = R.nrej[r] = 0;
  R.result[r] = GBDX_SUCCESSFUL;
  R.active[r] = 1;
  R.cpstride[r] = 1;
  R.cpslot[r] = 0;
  R.cpcompact[r] = 0;
  R.at_dtmin[r] = 0;
  R.live[r] = 0;
  if constexpr (XO) {
    // a passed controller and solver state (the resume record of
    // gbdx_fwd_extras, _integrate.py:1252-1271, 1309): the PID history (held
    // here as log2) or the constant grid, and whether the FSAL value the
    // element pass loads replaces the first evaluation
    if (P.state_in) {
      const double *st =
          GBDX_AT(P, P.state_in, i * int64_t(GBDX_STATE_HEAD + D), GBDX_STATE_HEAD + D,
                  P.batch * (GBDX_STATE_HEAD + D), GBDX_SITE_STATE);
      if (st[4] != 0.0) {
        if (P.controller == GBDX_PID) {
          R.hist1[r] = float(log2(st[0]));
          R.hist2[r] = float(log2(st[1]));
          R.at_dtmin[r] = st[2] != 0.0;
          if (P.dt0) {  // the first step is t0 + dt0, unclipped by dtmin / dtmax
            R.tnext[r] = fmin(a + P.dt0[ti] * dir, b);
            R.dtc[r] = R.tnext[r] - a;
          }
        } else {
          R.sc[r] = int(st[0]);
          R.nc[r] = int(st[1]);
          R.t0s[r] = st[2];
          R.t1s[r] = st[3];
        }
      }
      if (fsal && st[5] == 0.0 && st[6] == 0.0) R.first[r] = 0;
    }
  }
  if (P.controller != GBDX_PID) R.ginv[r] = 1.0 / double(R.nc[r]);
  if (P.save_t0) {
    *GBDX_AT(P, P.ts_out, i * P.n_save, 1, P.batch * P.n_save, GBDX_SITE_TS) = a * dir;
    R.save_index[r] = 1;
  }
  if (P.tape_t)
    *GBDX_AT(P, P.tape_t, i * (P.max_steps + 1), 1, P.batch * (P.max_steps + 1),
             GBDX_SITE_TAPE_T) = a;
  if constexpr (!XO) return;
  R.sdown[r] = P.save_steps;
  R.stslot[r] = -1;
  EV->evi[r] = -1;
  EV->tfin[r] = a;
  EV->thfin[r] = -1.f;
  if (P.n_event > 0) {
    // values at (t0, y0) (_integrate.py:1333-1426): a boolean linear
    // condition that already holds ends the solve before its first step; a
    // steady-state condition is checked once f(y0) is known (the first step's
    // first stage)
    const float *y0 = static_cast<const float *>(P.y0) + i * D;
#pragma unroll
    for (int e = 0; e < GBDX_MAX_EVENTS; e++) {
      if (e < P.n_event) {
        double v = 0.0;
        if (P.ev_kind[e] != GBDX_EV_STEADY) {
          for (int n = 0; n < (D < 4 ? D : 4); n++)
            v += P.ev_coef[6 * e + n] * double(y0[n]);
          v += P.ev_coef[6 * e + 4] * a + P.ev_coef[6 * e + 5];
          if (P.ev_kind[e] == GBDX_EV_LINEAR_BOOL) v = v > 0 ? 1.0 : 0.0;
          if (EV->evi[r] < 0 && P.ev_kind[e] == GBDX_EV_LINEAR_BOOL && v != 0.0) EV->evi[r] = e;
        }
        EV->evv[r][e] = v;
      }
    }
    if (EV->evi[r] >= 0) R.result[r] = GBDX_EVENT_OCCURRED;
  }
  // dense_ts[0] = t0 in the loop's time; the rest of the dense buffers was
  // filled with +inf before the launch (_integrate.py:1315-1323)
  if (P.dense_ts)
    *GBDX_AT(P, P.dense_ts, i * (P.max_steps + 1), 1, P.batch * (P.max_steps + 1),
             GBDX_SITE_DENSE_TS) = a;
}

// The controller's decision for row r after the error norm acc = sum of
// squared scaled errors over the D components (pid.py:466-567,
// constant.py:59-104, _integrate.py:410-413).
template <int M, bool XO>
__device__ void row_control(RowState<M> &R, int r, int D, const SolveParams &P) {
  const double dt = R.dtc[r];
  bool keep;
  double nt0, nt1, dtn;
  if (P.controller == GBDX_PID) {
    const float acc = R.acc[r];
    keep = acc < float(D);
    const float lg = 0.5f * (log2f(float(D)) - __log2f(acc));
    float ex = 0.f;
    if (P.c1_f != 0.f) ex += P.c1_f * lg;
    if (P.c2_f != 0.f) ex += P.c2_f * R.hist1[r];
    if (P.c3_f != 0.f) ex += P.c3_f * R.hist2[r];
    float factor = P.safety_f * exp2f(ex);
    const float hnew = isinf(lg) ? 0.f : lg;
    if (P.has_dtmin) keep = keep || R.at_dtmin[r];
    const float fmn = keep ? 1.f : P.factormin_f;
    const float fmx = keep ? P.factormax_f : P.safety_f;
    factor = fminf(fmaxf(factor, fmn), fmx);
    dtn = dt * double(factor);
    if (P.has_dtmax) dtn = fmin(dtn, P.dtmax);
    if (P.has_dtmin) {
      if (!P.force_dtmin && dtn < P.dtmin && R.result[r] == GBDX_SUCCESSFUL)
        R.result[r] = GBDX_DT_MIN_REACHED;
      if (R.at_dtmin[r] && factor == 1.f) dtn = P.dtmin;
      R.at_dtmin[r] = dtn <= P.dtmin;
      dtn = fmax(dtn, P.dtmin);
    }
    nt0 = keep ? R.tnext[r] : R.tprev[r];
    nt1 = nt0 + dtn;
    if (keep) {
      R.hist2[r] = R.hist1[r];
      R.hist1[r] = hnew;
    }
  } else {
    keep = true;
    const int s2 = R.sc[r] + 1;
    double tn = grid_time(R.t0s[r], R.t1s[r], s2, R.nc[r], R.ginv[r]);
    if (s2 == R.nc[r]) tn = R.t1s[r];
    R.sc[r] = s2;
    nt0 = R.tnext[r];
    nt1 = tn;
    dtn = tn - nt0;
  }
  // ClipStepSizeController around the PID controller (clip.py:330-389)
  bool made_jump = false;
  if constexpr (XO) {
    if (P.controller == GBDX_PID && (P.n_step_ts > 0 || P.n_jump_ts > 0)) {
      made_jump = clip_next(P, R.dir[r], R.sidx[r], R.jidx[r], nt0, nt1);
      dtn = nt1 - nt0;
    }
  }
  if (order_key(nt1) > order_key(R.floor1[r])) {
    nt1 = keep ? R.t1[r] : nt0 + 0.5 * (R.t1[r] - nt0);
    dtn = nt1 - nt0;
  }
  R.keep[r] = keep;
  R.tp_old[r] = R.tprev[r];
  R.tn_old[r] = R.tnext[r];
  if (keep) {
    R.nacc[r]++;
    // after a jump the FSAL solvers evaluate the first stage afresh
    // (runge_kutta.py:684-700)
    R.first[r] = made_jump ? 1 : 0;
    if (P.tape_t)
      *GBDX_AT(P, P.tape_t, R.idx[r] * (P.max_steps + 1) + R.nacc[r], 1,
               P.batch * (P.max_steps + 1), GBDX_SITE_TAPE_T) = R.tnext[r];
    // Online thinning of the state checkpoints: every accepted step while the
    // slots last, then every 2nd, 4th, ... step.
    if (P.tape_y) {
      const int n = R.nacc[r];
      int stride = R.cpstride[r];
      int compact = 0;
      int slot = -1;
      if (n % stride == 0) {
        slot = n / stride;
        if (slot >= P.checkpoints) {
          compact = 1;
          stride *= 2;
          slot = n / stride;
        }
      }
      R.cpstride[r] = stride;
      R.cpslot[r] = slot;
      R.cpcompact[r] = compact;
    }
  } else {
    R.nrej[r]++;
    if (P.tape_y) R.cpslot[r] = -1;
  }
  R.nsteps[r]++;
  R.tprev[r] = nt0;
  R.tnext[r] = nt1;
  R.dtc[r] = dtn;
}

// Brownian values W(t) of this thread's owned elements (rows r0 and r0 + 8,
// columns c, c + 1 of one quad of dimensions) for the rows with flag[row] set,
// at time tsel[row] (FP64, times dir).  The two lanes that share a quad split
// the work by row -- the even lane descends the tree for r0, the odd lane for
// r0 + 8, each for all four dimensions of the quad from its cached path -- and
// swap halves.  Every lane of the warp must call it.
template <class SH, class ROWS, int NE>
__device__ __forceinline__ void vbt_owned(const SolveParams &P, const ROWS &R, const int *flag,
                                          const double *tsel, VbtQuadCache &vc, float (&W)[NE],
                                          int warp, int lane) {
  static_assert(NE == 4, "one output tile per thread");
  int row0, col0;
  elem_rc<SH>(0, warp, lane, row0, col0);
  const bool odd = lane & 1;
  const int myrow = odd ? row0 + 8 : row0;
  float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
  if (flag[myrow]) w = vbt_w_quad(P, R.idx[myrow], tsel[myrow] * R.dir[myrow], col0 >> 2, vc);
  const float sx = odd ? w.x : w.z, sy = odd ? w.y : w.w;
  const float rx = __shfl_xor_sync(0xffffffffu, sx, 1), ry = __shfl_xor_sync(0xffffffffu, sy, 1);
  if (odd) {
    W[0] = rx;
    W[1] = ry;
    W[2] = w.z;
    W[3] = w.w;
  } else {
    W[0] = w.x;
    W[1] = w.y;
    W[2] = rx;
    W[3] = ry;
  }
}

// W(t0) of freshly loaded rows (SDE).
template <class SH, int M, int NE>
__device__ __forceinline__ void load_brownian(const SolveParams &P, const RowState<M> &R,
                                              VbtQuadCache &vc, float (&Wb)[NE], int warp,
                                              int lane) {
  float W[NE];
  vbt_owned<SH>(P, R, R.loaded, R.tprev, vc, W, warp, lane);
#pragma unroll
  for (int e = 0; e < NE; e++) {
    int row, col;
    elem_rc<SH>(e, warp, lane, row, col);
    if (R.loaded[row]) Wb[e] = W[e];
  }
}

// Initial state of freshly loaded rows: y0, a zero FSAL vector, the t0 save,
// the first state checkpoint and (SDE) the Brownian value at t0.
template <class SH, bool SDE, int M, int NE>
__device__ __forceinline__ void load_rows(float (&Y0)[NE], float (&F0)[NE], float (&Wb)[NE],
                                          const SolveParams &P, const RowState<M> &R, int warp,
                                          int lane) {
  constexpr int D = SH::D;
#pragma unroll
  for (int e = 0; e < NE; e += 2) {
    int row, col;
    elem_rc<SH>(e, warp, lane, row, col);
    if (R.loaded[row]) {
      const int64_t i = R.idx[row];
      const float *y0 = reinterpret_cast<const float *>(P.y0) + i * D + col;
      Y0[e] = y0[0];
      Y0[e + 1] = y0[1];
      F0[e] = F0[e + 1] = 0.f;
      if (P.save_t0) {
        float *o = GBDX_AT(P, reinterpret_cast<float *>(P.ys_out), (i * P.n_save) * D + col, 2,
                           P.batch * P.n_save * D, GBDX_SITE_YS);
        o[0] = Y0[e];
        o[1] = Y0[e + 1];
      }
      if (P.tape_y) {
        float *o = GBDX_AT(P, P.tape_y, (i * P.checkpoints) * D + col, 2,
                           P.batch * P.checkpoints * D, GBDX_SITE_TAPE_Y);
        o[0] = Y0[e];
        o[1] = Y0[e + 1];
      }
    }
  }
}

// Whether condition e fires between its values vo and vn: a boolean when it
// holds, a real value on the chosen sign change (_integrate.py:585-602).
__device__ __forceinline__ bool mlp_ev_fires(const SolveParams &P, int e, double vo, double vn) {
  if (P.ev_kind[e] != GBDX_EV_LINEAR) return vn != 0.0;
  const double so = isnan(vo) ? vo : double((vo > 0) - (vo < 0));
  const double sn = isnan(vn) ? vn : double((vn > 0) - (vn < 0));
  if (P.ev_dir[e] == GBDX_EV_UP) return so <= 0 && sn > 0;
  if (P.ev_dir[e] == GBDX_EV_DOWN) return so > 0 && sn <= 0;
  return so != sn;
}

// Per-tile partial sums of f.f and y.y of every row (the steady-state
// condition's norms, _event.py:120-175), one slot per 8-column tile.
template <class SH, int M, int NE>
__device__ __forceinline__ void steady_partials(RowEvents<M> &R, const float (&F)[NE],
                                                const float (&Y)[NE], int warp, int lane) {
#pragma unroll
  for (int j = 0; j < SH::TPW; j++) {
#pragma unroll
    for (int half = 0; half < 2; half++) {
      int row, col;
      elem_rc<SH>(j * 4 + half * 2, warp, lane, row, col);
      float pf = 0.f, py = 0.f;
#pragma unroll
      for (int q = 0; q < 2; q++) {
        const int e = j * 4 + half * 2 + q;
        pf = fmaf(F[e], F[e], pf);
        py = fmaf(Y[e], Y[e], py);
      }
      pf += __shfl_xor_sync(0xffffffffu, pf, 1);
      pf += __shfl_xor_sync(0xffffffffu, pf, 2);
      py += __shfl_xor_sync(0xffffffffu, py, 1);
      py += __shfl_xor_sync(0xffffffffu, py, 2);
      if ((lane & 3) == 0) {
        R.pf[row][(warp * SH::TPW + j) % SH::NT] = pf;
        R.py[row][(warp * SH::TPW + j) % SH::NT] = py;
      }
    }
  }
}

// Value of steady-state condition e for row r from its partials.
template <class SH, int M>
__device__ __forceinline__ double steady_value(const SolveParams &P, const RowEvents<M> &R, int r,
                                               int e) {
  float sf = 0.f, sy = 0.f;
#pragma unroll
  for (int n = 0; n < SH::NT; n++) {
    sf += R.pf[r][n];
    sy += R.py[r][n];
  }
  return sqrt(double(sf) / SH::D) < P.ev_coef[6 * e + 1] + P.ev_coef[6 * e] * sqrt(double(sy) / SH::D)
             ? 1.0
             : 0.0;
}

// The FSAL values of freshly loaded rows resumed from a record with a valid
// solver state (row_init cleared their `first`).
template <class SH, int M, int NE>
__device__ __forceinline__ void load_fsal_state(float (&F0)[NE], const SolveParams &P,
                                                const RowState<M> &R, int warp, int lane) {
  constexpr int D = SH::D;
#pragma unroll
  for (int e = 0; e < NE; e++) {
    int row, col;
    elem_rc<SH>(e, warp, lane, row, col);
    if (R.loaded[row] && !R.first[row])
      F0[e] = float(*GBDX_AT(P, P.state_in, R.idx[row] * int64_t(GBDX_STATE_HEAD + D) +
                                                GBDX_STATE_HEAD + col,
                             1, P.batch * (GBDX_STATE_HEAD + D), GBDX_SITE_STATE));
  }
}

// The solver's local interpolant inside a step, one component: its value at
// theta or its theta-derivative, from y0, y1 and the stage increments k(j)
// (the trajectory kernels' formulas).
template <int SOLVER, int S, bool DERIV, class KF>
__device__ __forceinline__ float mlp_interp(float th, float y0, float y1, const KF &k) {
  if constexpr (SOLVER == GBDX_TSIT5) {
    float a = 0.f;
#pragma unroll
    for (int j = 0; j < 7; j++)
      a = fmaf(DERIV ? tsit5_dw<float>(j, th) : tsit5_w<float>(j, th), k(j < S ? j : 0), a);
    return DERIV ? a : y0 + a;
  } else if constexpr (SOLVER == GBDX_DOPRI5) {
    float cm = 0.f;
#pragma unroll
    for (int j = 0; j < S; j++) cm = fmaf(float(Tab<GBDX_DOPRI5>::cmid(j < 7 ? j : 0)), k(j), cm);
    const float ym = y0 + cm, fa = k(0), fb = k(S - 1);
    const float a = 2.f * (fb - fa) - 8.f * (y1 + y0) + 16.f * ym;
    const float b = 5.f * fa - 3.f * fb + 18.f * y0 + 14.f * y1 - 32.f * ym;
    const float c = fb - 4.f * fa - 11.f * y0 - 5.f * y1 + 16.f * ym;
    if (DERIV) return ((4.f * a * th + 3.f * b) * th + 2.f * c) * th + fa;
    return (((a * th + b) * th + c) * th + fa) * th + y0;
  } else if constexpr (SOLVER == GBDX_HEUN) {
    const float ka = k(0), kb = k(S - 1);
    const float a = ka + kb + 2.f * y0 - 2.f * y1;
    const float b = -2.f * ka - kb - 3.f * y0 + 3.f * y1;
    if (DERIV) return (3.f * a * th + 2.f * b) * th + ka;
    return ((a * th + b) * th + ka) * th + y0;
  } else {
    return DERIV ? y1 - y0 : y0 + th * (y1 - y0);
  }
}

// The event's root find on row r's last step (_integrate.py:704-779), as the
// trajectory kernels do it: Newton's method with cauchy termination on
// g(t) = w . interp(t) + wt t + c over [tp, tn] from t = tn, each iterate
// clipped to the step; components 0..3 of the step's y0, y1 and stages come
// from the row state.  Returns the root; ok = false after 256 iterations.
template <int SOLVER, int S, int M>
__device__ double mlp_ev_root(const SolveParams &P, const RowEvents<M> &R, int r,
                              const double (&cf)[6], int nc, double tp, double tn, bool &ok) {
  ok = true;
  const double span = tn - tp;
  double t = tn;
  for (int it = 1; it <= 256; it++) {
    const float th = float(span == 0.0 ? 0.0 : (t - tp) / span);
    double g = 0.0, gp = 0.0;
    for (int n = 0; n < nc; n++) {
      auto k = [&](int j) { return R.ek[r][j][n]; };
      g += cf[n] * double(mlp_interp<SOLVER, S, false>(th, R.ey0[r][n], R.ey1[r][n], k));
      gp += cf[n] * (span == 0.0 ? 0.0
                                 : double(mlp_interp<SOLVER, S, true>(th, R.ey0[r][n],
                                                                       R.ey1[r][n], k)) / span);
    }
    g += cf[4] * t;
    g += cf[5];
    gp += cf[4];
    const double diff = g / gp;
    double nt = t - diff;
    nt = fmax(fmin(nt, tn), tp);
    if (isnan(nt)) {
      ok = false;
      return t;
    }
    const double size = fabs(diff) / (P.newton_atol + P.newton_rtol * fabs(nt));
    t = nt;
    if (it >= 2 && size < 1.0 && fabs(g) < P.newton_atol) return t;
  }
  ok = false;
  return t;
}

// ---------------------------------------------------------------------------
// The kernel.
// ---------------------------------------------------------------------------
// Bytes of dynamic shared memory before the event state of the XO kernel.
template <class Sm>
constexpr size_t mlp_events_offset() {
  return (sizeof(Sm) + 15) / 16 * 16;
}

// XO (extended outputs: SaveAt(steps=n), SaveAt(dense=True), the clip
// controller and events) is a template flag, as in the trajectory kernels, so
// that the kernels without them keep their registers.
template <int SOLVER, int D, int H, bool PRECISE, bool SDE, bool XO>
__global__ void __launch_bounds__(256) mlp_fused_kernel(SolveParams P) {
  using SH = MlpShape<D, H>;
  using FLD = MlpField<SH, PRECISE, SDE>;
  using Sm = typename FLD::Sm;
  using TB = Tab<SOLVER>;
  constexpr int S = TB::S, NE = SH::NE, M = SH::M;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Sm &sm = *reinterpret_cast<Sm *>(smem_raw);
  RowState<M> &R = sm.rows;
  RowEvents<M> *EV =
      XO ? reinterpret_cast<RowEvents<M> *>(smem_raw + mlp_events_offset<Sm>()) : nullptr;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float *W = P.mlp;

  FLD::stage(sm, P, tid);
  bool ev_steady = false;
  if constexpr (XO) {
#pragma unroll
    for (int e = 0; e < GBDX_MAX_EVENTS; e++)
      ev_steady |= e < P.n_event && P.ev_kind[e] == GBDX_EV_STEADY;
  }
  if (tid < M) {
    const unsigned long long q = atomicAdd(P.queue, 1ull);
    if (q < (unsigned long long)P.batch) {
      row_init<M, XO>(R, EV, tid, P.order ? (int64_t)P.order[q] : (int64_t)q, P, D,
                       TB::FSAL);
      R.loaded[tid] = 1;
    } else {
      R.active[tid] = 0;
      R.loaded[tid] = 0;
    }
  }
  __syncthreads();

  float Y0[NE], F0[NE], Wb[NE];
#pragma unroll
  for (int e = 0; e < NE; e++) {
    int row, col;
    elem_rc<SH>(e, warp, lane, row, col);
    Y0[e] = 0.f;
    F0[e] = 0.f;
    Wb[e] = 0.f;
  }
  VbtQuadCache vc;
  vc.traj = -1;
  vc.node = 0;
  load_rows<SH, SDE>(Y0, F0, Wb, P, R, warp, lane);
  if constexpr (XO && TB::FSAL) {
    if (P.state_in) load_fsal_state<SH>(F0, P, R, warp, lane);
  }
  if constexpr (SDE) load_brownian<SH>(P, R, vc, Wb, warp, lane);
  __syncthreads();
  if (tid < M) R.loaded[tid] = 0;

  float K[S][NE], Yi[NE], F[NE], sig[NE], dW[NE], Wn[NE];
  while (true) {
    // ---- one lockstep step -------------------------------------------------
    int live = 0, first_live = 0;
    if (tid < M) {
      live = row_running(R, tid, P.max_steps);
      first_live = live && R.first[tid];
      R.live[tid] = live;
      R.acc[tid] = 0.f;
      R.anynan[tid] = 0;
      // control h = dir * dt as FP32 (WrapTerm, _term.py:742-745)
      R.h[tid] = live ? float(R.dir[tid] > 0 ? R.dtc[tid] : -R.dtc[tid]) : 0.f;
    }
    const int any_first = __syncthreads_or(first_live);
    float hrow[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) {
      int row, col;
      elem_rc<SH>(e, warp, lane, row, col);
      hrow[e] = R.h[row];
    }
    if constexpr (SDE) {
      // Brownian increment over [tprev, tnext] of every owned element; W at
      // tprev is carried from the previous accepted step.
      vbt_owned<SH>(P, R, R.live, R.tnext, vc, Wn, warp, lane);
#pragma unroll
      for (int e = 0; e < NE; e++) dW[e] = Wn[e] - Wb[e];
    }
    // stage 0 (FSAL reuse unless some row is on its first step)
    if (!TB::FSAL || any_first) {
      FLD::put_x(sm, Y0, warp, lane);
      __syncthreads();
      FLD::eval(sm, W, F, sig, tid, warp, lane);
    } else {
#pragma unroll
      for (int e = 0; e < NE; e++) F[e] = F0[e];
    }
    // a steady-state condition already true at (t0, y0) ends the solve before
    // its first step (_integrate.py:1333-1426); F holds f(y0) for a fresh row
    if constexpr (XO) {
      if (ev_steady) {
        const int fresh = tid < M && live && R.nsteps[tid] == 0;
        if (__syncthreads_or(fresh)) {
          steady_partials<SH>(*EV, F, Y0, warp, lane);
          __syncthreads();
          if (fresh) {
#pragma unroll
            for (int e = 0; e < GBDX_MAX_EVENTS; e++) {
              if (e < P.n_event && P.ev_kind[e] == GBDX_EV_STEADY) {
                const double v = steady_value<SH>(P, *EV, tid, e);
                EV->evv[tid][e] = v;
                if (EV->evi[tid] < 0 && v != 0.0) EV->evi[tid] = e;
              }
            }
            if (EV->evi[tid] >= 0) {
              R.result[tid] = GBDX_EVENT_OCCURRED;
              live = 0;
              R.live[tid] = 0;
            }
          }
          __syncthreads();
        }
      }
    }
#pragma unroll
    for (int e = 0; e < NE; e++) K[0][e] = SDE ? F[e] * hrow[e] + sig[e] * dW[e] : F[e] * hrow[e];
#pragma unroll
    for (int i = 1; i < S; i++) {
#pragma unroll
      for (int e = 0; e < NE; e++) {
        float a = Y0[e];
#pragma unroll
        for (int j = 0; j < i; j++)
          if (TB::a(i, j) != 0.0) a = fmaf(float(TB::a(i, j)), K[j][e], a);
        Yi[e] = a;
      }
      __syncthreads();  // the previous product has finished reading X
      FLD::put_x(sm, Yi, warp, lane);
      __syncthreads();
      FLD::eval(sm, W, F, sig, tid, warp, lane);
#pragma unroll
      for (int e = 0; e < NE; e++)
        K[i][e] = SDE ? F[e] * hrow[e] + sig[e] * dW[e] : F[e] * hrow[e];
    }
    // y1, error estimate, per-row scaled error norm
    float Y1[NE], Er[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) {
      if constexpr (TB::SSAL) {
        Y1[e] = Yi[e];
      } else {
        float a = Y0[e];
#pragma unroll
        for (int j = 0; j < S; j++) a = fmaf(float(TB::b(j)), K[j][e], a);
        Y1[e] = a;
      }
      float er = 0.f;
#pragma unroll
      for (int j = 0; j < S; j++)
        if (TB::e(j) != 0.0) er = fmaf(float(TB::e(j)), K[j][e], er);
      Er[e] = isnan(er) ? INFINITY : er;
    }
    if (P.controller == GBDX_PID) {
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        if (isnan(Y1[e])) R.anynan[row] = 1;
      }
      __syncthreads();
      // rows of this thread: for each tile two rows (g, g + 8)
#pragma unroll
      for (int j = 0; j < SH::TPW; j++) {
#pragma unroll
        for (int half = 0; half < 2; half++) {
          int row, col;
          elem_rc<SH>(j * 4 + half * 2, warp, lane, row, col);
          const bool nanrow = R.anynan[row];
          float part = 0.f;
#pragma unroll
          for (int q = 0; q < 2; q++) {
            const int e = j * 4 + half * 2 + q;
            const float ym = fmaxf(fabsf(Y0[e]), fabsf(nanrow ? Y0[e] : Y1[e]));
            const float s = __fdividef(Er[e], fmaf(ym, P.rtol_f, P.atol_f));
            part = fmaf(s, s, part);
          }
          part += __shfl_xor_sync(0xffffffffu, part, 1);
          part += __shfl_xor_sync(0xffffffffu, part, 2);
          if ((lane & 3) == 0) R.part[row][(warp * SH::TPW + j) % SH::NT] = part;
        }
      }
      __syncthreads();
      if (tid < M && live) {
        float a = 0.f;
#pragma unroll
        for (int n = 0; n < SH::NT; n++) a += R.part[tid][n];
        R.acc[tid] = a;
      }
    }
    __syncthreads();
    if (tid < M && live) row_control<M, XO>(R, tid, D, P);
    __syncthreads();
    // ---- events at the new state (_integrate.py:542-633) --------------------
    // The first condition (in order) that fires ends the solve; with a root
    // finder the final time is the root inside this step and no save after
    // it is made.
    if constexpr (XO) {
    if (P.n_event > 0) {
      RowEvents<M> &E = *EV;
      if constexpr (!TB::FSAL) {
        // f(y1) for a steady-state condition (FSAL solvers have it in F)
        if (ev_steady && __syncthreads_or(tid < M && live && R.keep[tid])) {
          FLD::put_x(sm, Y1, warp, lane);
          __syncthreads();
          FLD::eval(sm, W, F, sig, tid, warp, lane);
        }
      }
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        if (col < 4 && R.live[row] && R.keep[row]) {
          E.ey0[row][col] = Y0[e];
          E.ey1[row][col] = Y1[e];
#pragma unroll
          for (int j = 0; j < S; j++) E.ek[row][j][col] = K[j][e];
        }
      }
      if (ev_steady) steady_partials<SH>(E, F, Y1, warp, lane);
      __syncthreads();
      if (tid < M) {
        E.tsave[tid] = R.tn_old[tid];
        if (live && R.keep[tid]) {
          const double tn = R.tn_old[tid], tp = R.tp_old[tid];
          int fired = -1;
#pragma unroll
          for (int e = 0; e < GBDX_MAX_EVENTS; e++) {
            if (e < P.n_event) {
              double v;
              if (P.ev_kind[e] == GBDX_EV_STEADY) {
                v = steady_value<SH>(P, E, tid, e);
              } else {
                v = 0.0;
                for (int n = 0; n < (D < 4 ? D : 4); n++)
                  v += P.ev_coef[6 * e + n] * double(E.ey1[tid][n]);
                v += P.ev_coef[6 * e + 4] * tn;
                v += P.ev_coef[6 * e + 5];
                if (P.ev_kind[e] == GBDX_EV_LINEAR_BOOL) v = v > 0 ? 1.0 : 0.0;
              }
              if (fired < 0 && mlp_ev_fires(P, e, E.evv[tid][e], v)) fired = e;
              E.evv[tid][e] = v;
            }
          }
          if (fired >= 0) {
            E.evi[tid] = fired;
            R.result[tid] = GBDX_EVENT_OCCURRED;
            E.tfin[tid] = tn;
            if (P.event_root) {
              // a boolean condition's root is the end of the step
              double root = tn;
              if (P.ev_kind[fired] == GBDX_EV_LINEAR) {
                double cf[6];
#pragma unroll
                for (int n = 0; n < 6; n++) cf[n] = P.ev_coef[6 * fired + n];
                bool ok = true;
                root = mlp_ev_root<SOLVER, S>(P, E, tid, cf, D < 4 ? D : 4, tp, tn, ok);
                if (!ok) R.result[tid] = GBDX_NONLINEAR_MAX_STEPS;
              }
              const double span = tn - tp;
              E.tfin[tid] = root;
              E.tsave[tid] = root;
              E.thfin[tid] = float(span == 0.0 ? 0.0 : (root - tp) / span);
            }
          }
        }
      }
      __syncthreads();
    }
    }
    // ---- SaveAt(ts) inside accepted steps (_integrate.py:456-487) ----------
    while (true) {
      int fl = 0;
      if (tid < M) {
        R.sflag[tid] = 0;
        if (live && R.keep[tid] && R.ts_index[tid] < P.n_ts) {
          const double tsv = __ldg(P.save_ts + R.ts_index[tid]);
          const double tsd = R.dir[tid] * tsv;
          if (tsd <= ((XO && P.n_event > 0) ? EV->tsave[tid] : R.tn_old[tid])) {
            const double tp = R.tp_old[tid], tn = R.tn_old[tid];
            R.theta[tid] = float(tp == tn ? 0.0 : (tsd - tp) / (tn - tp));
            R.sslot[tid] = R.save_index[tid];
            *GBDX_AT(P, P.ts_out, R.idx[tid] * P.n_save + R.save_index[tid], 1,
                     P.batch * P.n_save, GBDX_SITE_TS) = tsv;
            R.ts_index[tid]++;
            R.save_index[tid]++;
            R.sflag[tid] = 1;
            fl = 1;
          }
        }
      }
      if (!__syncthreads_or(fl)) break;
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        if (R.sflag[row]) {
          const float th = R.theta[row];
          float v;
          if constexpr (SOLVER == GBDX_TSIT5) {
            float a = 0.f;
#pragma unroll
            for (int j = 0; j < 7; j++) a = fmaf(tsit5_w<float>(j, th), K[j < S ? j : 0][e], a);
            v = Y0[e] + a;
          } else if constexpr (SOLVER == GBDX_DOPRI5) {
            float cm = 0.f;
#pragma unroll
            for (int j = 0; j < S; j++)
              cm = fmaf(float(Tab<GBDX_DOPRI5>::cmid(j < 7 ? j : 0)), K[j][e], cm);
            const float y0 = Y0[e], y1 = Y1[e], ym = y0 + cm, fa = K[0][e], fb = K[S - 1][e];
            const float a = 2.f * (fb - fa) - 8.f * (y1 + y0) + 16.f * ym;
            const float b = 5.f * fa - 3.f * fb + 18.f * y0 + 14.f * y1 - 32.f * ym;
            const float c = fb - 4.f * fa - 11.f * y0 - 5.f * y1 + 16.f * ym;
            v = (((a * th + b) * th + c) * th + fa) * th + y0;
          } else if constexpr (SOLVER == GBDX_HEUN) {
            const float y0 = Y0[e], y1 = Y1[e], ka = K[0][e], kb = K[S - 1][e];
            const float a = ka + kb + 2.f * y0 - 2.f * y1;
            const float b = -2.f * ka - kb - 3.f * y0 + 3.f * y1;
            v = ((a * th + b) * th + ka) * th + y0;
          } else {
            v = Y0[e] + th * (Y1[e] - Y0[e]);
          }
          *GBDX_AT(P, reinterpret_cast<float *>(P.ys_out),
                   (R.idx[row] * P.n_save + R.sslot[row]) * D + col, 1, P.batch * P.n_save * D,
                   GBDX_SITE_YS) = v;
        }
      }
      __syncthreads();
    }
    // ---- SaveAt(steps=n), after the step's ts saves (_integrate.py:492-527),
    // and SaveAt(dense=True) step times (:529-540) ----------------------------
    if (XO && (P.save_steps > 0 || P.dense_ts != nullptr)) {
      if (tid < M) {
        R.stslot[tid] = -1;
        if (live && R.keep[tid]) {
          const int64_t i = R.idx[tid];
          if (P.save_steps > 0 && --R.sdown[tid] == 0) {
            R.sdown[tid] = P.save_steps;
            // not past an event's root
            if (!(P.n_event > 0 && order_key(R.tn_old[tid]) > order_key(EV->tsave[tid]))) {
              R.stslot[tid] = R.save_index[tid]++;
              *GBDX_AT(P, P.ts_out, i * P.n_save + R.stslot[tid], 1, P.batch * P.n_save,
                       GBDX_SITE_TS) = R.dir[tid] * R.tn_old[tid];
            }
          }
          // nacc already counts this step
          if (P.dense_ts)
            *GBDX_AT(P, P.dense_ts, i * (P.max_steps + 1) + R.nacc[tid], 1,
                     P.batch * (P.max_steps + 1), GBDX_SITE_DENSE_TS) = R.tn_old[tid];
        }
      }
      __syncthreads();
    }
    // ---- accept: advance the state, FSAL vector, Brownian cache, tape -------
#pragma unroll
    for (int e = 0; e < NE; e++) {
      int row, col;
      elem_rc<SH>(e, warp, lane, row, col);
      if (R.live[row] && R.keep[row]) {
        if constexpr (XO) {
        if (R.stslot[row] >= 0)
          *GBDX_AT(P, reinterpret_cast<float *>(P.ys_out),
                   (R.idx[row] * P.n_save + R.stslot[row]) * D + col, 1,
                   P.batch * P.n_save * D, GBDX_SITE_YS) = Y1[e];
        if (P.dense_info) {
          // the step's (y0, y1, k_0..k_{S-1}), component col of each
          constexpr int REC = (2 + S) * D;
          float *rec = GBDX_AT(P, static_cast<float *>(P.dense_info),
                               (R.idx[row] * P.max_steps + R.nacc[row] - 1) * REC, REC,
                               P.batch * P.max_steps * REC, GBDX_SITE_DENSE_INFO);
          rec[col] = Y0[e];
          rec[D + col] = Y1[e];
#pragma unroll
          for (int j = 0; j < S; j++) rec[(2 + j) * D + col] = K[j][e];
        }
        if (P.n_event > 0 && EV->evi[row] >= 0 && EV->thfin[row] >= 0.f) {
          // the state at the event's root (or the step's end for a boolean)
          Y1[e] = mlp_interp<SOLVER, S, false>(EV->thfin[row], Y0[e], Y1[e],
                                               [&](int j) { return K[j][e]; });
        }
        }
        Y0[e] = Y1[e];
        if (TB::FSAL) F0[e] = F[e];  // field value of the last stage (FSAL)
        if (SDE) Wb[e] = Wn[e];
        if (P.tape_y && R.cpslot[row] >= 0) {
          const int64_t b0 = R.idx[row] * P.checkpoints * D + col;
          const int64_t ext = P.batch * P.checkpoints * D;
          if (R.cpcompact[row] & 1)
            for (int s2 = 1; s2 < P.checkpoints / 2; s2++)
              *GBDX_AT(P, P.tape_y, b0 + s2 * D, 1, ext, GBDX_SITE_TAPE_Y) =
                  *GBDX_AT(P, P.tape_y, b0 + 2 * s2 * D, 1, ext, GBDX_SITE_TAPE_Y);
          *GBDX_AT(P, P.tape_y, b0 + R.cpslot[row] * D, 1, ext, GBDX_SITE_TAPE_Y) = Y0[e];
        }
      }
    }
    // ---- finished rows: t1 save, outputs, refill ----------------------------
    int fin = 0;
    if (tid < M) {
      R.fin[tid] = 0;
      if (R.active[tid] && !row_running(R, tid, P.max_steps)) {
        const int64_t i = R.idx[tid];
        const int dir = R.dir[tid];
        const double t0 = P.t0[i * P.time_stride] * dir;
        int si = R.save_index[tid];
        R.nfill[tid] = (t0 == R.t1[tid]) ? P.n_ts : 0;
        R.sslot[tid] = si;  // first slot written by the element pass
        const int64_t tse = P.batch * P.n_save;
        for (int m = 0; m < R.nfill[tid]; m++)
          *GBDX_AT(P, P.ts_out, i * P.n_save + si + m, 1, tse, GBDX_SITE_TS) = t0 * dir;
        si += R.nfill[tid];
        // the t1 value is already saved when SaveAt(steps=n) saved the last
        // step (_integrate.py:847-877); with an event root finder the final
        // value is saved whenever the steps saved the t1 value, as that save
        // fell after the event (:860-872), and the final time is the event's
        R.sflag[tid] = P.save_t1;
        double tf = R.tprev[tid];
        if constexpr (XO) {
          const bool via_steps = P.save_steps > 0 && R.sdown[tid] == P.save_steps;
          const bool root = P.n_event > 0 && P.event_root;
          R.sflag[tid] = root ? (P.save_t1 || via_steps) : (P.save_t1 && !via_steps);
          if (root && EV->evi[tid] >= 0) tf = EV->tfin[tid];
          if (P.event_index) P.event_index[i] = EV->evi[tid];
          if (P.dense_n) P.dense_n[i] = R.nacc[tid] + 1;
          if (P.state_out) {
            // SaveAt(controller_state=, solver_state=, made_jump=)
            // (_integrate.py:1489-1500): the head of the record; the
            // element pass writes the FSAL value
            double *so = GBDX_AT(P, P.state_out, i * int64_t(GBDX_STATE_HEAD + D),
                                 GBDX_STATE_HEAD, P.batch * (GBDX_STATE_HEAD + D),
                                 GBDX_SITE_STATE);
            if (P.controller == GBDX_PID) {
              so[0] = exp2(double(R.hist1[tid]));
              so[1] = exp2(double(R.hist2[tid]));
              so[2] = R.at_dtmin[tid] ? 1.0 : 0.0;
              so[3] = 0.0;
            } else {
              so[0] = R.sc[tid];
              so[1] = R.nc[tid];
              so[2] = R.t0s[tid];
              so[3] = R.t1s[tid];
            }
            so[4] = 1.0;
            so[5] = (TB::FSAL && !R.first[tid]) ? 0.0 : 1.0;
            so[6] = 0.0;  // made_jump: set by a ClipStepSizeController only
          }
        }
        if (R.sflag[tid])
          *GBDX_AT(P, P.ts_out, i * P.n_save + si++, 1, tse, GBDX_SITE_TS) = tf * dir;
        if (!P.saves_prefilled)
          for (int m = si; m < P.n_save; m++)  // direction * inf
            *GBDX_AT(P, P.ts_out, i * P.n_save + m, 1, tse, GBDX_SITE_TS) =
                dir > 0 ? INFINITY : -INFINITY;
        int res = R.result[tid];
        if (res == GBDX_SUCCESSFUL && order_key(R.tprev[tid]) < order_key(R.t1[tid]))
          res = GBDX_MAX_STEPS_REACHED;
        P.result_out[i] = res;
        P.stats_out[i * 3 + 0] = R.nsteps[tid];
        P.stats_out[i * 3 + 1] = R.nacc[tid];
        P.stats_out[i * 3 + 2] = R.nrej[tid];
        if (P.tape_n) {
          P.tape_n[i] = R.nacc[tid];
          P.tape_stride[i] = R.cpstride[tid];
        }
        R.fin[tid] = 1;
        fin = 1;
      }
    }
    if (__syncthreads_or(fin)) {
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        if (R.fin[row]) {
          float *o = reinterpret_cast<float *>(P.ys_out);
          const int64_t b0 = R.idx[row] * P.n_save * D + col, ext = P.batch * P.n_save * D;
          int si = R.sslot[row];
          for (int m = 0; m < R.nfill[row]; m++)
            *GBDX_AT(P, o, b0 + (si + m) * D, 1, ext, GBDX_SITE_YS) = Y0[e];
          si += R.nfill[row];
          if (R.sflag[row]) *GBDX_AT(P, o, b0 + (si++) * D, 1, ext, GBDX_SITE_YS) = Y0[e];
          if (!P.saves_prefilled)
            for (int m = si; m < P.n_save; m++)
              *GBDX_AT(P, o, b0 + m * D, 1, ext, GBDX_SITE_YS) = INFINITY;
          if constexpr (XO) {
            if (P.state_out)  // the record's FSAL value (0 where there is none)
              *GBDX_AT(P, P.state_out,
                       R.idx[row] * int64_t(GBDX_STATE_HEAD + D) + GBDX_STATE_HEAD + col, 1,
                       P.batch * (GBDX_STATE_HEAD + D), GBDX_SITE_STATE) =
                  (TB::FSAL && !R.first[row]) ? double(F0[e]) : 0.0;
          }
        }
      }
      __syncthreads();
      if (tid < M && R.fin[tid]) {
        const unsigned long long q = atomicAdd(P.queue, 1ull);
        if (q < (unsigned long long)P.batch) {
          row_init<M, XO>(R, EV, tid, P.order ? (int64_t)P.order[q] : (int64_t)q, P, D,
                       TB::FSAL);
          R.loaded[tid] = 1;
        } else {
          R.active[tid] = 0;
        }
      }
      __syncthreads();
      load_rows<SH, SDE>(Y0, F0, Wb, P, R, warp, lane);
      if constexpr (XO && TB::FSAL) {
        if (P.state_in) load_fsal_state<SH>(F0, P, R, warp, lane);
      }
      if constexpr (SDE) load_brownian<SH>(P, R, vc, Wb, warp, lane);
      __syncthreads();
      if (tid < M) R.loaded[tid] = 0;
    }
    if (!__syncthreads_or(tid < M && R.active[tid])) break;
  }
}

}  // namespace gbdx
