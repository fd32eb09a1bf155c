// gbdx_backsolve.cuh -- BacksolveAdjoint backward for MLP fields
// (diffrax/_adjoint.py:572-734, AdjointTerm diffrax/_term.py:767-910).
//
// Per trajectory the backward is a chain of reverse-time solves of the
// augmented state z = (y, a, a_theta), one per pair of adjacent saved times
// ts[j] -> ts[j-1] (t0 after the first save unless t0 itself was saved),
// started from the saved y with a += dL/dys[j] (_adjoint.py:646-650).  The
// augmented field is AdjointTerm.vf: (f, -a^T df/dy, -a^T df/dtheta).  Solver
// and controller state carry from segment to segment; every segment starts
// with a fresh FSAL evaluation (made_jump) and the initial step of
// diffeqsolve with a passed controller state (_integrate.py:1252-1265).
//
// A CTA of 8 warps integrates a tile of M trajectories ("rows") in lockstep,
// as the forward kernel does; each row walks its own segments and refills
// from the work counter after its last one.  Per RK stage the tile evaluates
// f and the VJP a^T df/dy as chains of tensor-core products of the BF16
// weights with three-piece BF16 operands (24 significant bits; or FP32
// CUDA-core products in the parity mode) and records, per
// row, the vector pairs whose outer products are -a^T df/dtheta:
//   (dz0, x) for W0/b0, (dz1, h1) for W1/b1, (a, h2) for W2/b2,
// where x is the stage input, h1, h2 the hidden activations and dz0, dz1 the
// cotangents of the pre-activations.  The parameter part of the state never
// exists per stage: after the stages a parameter pass contracts the records
// with the tableau weights for every parameter of the row,
//   da_theta = -h sum_j b_j u_j (x) v_j,   err_theta = -h sum_j e_j u_j (x) v_j.
//   * PIDController with rms_norm (the reference's default): the error norm
//     runs over a_theta, so every row keeps its a_theta in HBM (double
//     buffered).  Before the controller decision the pass reads a_theta0,
//     writes the candidate a_theta1 and adds the scaled squared errors to the
//     row's norm; the buffers flip on accept, and a finished row folds its
//     a_theta into the CTA's Kahan partial gradient.
//   * adjoint_rms_seminorm or ConstantStepSize: the norm does not see
//     a_theta; after the decision the pass adds the accepted increments to
//     the row's a_theta in place.
// Either way a finished row folds its a_theta into the CTA's Kahan partial.
#pragma once

#include <cuda_bf16.h>

#include "gbdx_common.cuh"
#include "gbdx_mlp_bwd.cuh"
#include "gbdx_mma.cuh"
#include "gbdx_traj.cuh"

namespace gbdx {

template <int D_, int H_>
struct BsShape {
  static constexpr int D = D_, H = H_;
  static constexpr int M = D_ >= 64 ? 16 : 32;  // rows per CTA
  static constexpr int THREADS = 256, WARPS = 8;
  // The weights are the model's BF16 values (as in the forward kernel).
  // Width 256: W1 stays in shared memory; W0 and W2 are read as pre-arranged
  // BF16 fragments from global memory (L2).  Narrower fields keep all three
  // in shared memory.
  static constexpr bool GFRAG = H_ >= 256;
  static constexpr int PD = D + 8, PH = H + 8;
  static constexpr int MT = M / 16, NT = D / 8, NTH = H / 8;
  static constexpr int TPW = MT * NT / WARPS;    // output tiles per warp
  static constexpr int TPWH = MT * NTH / WARPS;  // hidden tiles per warp
  static constexpr int NE = 4 * TPW;             // owned elements per thread
  static_assert(MT * NT % WARPS == 0 && TPW >= 1, "tile split");
  static_assert(MT * NTH % WARPS == 0 && NTH % TPWH == 0, "hidden tile split");
  static_assert(NT % TPW == 0, "output tile split");
  static_assert(NT <= 8, "error-norm partials: at most 8 column tiles");
  // flat parameter offsets (FP32, row-major [out][in]), as MlpShape
  static constexpr int OW0 = 0, OB0 = OW0 + H * D, OW1 = OB0 + H, OB1 = OW1 + H * H,
                       OW2 = OB1 + H, OB2 = OW2 + D * H, NP = OB2 + D;
  // per (stage, row) record: x, a, h1, h2, dz0, dz1 (FP32)
  static constexpr int RX = 0, RG = D, RH1 = 2 * D, RH2 = 2 * D + H, RZ0 = 2 * D + 2 * H,
                       RZ1 = 2 * D + 3 * H, REC = 2 * D + 4 * H;
  static_assert(NP % 4 == 0 && D % 4 == 0 && H % 4 == 0, "vector alignment");
};

template <int M>
struct BsRows {
  double tprev[M], tnext[M], te[M], floor_te[M], dtc[M], t0s[M], t1s[M];
  long long idx[M];
  float h[M], hist1[M], hist2[M], acc[M];
  int active[M], want[M], first[M], keep[M], nan_y[M], nan_a[M], dir[M];
  int seg[M], jold[M], trans[M], newtraj[M], done[M], firstseg[M];
  int nseg[M], nsteps[M], nacc[M], nrej[M], result[M], sres[M], sc[M], nc[M], at_dtmin[M];
  double ginv[M];  // RN(1 / nc), for the grid fraction
  int live[M], cur[M], zero[M];
  float part[M][8];  // error-norm partials per 8-column tile, summed in order
};

template <class SH, bool GF>
struct BsWeights;
template <class SH>
struct BsWeights<SH, false> {
  __nv_bfloat16 W0[SH::H][SH::PD];
  __nv_bfloat16 W1[SH::H][SH::PH];
  __nv_bfloat16 W2[SH::D][SH::PH];
};
template <class SH>
struct BsWeights<SH, true> {
  __nv_bfloat16 W1[SH::H][SH::PH];
};

template <class SH, bool PRECISE>
struct BsSmem;

// Stage operands as three BF16 pieces each (24 significant bits): X the
// stage input, G its cotangent a, R1 h1 then dz0, R2 h2 then dz1.
template <class SH>
struct BsAct {
  __nv_bfloat16 X[SH::M][SH::PD], Xl[SH::M][SH::PD], Xl2[SH::M][SH::PD];
  __nv_bfloat16 G[SH::M][SH::PD], Gl[SH::M][SH::PD], Gl2[SH::M][SH::PD];
  __nv_bfloat16 R1[SH::M][SH::PH], R1l[SH::M][SH::PH], R1l2[SH::M][SH::PH];
  __nv_bfloat16 R2[SH::M][SH::PH], R2l[SH::M][SH::PH], R2l2[SH::M][SH::PH];
};
// Operands of the tensor-core parameter pass of one row and one layer
// W [NO][NI]: o-side vectors U0 = -h u0, A2 = sum_j b_j du_j,
// A3 = sum_j e_j du_j and the stage differences du_j = -h (u_j - u_0) (BF16,
// [o][k = j - 1]); i-side vectors v0, B1 = v0 + sum_j b_j dv_j,
// B3 = sum_j e_j dv_j and b_j dv_j, e_j dv_j (BF16, [k][i]).
template <int NO, int NI>
struct __align__(16) BsLayerOps {
  float U0[NO], A2[NO], A3[NO], v0[NI], B1[NI], B3[NI];
  __nv_bfloat16 Du[NO][24];
  __nv_bfloat16 Bb[16][NI + 8], Be[16][NI + 8];
};
// The three layers of one row together, so that the row's weight tiles
// stream as one sequence.
template <class SH>
struct BsPassOps {
  BsLayerOps<SH::H, SH::D> l0;
  BsLayerOps<SH::H, SH::H> l1;
  BsLayerOps<SH::D, SH::H> l2;
};

template <class SH>
struct BsSmem<SH, false> : BsWeights<SH, SH::GFRAG> {
  float b0[SH::H], b1[SH::H], b2[SH::D];
  union {  // the stage products and the parameter pass never overlap
    BsAct<SH> a;
    BsPassOps<SH> p;
    float cf[SH::H][16];  // FP32 parameter-pass coefficients
  };
  float red[SH::WARPS];
  float rsum[SH::WARPS][SH::M];  // per-warp parameter-pass norm partials
  BsRows<SH::M> rows;
};

// FP32 stage operands of the parity mode.
template <class SH>
struct BsActF32 {
  float X[SH::M][SH::D + 1], G[SH::M][SH::D + 1];
  float R1[SH::M][SH::H + 1], R2[SH::M][SH::H + 1];
};

template <class SH>
struct BsSmem<SH, true> {
  float b0[SH::H], b1[SH::H], b2[SH::D];
  BsActF32<SH> a;
  __align__(16) float cf[SH::H][16];
  float red[SH::WARPS];
  BsRows<SH::M> rows;
};

template <class SH, bool PRECISE>
struct BsField {
  using Sm = BsSmem<SH, PRECISE>;
  static constexpr int D = SH::D, H = SH::H, M = SH::M, NE = SH::NE, REC = SH::REC;

  __device__ static void stage(Sm &sm, const float *P, int tid) {
    for (int i = tid; i < H; i += SH::THREADS) {
      sm.b0[i] = P[SH::OB0 + i];
      sm.b1[i] = P[SH::OB1 + i];
    }
    for (int i = tid; i < D; i += SH::THREADS) sm.b2[i] = P[SH::OB2 + i];
    if constexpr (!PRECISE) {
      if constexpr (SH::GFRAG) {
        for (int i = tid; i < H * H; i += SH::THREADS)
          sm.W1[i / H][i % H] = __float2bfloat16_rn(P[SH::OW1 + i]);
      } else {
        for (int i = tid; i < H * D; i += SH::THREADS)
          sm.W0[i / D][i % D] = __float2bfloat16_rn(P[SH::OW0 + i]);
        for (int i = tid; i < H * H; i += SH::THREADS)
          sm.W1[i / H][i % H] = __float2bfloat16_rn(P[SH::OW1 + i]);
        for (int i = tid; i < D * H; i += SH::THREADS)
          sm.W2[i / H][i % H] = __float2bfloat16_rn(P[SH::OW2 + i]);
      }
    }
  }

  // Stage inputs (owned layout) -> product operands and the x, a records.
  __device__ static void put(Sm &sm, const float (&Y)[NE], const float (&A)[NE], float *rec,
                             int warp, int lane) {
#pragma unroll
    for (int e = 0; e < NE; e += 2) {
      int row, col;
      elem_rc<SH>(e, warp, lane, row, col);
      if constexpr (PRECISE) {
        sm.a.X[row][col] = Y[e];
        sm.a.X[row][col + 1] = Y[e + 1];
        sm.a.G[row][col] = A[e];
        sm.a.G[row][col + 1] = A[e + 1];
      } else {
        store_split3x2(Y[e], Y[e + 1], &sm.a.X[row][col], &sm.a.Xl[row][col],
                       &sm.a.Xl2[row][col]);
        store_split3x2(A[e], A[e + 1], &sm.a.G[row][col], &sm.a.Gl[row][col],
                       &sm.a.Gl2[row][col]);
      }
      *reinterpret_cast<float2 *>(rec + row * REC + SH::RX + col) = make_float2(Y[e], Y[e + 1]);
      *reinterpret_cast<float2 *>(rec + row * REC + SH::RG + col) = make_float2(A[e], A[e + 1]);
    }
  }

  // acc += (A0 + A1 + A2) W^T over K, W the BF16 weights row-major [n][k].
  template <int K, int NTW>
  __device__ static __forceinline__ void fwd_gemm(float (&acc)[NTW][4], const __nv_bfloat16 *A0,
                                                  const __nv_bfloat16 *A1,
                                                  const __nv_bfloat16 *A2, int lda,
                                                  const __nv_bfloat16 *W, int ldw, int lane) {
    warp_tile_gemm_p<K, NTW, 3>(acc, A0, A1, A2, lda, W, ldw, lane);
  }
  // acc += (A0 + A1 + A2) W over K, W row-major [k][n] (transposed loads).
  template <int K, int NTW>
  __device__ static __forceinline__ void vjp_gemm(float (&acc)[NTW][4], const __nv_bfloat16 *A0,
                                                  const __nv_bfloat16 *A1,
                                                  const __nv_bfloat16 *A2, int lda,
                                                  const __nv_bfloat16 *W, int ldw, int n0,
                                                  int lane) {
    warp_tile_gemm_bt3<K, NTW>(acc, A0, A1, A2, lda, W, ldw, n0, lane);
  }

  // Hidden-tile epilogue helper: write v to R (split) and to the record.
  __device__ static __forceinline__ void put_hidden(Sm &sm, int which, int row, int col,
                                                    float v0, float v1, float *rec, int roff) {
    if constexpr (PRECISE) {
      auto R = which == 1 ? sm.a.R1 : sm.a.R2;
      R[row][col] = v0;
      R[row][col + 1] = v1;
    } else {
      if (which == 1)
        store_split3x2(v0, v1, &sm.a.R1[row][col], &sm.a.R1l[row][col], &sm.a.R1l2[row][col]);
      else
        store_split3x2(v0, v1, &sm.a.R2[row][col], &sm.a.R2l[row][col], &sm.a.R2l2[row][col]);
    }
    *reinterpret_cast<float2 *>(rec + row * REC + roff + col) = make_float2(v0, v1);
  }

  // F = MLP(X) and GY = A^T dMLP/dX (owned layout) with the stage records.
  // X and G must have been written and synchronised.  Ends with every warp
  // past its last read of R1 only after the caller's next barrier.
  __device__ static void eval(Sm &sm, const float *P, const BsParams &Q, float (&F)[NE],
                              float (&GY)[NE], float *rec, int tid, int warp, int lane) {
    if constexpr (PRECISE) {
      const float *W0 = P + SH::OW0, *W1 = P + SH::OW1, *W2 = P + SH::OW2;
      for (int i = tid; i < M * H; i += SH::THREADS) {
        const int r = i / H, n = i % H;
        float a = sm.b0[n];
        for (int k = 0; k < D; k++) a = fmaf(sm.a.X[r][k], __ldg(W0 + n * D + k), a);
        const float v = tanhf(a);
        sm.a.R1[r][n] = v;
        rec[r * REC + SH::RH1 + n] = v;
      }
      __syncthreads();
      for (int i = tid; i < M * H; i += SH::THREADS) {
        const int r = i / H, n = i % H;
        float a = sm.b1[n];
        for (int k = 0; k < H; k++) a = fmaf(sm.a.R1[r][k], __ldg(W1 + n * H + k), a);
        const float v = tanhf(a);
        sm.a.R2[r][n] = v;
        rec[r * REC + SH::RH2 + n] = v;
      }
      __syncthreads();
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        float a = sm.b2[col];
        for (int k = 0; k < H; k++) a = fmaf(sm.a.R2[row][k], __ldg(W2 + col * H + k), a);
        F[e] = a;
      }
      __syncthreads();
      // dz1 = (G W2) * (1 - h2^2), in place of h2
      for (int i = tid; i < M * H; i += SH::THREADS) {
        const int r = i / H, n = i % H;
        float a = 0.f;
        for (int d = 0; d < D; d++) a = fmaf(sm.a.G[r][d], __ldg(W2 + d * H + n), a);
        const float h2 = sm.a.R2[r][n];
        const float v = a * (1.f - h2 * h2);
        sm.a.R2[r][n] = v;
        rec[r * REC + SH::RZ1 + n] = v;
      }
      __syncthreads();
      // dz0 = (dz1 W1) * (1 - h1^2), in place of h1
      for (int i = tid; i < M * H; i += SH::THREADS) {
        const int r = i / H, n = i % H;
        float a = 0.f;
        for (int o = 0; o < H; o++) a = fmaf(sm.a.R2[r][o], __ldg(W1 + o * H + n), a);
        const float h1 = sm.a.R1[r][n];
        const float v = a * (1.f - h1 * h1);
        sm.a.R1[r][n] = v;
        rec[r * REC + SH::RZ0 + n] = v;
      }
      __syncthreads();
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        float a = 0.f;
        for (int o = 0; o < H; o++) a = fmaf(sm.a.R1[row][o], __ldg(W0 + o * D + col), a);
        GY[e] = a;
      }
    } else {
      const int g = lane >> 2, c = lane & 3;
      const int th0 = warp * SH::TPWH, mth = th0 / SH::NTH, nth0 = th0 % SH::NTH;
      const int to0 = warp * SH::TPW, mto = to0 / SH::NT, nto0 = to0 % SH::NT;
      {  // layer 0: h1 = tanh(X W0^T + b0) -> R1
        float acc[SH::TPWH][4];
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        if constexpr (SH::GFRAG)
          gemm_gfrag_p<D, SH::TPWH, 3>(acc, &sm.a.X[mth * 16][0], &sm.a.Xl[mth * 16][0],
                                       &sm.a.Xl2[mth * 16][0], SH::PD, Q.w0f, nth0, lane);
        else
          fwd_gemm<D, SH::TPWH>(acc, &sm.a.X[mth * 16][0], &sm.a.Xl[mth * 16][0],
                                &sm.a.Xl2[mth * 16][0], SH::PD, &sm.W0[nth0 * 8][0], SH::PD,
                                lane);
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) {
          const int col = (nth0 + j) * 8 + 2 * c, r0 = mth * 16 + g;
          const float bb0 = sm.b0[col], bb1 = sm.b0[col + 1];
          put_hidden(sm, 1, r0, col, tanhf(acc[j][0] + bb0), tanhf(acc[j][1] + bb1), rec,
                     SH::RH1);
          put_hidden(sm, 1, r0 + 8, col, tanhf(acc[j][2] + bb0), tanhf(acc[j][3] + bb1), rec,
                     SH::RH1);
        }
      }
      __syncthreads();
      {  // layer 1: h2 = tanh(R1 W1^T + b1) -> R2
        float acc[SH::TPWH][4];
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        fwd_gemm<H, SH::TPWH>(acc, &sm.a.R1[mth * 16][0], &sm.a.R1l[mth * 16][0],
                              &sm.a.R1l2[mth * 16][0], SH::PH, &sm.W1[nth0 * 8][0], SH::PH,
                              lane);
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) {
          const int col = (nth0 + j) * 8 + 2 * c, r0 = mth * 16 + g;
          const float bb0 = sm.b1[col], bb1 = sm.b1[col + 1];
          put_hidden(sm, 2, r0, col, tanhf(acc[j][0] + bb0), tanhf(acc[j][1] + bb1), rec,
                     SH::RH2);
          put_hidden(sm, 2, r0 + 8, col, tanhf(acc[j][2] + bb0), tanhf(acc[j][3] + bb1), rec,
                     SH::RH2);
        }
      }
      __syncthreads();
      {  // layer 2: F = R2 W2^T + b2 (owned layout)
        float acc[SH::TPW][4];
#pragma unroll
        for (int j = 0; j < SH::TPW; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        if constexpr (SH::GFRAG)
          gemm_gfrag_p<H, SH::TPW, 3>(acc, &sm.a.R2[mto * 16][0], &sm.a.R2l[mto * 16][0],
                                      &sm.a.R2l2[mto * 16][0], SH::PH, Q.w2f, nto0, lane);
        else
          fwd_gemm<H, SH::TPW>(acc, &sm.a.R2[mto * 16][0], &sm.a.R2l[mto * 16][0],
                               &sm.a.R2l2[mto * 16][0], SH::PH, &sm.W2[nto0 * 8][0], SH::PH,
                               lane);
#pragma unroll
        for (int e = 0; e < NE; e++) {
          int row, col;
          elem_rc<SH>(e, warp, lane, row, col);
          F[e] = acc[e >> 2][e & 3] + sm.b2[col];
        }
      }
      __syncthreads();  // every warp has read h2 as an operand
      {  // dz1 = (G W2) * (1 - h2^2) -> R2 in place
        float acc[SH::TPWH][4];
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        if constexpr (SH::GFRAG)
          gemm_gfrag_p<D, SH::TPWH, 3>(acc, &sm.a.G[mth * 16][0], &sm.a.Gl[mth * 16][0],
                                       &sm.a.Gl2[mth * 16][0], SH::PD, Q.w2v, nth0, lane);
        else
          vjp_gemm<D, SH::TPWH>(acc, &sm.a.G[mth * 16][0], &sm.a.Gl[mth * 16][0],
                                &sm.a.Gl2[mth * 16][0], SH::PD, &sm.W2[0][0], SH::PH, nth0 * 8,
                                lane);
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++)
#pragma unroll
          for (int hr = 0; hr < 2; hr++) {
            const int row = mth * 16 + g + hr * 8, col = (nth0 + j) * 8 + 2 * c;
            const float a0 = __bfloat162float(sm.a.R2[row][col]) +
                             __bfloat162float(sm.a.R2l[row][col]) +
                             __bfloat162float(sm.a.R2l2[row][col]);
            const float a1 = __bfloat162float(sm.a.R2[row][col + 1]) +
                             __bfloat162float(sm.a.R2l[row][col + 1]) +
                             __bfloat162float(sm.a.R2l2[row][col + 1]);
            put_hidden(sm, 2, row, col, acc[j][2 * hr] * (1.f - a0 * a0),
                       acc[j][2 * hr + 1] * (1.f - a1 * a1), rec, SH::RZ1);
          }
      }
      __syncthreads();
      {  // dz0 = (R2 W1) * (1 - h1^2) -> R1 in place
        float acc[SH::TPWH][4];
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        vjp_gemm<H, SH::TPWH>(acc, &sm.a.R2[mth * 16][0], &sm.a.R2l[mth * 16][0],
                              &sm.a.R2l2[mth * 16][0], SH::PH, &sm.W1[0][0], SH::PH, nth0 * 8,
                              lane);
#pragma unroll
        for (int j = 0; j < SH::TPWH; j++)
#pragma unroll
          for (int hr = 0; hr < 2; hr++) {
            const int row = mth * 16 + g + hr * 8, col = (nth0 + j) * 8 + 2 * c;
            const float a0 = __bfloat162float(sm.a.R1[row][col]) +
                             __bfloat162float(sm.a.R1l[row][col]) +
                             __bfloat162float(sm.a.R1l2[row][col]);
            const float a1 = __bfloat162float(sm.a.R1[row][col + 1]) +
                             __bfloat162float(sm.a.R1l[row][col + 1]) +
                             __bfloat162float(sm.a.R1l2[row][col + 1]);
            put_hidden(sm, 1, row, col, acc[j][2 * hr] * (1.f - a0 * a0),
                       acc[j][2 * hr + 1] * (1.f - a1 * a1), rec, SH::RZ0);
          }
      }
      __syncthreads();
      {  // GY = R1 W0 (owned layout)
        float acc[SH::TPW][4];
#pragma unroll
        for (int j = 0; j < SH::TPW; j++) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
        if constexpr (SH::GFRAG)
          gemm_gfrag_p<H, SH::TPW, 3>(acc, &sm.a.R1[mto * 16][0], &sm.a.R1l[mto * 16][0],
                                      &sm.a.R1l2[mto * 16][0], SH::PH, Q.w0v, nto0, lane);
        else
          vjp_gemm<H, SH::TPW>(acc, &sm.a.R1[mto * 16][0], &sm.a.R1l[mto * 16][0],
                               &sm.a.R1l2[mto * 16][0], SH::PH, &sm.W0[0][0], SH::PD, nto0 * 8,
                               lane);
#pragma unroll
        for (int e = 0; e < NE; e++) GY[e] = acc[e >> 2][e & 3];
      }
    }
  }
};

// ---------------------------------------------------------------------------
// The parameter pass of one row and one layer W [NO][NI], b [NO]: stage
// vectors u (length NO, record offset UOFF) and v (length NI, VOFF).
// NORM: a1 = a0 + da written to the candidate buffer, returns this thread's
// share of sum (err / (atol + rtol max(|a0|, |a1|)))^2.  Otherwise da is added
// to the CTA partial (Kahan).
// ---------------------------------------------------------------------------
__device__ __forceinline__ void kahan4(float *sum, float *comp, const float (&x)[4]) {
  float4 s = *reinterpret_cast<float4 *>(sum), c = *reinterpret_cast<float4 *>(comp);
  float sv[4] = {s.x, s.y, s.z, s.w}, cv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
  for (int q = 0; q < 4; q++) {
    const float y = x[q] - cv[q];
    const float t = sv[q] + y;
    cv[q] = (t - sv[q]) - y;
    sv[q] = t;
  }
  *reinterpret_cast<float4 *>(sum) = make_float4(sv[0], sv[1], sv[2], sv[3]);
  *reinterpret_cast<float4 *>(comp) = make_float4(cv[0], cv[1], cv[2], cv[3]);
}

// (err / (atol + rtol max(|a0|, |a1|)))^2.  pid.py:475-492 scales a NaN
// candidate by a0: fmaxf returns its non-NaN operand.  A NaN error
// (infinite in _integrate.py:386) makes the row's norm NaN, which the
// controller treats as infinite: rejected, factor clipped to factormin.
__device__ __forceinline__ float scaled_sq(float a0, float a1, float err, float rtol,
                                           float atol) {
  const float m = fmaxf(fabsf(a0), fabsf(a1));
  const float s = __fdividef(err, fmaf(m, rtol, atol));
  return s * s;
}

template <class SH, int SOLVER, int NO, int NI, int UOFF, int VOFF, int WOFF, int BOFF, bool NORM>
__device__ __forceinline__ float theta_layer(float (*cf)[16], const float *rec_r, float h,
                                             const float *a0, float *a1, float *psum,
                                             float *pcomp, float rtol, float atol, int tid) {
  using TB = Tab<SOLVER>;
  constexpr int S = TB::S, STR = SH::M * SH::REC;
  // 1. per-output coefficients: cf[o][j] = -h b_j u_j[o], cf[o][8 + j] = -h e_j u_j[o]
  for (int o = tid; o < NO; o += SH::THREADS) {
#pragma unroll
    for (int j = 0; j < S; j++) {
      const float u = -h * rec_r[j * STR + UOFF + o];
      cf[o][j] = float(TB::b(j)) * u;
      cf[o][8 + j] = float(TB::e(j)) * u;
    }
  }
  __syncthreads();
  constexpr int TPR = NI / 4, RPI = SH::THREADS / TPR;
  static_assert(SH::THREADS % TPR == 0, "parameter pass split");
  const int i4 = (tid % TPR) * 4, orow = tid / TPR;
  float v[S][4];
#pragma unroll
  for (int j = 0; j < S; j++) {
    const float4 t = *reinterpret_cast<const float4 *>(rec_r + j * STR + VOFF + i4);
    v[j][0] = t.x;
    v[j][1] = t.y;
    v[j][2] = t.z;
    v[j][3] = t.w;
  }
  float accn = 0.f;
  // U output rows per batch: their loads are all issued before any is used,
  // so every thread keeps U vector loads in flight.
  constexpr int U = 8;
  for (int ob = orow; ob < NO; ob += RPI * U) {
    float x0[U][4];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int o = ob + u * RPI;
#pragma unroll
      for (int q = 0; q < 4; q++) x0[u][q] = 0.f;
      if (o < NO && a0) {
        const float4 t = __ldcs(reinterpret_cast<const float4 *>(a0 + WOFF + o * NI + i4));
        x0[u][0] = t.x;
        x0[u][1] = t.y;
        x0[u][2] = t.z;
        x0[u][3] = t.w;
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int o = ob + u * RPI;
      if (o >= NO) break;
      const int p = WOFF + o * NI + i4;
      float db[4], de[4];
#pragma unroll
      for (int q = 0; q < 4; q++) db[q] = de[q] = 0.f;
#pragma unroll
      for (int j = 0; j < S; j++) {
        const float cb = cf[o][j], ce = cf[o][8 + j];
#pragma unroll
        for (int q = 0; q < 4; q++) {
          if (TB::b(j) != 0.0) db[q] = fmaf(cb, v[j][q], db[q]);
          if (NORM && TB::e(j) != 0.0) de[q] = fmaf(ce, v[j][q], de[q]);
        }
      }
      float x1[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        x1[q] = x0[u][q] + db[q];
        if (NORM) accn += scaled_sq(x0[u][q], x1[q], de[q], rtol, atol);
      }
      __stcs(reinterpret_cast<float4 *>(a1 + p), make_float4(x1[0], x1[1], x1[2], x1[3]));
    }
  }
  // biases (v = 1)
  for (int o = tid; o < NO; o += SH::THREADS) {
    float db = 0.f, de = 0.f;
#pragma unroll
    for (int j = 0; j < S; j++) {
      db += cf[o][j];
      de += cf[o][8 + j];
    }
    const int p = BOFF + o;
    const float x0 = a0 ? a0[p] : 0.f;
    const float x1 = x0 + db;
    a1[p] = x1;
    if (NORM) accn += scaled_sq(x0, x1, de, rtol, atol);
  }
  __syncthreads();  // cf is rewritten by the next layer
  return accn;
}

template <class SH, int SOLVER, bool NORM>
__device__ __forceinline__ float theta_pass(float (*cf)[16], const float *rec_r, float h,
                                            const float *a0, float *a1, float *psum,
                                            float *pcomp, float rtol, float atol, int tid) {
  constexpr int D = SH::D, H = SH::H;
  float s = 0.f;
  s += theta_layer<SH, SOLVER, H, D, SH::RZ0, SH::RX, SH::OW0, SH::OB0, NORM>(
      cf, rec_r, h, a0, a1, psum, pcomp, rtol, atol, tid);
  s += theta_layer<SH, SOLVER, H, H, SH::RZ1, SH::RH1, SH::OW1, SH::OB1, NORM>(
      cf, rec_r, h, a0, a1, psum, pcomp, rtol, atol, tid);
  s += theta_layer<SH, SOLVER, D, H, SH::RG, SH::RH2, SH::OW2, SH::OB2, NORM>(
      cf, rec_r, h, a0, a1, psum, pcomp, rtol, atol, tid);
  return s;
}

// Tensor-core parameter pass under the tracked norm.
// With du_j = -h (u_j - u_0), dv_j = v_j - v_0 and sum_j b_j = 1, sum_j e_j = 0,
//   da  = -h sum_j b_j u_j v_j = U0 B1 + A2 v0 + sum_j du_j (b_j dv_j),
//   err = -h sum_j e_j u_j v_j = U0 B3 + A3 v0 + sum_j du_j (e_j dv_j):
// a rank-2 FP32 part, computed into the accumulators, plus a product over the
// stages whose factors are O(h) stage differences, so one BF16 tensor-core
// product per m16n8 tile carries it to well below FP32 rounding of da.  The
// error estimate loses no digits to the cancellation of its weights.
//
// In the tensor-core mode a row's weight gradients are stored in fragment
// order: tile t of a layer holds its 128 values at WOFF + 128 t + 4 lane + q,
// q indexing the accumulator elements (g, 2c), (g, 2c + 1), (g + 8, 2c),
// (g + 8, 2c + 1).  Warp w takes a contiguous run of each layer's m16n8
// tiles.

// Layer L of the field: W [NO][NI], its stage vectors u (record offset UOFF)
// and v (VOFF), its weights and biases in the flat parameter vector.
template <class SH, int L>
struct BsLayer;
template <class SH>
struct BsLayer<SH, 0> {
  static constexpr int NO = SH::H, NI = SH::D, UOFF = SH::RZ0, VOFF = SH::RX, WOFF = SH::OW0,
                       BOFF = SH::OB0;
  __device__ static BsLayerOps<NO, NI> &ops(BsPassOps<SH> &p) { return p.l0; }
};
template <class SH>
struct BsLayer<SH, 1> {
  static constexpr int NO = SH::H, NI = SH::H, UOFF = SH::RZ1, VOFF = SH::RH1, WOFF = SH::OW1,
                       BOFF = SH::OB1;
  __device__ static BsLayerOps<NO, NI> &ops(BsPassOps<SH> &p) { return p.l1; }
};
template <class SH>
struct BsLayer<SH, 2> {
  static constexpr int NO = SH::D, NI = SH::H, UOFF = SH::RG, VOFF = SH::RH2, WOFF = SH::OW2,
                       BOFF = SH::OB2;
  __device__ static BsLayerOps<NO, NI> &ops(BsPassOps<SH> &p) { return p.l2; }
};

// A row's weight tiles as one sequence of batches of U tiles per warp: the
// one batch of layer 0, the NB1 batches of layer 1, the one batch of layer 2.
// A batch's a_theta0 loads are issued one batch ahead (two register buffers),
// across layer and row boundaries.
template <class SH>
struct BsTiles {
  template <int L>
  static constexpr int tpw() {
    return (BsLayer<SH, L>::NO / 16) * (BsLayer<SH, L>::NI / 8) / SH::WARPS;
  }
  static constexpr int T0 = tpw<0>(), T1 = tpw<1>(), T2 = tpw<2>();
  static constexpr int U = T0 < 16 ? T0 : 16, NB1 = T1 / U, NB = NB1 + 2;
  // L2 prefetch distance, in batches: measured best at 2 for the tracked
  // norm's pass (a_theta0 read, the candidate written to the other buffer)
  // and 3 for the in-place pass of the seminorm
  template <bool NORM>
  static constexpr int pf() {
    return NORM ? 2 : 3;
  }
  static_assert(T0 * SH::WARPS == (BsLayer<SH, 0>::NO / 16) * (BsLayer<SH, 0>::NI / 8) &&
                    T1 * SH::WARPS == (BsLayer<SH, 1>::NO / 16) * (BsLayer<SH, 1>::NI / 8) &&
                    T2 * SH::WARPS == (BsLayer<SH, 2>::NO / 16) * (BsLayer<SH, 2>::NI / 8),
                "parameter tiles split over the warps");
  static_assert(T0 == U && T2 == U && T1 % (2 * U) == 0, "parameter tile batches");
};

// Batch i (0 <= i < NB) of a row in this warp's run: layer 0, NB1 batches of
// layer 1, layer 2.
template <class SH>
__device__ __forceinline__ const float *batch_ptr(const float *a0, int i, int warp) {
  using TL = BsTiles<SH>;
  if (i == 0) return a0 + BsLayer<SH, 0>::WOFF + warp * TL::T0 * 128;
  if (i <= TL::NB1) return a0 + BsLayer<SH, 1>::WOFF + (warp * TL::T1 + (i - 1) * TL::U) * 128;
  return a0 + BsLayer<SH, 2>::WOFF + warp * TL::T2 * 128;
}

// Bulk prefetch into L2 of batch i of the row (i >= NB: batch i - NB of the
// next row, when there is one), BsTiles::pf batches ahead of the register
// loads, so that those find their lines in L2.
template <class SH>
__device__ __forceinline__ void batch_prefetch(const float *a0, const float *a0n, bool next,
                                               int i, int warp, int lane) {
  using TL = BsTiles<SH>;
  const float *base = a0;
  if (i >= TL::NB) {
    i -= TL::NB;
    base = next ? a0n : nullptr;
  }
  if (lane == 0 && base && i < TL::NB) {
    const float *p = batch_ptr<SH>(base, i, warp);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(p),
                 "r"(uint32_t(TL::U * 128 * sizeof(float)))
                 : "memory");
  }
}

// The a_theta0 values of U tiles of layer L from tile tb of this warp's run
// (zeros for a row whose a_theta is still zero).
template <class SH, int L>
__device__ __forceinline__ void batch_load(float (&x)[BsTiles<SH>::U][4], const float *a0,
                                           int tb, int warp, int lane) {
  using TL = BsTiles<SH>;
  constexpr int TPW = TL::template tpw<L>(), WOFF = BsLayer<SH, L>::WOFF;
#pragma unroll
  for (int u = 0; u < TL::U; u++) {
    const int t = warp * TPW + tb + u;
    if (a0) {
      const float4 v = __ldcs(reinterpret_cast<const float4 *>(a0 + WOFF + t * 128 + lane * 4));
      x[u][0] = v.x;
      x[u][1] = v.y;
      x[u][2] = v.z;
      x[u][3] = v.w;
    } else {
      x[u][0] = x[u][1] = x[u][2] = x[u][3] = 0.f;
    }
  }
}

// U tiles of layer L from tile tb: a1 = a0 + da (fragment layout); returns
// their share of the scaled squared errors when NORM.
template <class SH, int S, int L, bool NORM>
__device__ __forceinline__ float batch_tiles(BsPassOps<SH> &pp,
                                             const float (&x0)[BsTiles<SH>::U][4], float *a1,
                                             int tb, int warp, int lane, float rtol, float atol) {
  using TL = BsTiles<SH>;
  using LY = BsLayer<SH, L>;
  constexpr int TPW = TL::template tpw<L>(), NI = LY::NI, NTL = NI / 8, WOFF = LY::WOFF;
  auto &ps = LY::ops(pp);
  const int g = lane >> 2, c = lane & 3;
  float accn = 0.f;
  // A batch starts on a multiple of U tiles; when U divides the tiles of an
  // output block, its tiles share one block: its A fragment and o-side
  // values are loaded once for the batch.
  constexpr bool ONE_BLOCK = NTL % TL::U == 0;
  const int tf = warp * TPW + tb;
  uint32_t ab[4];
  float u0a_b = 0.f, u0b_b = 0.f, a2a_b = 0.f, a2b_b = 0.f, a3a_b = 0.f, a3b_b = 0.f;
  if constexpr (ONE_BLOCK) {
    const int ot = tf / NTL, og = ot * 16 + g;
    ldsm_a(ab, &ps.Du[ot * 16][0], 24, lane);
    u0a_b = ps.U0[og];
    u0b_b = ps.U0[og + 8];
    a2a_b = ps.A2[og];
    a2b_b = ps.A2[og + 8];
    if constexpr (NORM) {
      a3a_b = ps.A3[og];
      a3b_b = ps.A3[og + 8];
    }
  }
#pragma unroll
  for (int u = 0; u < TL::U; u++) {
    const int t = tf + u, ot = t / NTL, nt = t % NTL;
    const int og = ot * 16 + g, ic = nt * 8 + 2 * c;
    uint32_t a[4], bb[2], be[2];
    if constexpr (ONE_BLOCK) {
#pragma unroll
      for (int k = 0; k < 4; k++) a[k] = ab[k];
    } else {
      ldsm_a(a, &ps.Du[ot * 16][0], 24, lane);
    }
    ldsm_bt1(bb, &ps.Bb[0][0], NI + 8, 0, nt * 8, lane);
    const float u0a = ONE_BLOCK ? u0a_b : ps.U0[og], u0b = ONE_BLOCK ? u0b_b : ps.U0[og + 8];
    const float a2a = ONE_BLOCK ? a2a_b : ps.A2[og], a2b = ONE_BLOCK ? a2b_b : ps.A2[og + 8];
    const float2 v0 = *reinterpret_cast<const float2 *>(&ps.v0[ic]);
    const float2 b1 = *reinterpret_cast<const float2 *>(&ps.B1[ic]);
    float cb[4] = {fmaf(u0a, b1.x, a2a * v0.x), fmaf(u0a, b1.y, a2a * v0.y),
                   fmaf(u0b, b1.x, a2b * v0.x), fmaf(u0b, b1.y, a2b * v0.y)};
    if constexpr (S > 1) mma_bf16(cb, a, bb[0], bb[1]);
    float x1[4];
#pragma unroll
    for (int q = 0; q < 4; q++) x1[q] = x0[u][q] + cb[q];
    if constexpr (NORM) {
      ldsm_bt1(be, &ps.Be[0][0], NI + 8, 0, nt * 8, lane);
      const float a3a = ONE_BLOCK ? a3a_b : ps.A3[og], a3b = ONE_BLOCK ? a3b_b : ps.A3[og + 8];
      const float2 b3 = *reinterpret_cast<const float2 *>(&ps.B3[ic]);
      float ce[4] = {fmaf(u0a, b3.x, a3a * v0.x), fmaf(u0a, b3.y, a3a * v0.y),
                     fmaf(u0b, b3.x, a3b * v0.x), fmaf(u0b, b3.y, a3b * v0.y)};
      if constexpr (S > 1) mma_bf16(ce, a, be[0], be[1]);
#pragma unroll
      for (int q = 0; q < 4; q++) accn += scaled_sq(x0[u][q], x1[q], ce[q], rtol, atol);
    }
    __stcs(reinterpret_cast<float4 *>(a1 + WOFF + t * 128 + lane * 4),
           make_float4(x1[0], x1[1], x1[2], x1[3]));
  }
  return accn;
}

// A row's tiles, its layer-0 batch already loading into xa and its first
// layer-1 batch into xb; ends with batch 0 of the next row (a0n, when next)
// loading into xa.
template <class SH, int S, bool NORM>
__device__ __forceinline__ float row_tiles(BsPassOps<SH> &pp, float (&xa)[BsTiles<SH>::U][4],
                                           float (&xb)[BsTiles<SH>::U][4], const float *a0,
                                           float *a1, bool next, const float *a0n, int warp,
                                           int lane, float rtol, float atol) {
  using TL = BsTiles<SH>;
  constexpr int U = TL::U;
  float s = batch_tiles<SH, S, 0, NORM>(pp, xa, a1, 0, warp, lane, rtol, atol);
#pragma unroll 1
  for (int tb = 0, i = 2; tb < TL::T1; tb += 2 * U, i += 2) {
    // batch i: layer-1 tile tb + U; batch i + 1: the next
    batch_load<SH, 1>(xa, a0, tb + U, warp, lane);
    batch_prefetch<SH>(a0, a0n, next, i + TL::template pf<NORM>(), warp, lane);
    s += batch_tiles<SH, S, 1, NORM>(pp, xb, a1, tb, warp, lane, rtol, atol);
    if (tb + 2 * U < TL::T1)
      batch_load<SH, 1>(xb, a0, tb + 2 * U, warp, lane);
    else
      batch_load<SH, 2>(xb, a0, 0, warp, lane);
    batch_prefetch<SH>(a0, a0n, next, i + 1 + TL::template pf<NORM>(), warp, lane);
    s += batch_tiles<SH, S, 1, NORM>(pp, xa, a1, tb + U, warp, lane, rtol, atol);
  }
  if (next) {
    batch_load<SH, 0>(xa, a0n, 0, warp, lane);
    batch_prefetch<SH>(a0, a0n, next, TL::NB + TL::template pf<NORM>(), warp, lane);
  }
  s += batch_tiles<SH, S, 2, NORM>(pp, xb, a1, 0, warp, lane, rtol, atol);
  return s;
}

// One layer's stage records of a row, loaded into registers (this thread's
// i-side value v_j[tid], o-side value -h u_j[tid]) with the bias's a_theta0.
template <int S>
struct LayerRecs {
  float vv[S], uu[S], xb;
};
template <class SH, int L>
__device__ __forceinline__ float bias_load(const float *a0, int tid) {
  return (tid < BsLayer<SH, L>::NO && a0) ? a0[BsLayer<SH, L>::BOFF + tid] : 0.f;
}
template <class SH, int S, int L>
__device__ __forceinline__ void layer_recs(LayerRecs<S> &lr, const float *rec_r, float h,
                                           float xb, int tid) {
  using LY = BsLayer<SH, L>;
  constexpr int STR = SH::M * SH::REC;
  static_assert(LY::NI <= SH::THREADS && LY::NO <= SH::THREADS, "one operand row per thread");
  const bool own_i = tid < LY::NI, own_o = tid < LY::NO;
#pragma unroll
  for (int j = 0; j < S; j++) {
    lr.vv[j] = own_i ? rec_r[j * STR + LY::VOFF + tid] : 0.f;
    lr.uu[j] = own_o ? -h * rec_r[j * STR + LY::UOFF + tid] : 0.f;
  }
  lr.xb = xb;
}

// The layer's operands from its records, and its bias: da = U0 + A2,
// err = A3 (the bias's v is 1).  Returns the bias's scaled squared error.
template <class SH, int SOLVER, int L, bool NORM>
__device__ __forceinline__ float layer_ops(BsPassOps<SH> &pp, const LayerRecs<Tab<SOLVER>::S> &lr,
                                           float *a1, float rtol, float atol, int tid) {
  using TB = Tab<SOLVER>;
  using LY = BsLayer<SH, L>;
  constexpr int S = TB::S;
  static_assert(S - 1 <= 16, "stage differences fit one k16 slice");
  auto &ps = LY::ops(pp);
  float accn = 0.f;
  if (tid < LY::NI) {
    const int i = tid;
    float b1 = lr.vv[0], b3 = 0.f;
#pragma unroll
    for (int k = 0; k < 16; k++) {
      float bb = 0.f, be = 0.f;
      if (k + 1 < S) {
        const float dv = lr.vv[k + 1] - lr.vv[0];
        bb = float(TB::b(k + 1)) * dv;
        be = float(TB::e(k + 1)) * dv;
        b1 += bb;
        b3 += be;
      }
      ps.Bb[k][i] = __float2bfloat16_rn(bb);
      ps.Be[k][i] = __float2bfloat16_rn(be);
    }
    ps.v0[i] = lr.vv[0];
    ps.B1[i] = b1;
    ps.B3[i] = b3;
  }
  if (tid < LY::NO) {
    const int o = tid;
    float a2 = 0.f, a3 = 0.f;
#pragma unroll
    for (int k = 0; k < 16; k++) {
      float du = 0.f;
      if (k + 1 < S) {
        du = lr.uu[k + 1] - lr.uu[0];
        a2 = fmaf(float(TB::b(k + 1)), du, a2);
        a3 = fmaf(float(TB::e(k + 1)), du, a3);
      }
      ps.Du[o][k] = __float2bfloat16_rn(du);
    }
    ps.U0[o] = lr.uu[0];
    ps.A2[o] = a2;
    ps.A3[o] = a3;
    const float x1 = lr.xb + (lr.uu[0] + a2);
    a1[LY::BOFF + o] = x1;
    if (NORM) accn = scaled_sq(lr.xb, x1, a3, rtol, atol);
  }
  return accn;
}

// The parameter pass over the CTA's selected rows (sel(r): CTA-uniform), a
// row's a_theta0 / a_theta1 from ptrs(r, a0, a1).  Per row: its stage
// records and bias values are loaded, the three layers' operands written,
// one barrier, then the row's tiles as one stream whose loads run one batch
// ahead, into the next row's first batch.  NORM: warp w's share of row r's
// scaled squared errors goes to rsum[w][r] (the caller sums over w).
template <class SH, int SOLVER, bool NORM, class Sel, class Ptrs>
__device__ __forceinline__ void theta_rows_tc(BsPassOps<SH> &pp, float (*rsum)[SH::M],
                                              const float *rec, const float *hrow, Sel sel,
                                              Ptrs ptrs, float rtol, float atol, int tid,
                                              int warp, int lane) {
  using TL = BsTiles<SH>;
  constexpr int S = Tab<SOLVER>::S, M = SH::M;
  auto next_row = [&](int r) {
    for (r = r + 1; r < M; r++)
      if (sel(r)) break;
    return r;
  };
  int r = next_row(-1);
  if (r >= M) return;
  const float *a0;
  float *a1;
  ptrs(r, a0, a1);
  float xa[TL::U][4], xb[TL::U][4];
  batch_load<SH, 0>(xa, a0, 0, warp, lane);
#pragma unroll
  for (int i = 1; i <= TL::template pf<NORM>(); i++)
    batch_prefetch<SH>(a0, nullptr, false, i, warp, lane);
  while (r < M) {
    const int rn = next_row(r);
    const float *a0n = nullptr;
    float *a1n = nullptr;
    if (rn < M) ptrs(rn, a0n, a1n);
    const float *rec_r = rec + size_t(r) * SH::REC;
    const float h = hrow[r];
    float accn;
    {
      const float xb0 = bias_load<SH, 0>(a0, tid), xb1 = bias_load<SH, 1>(a0, tid),
                  xb2 = bias_load<SH, 2>(a0, tid);
      batch_load<SH, 1>(xb, a0, 0, warp, lane);
      batch_prefetch<SH>(a0, a0n, rn < M, 1 + TL::template pf<NORM>(), warp, lane);
      LayerRecs<S> lr;
      layer_recs<SH, S, 0>(lr, rec_r, h, xb0, tid);
      accn = layer_ops<SH, SOLVER, 0, NORM>(pp, lr, a1, rtol, atol, tid);
      layer_recs<SH, S, 1>(lr, rec_r, h, xb1, tid);
      accn += layer_ops<SH, SOLVER, 1, NORM>(pp, lr, a1, rtol, atol, tid);
      layer_recs<SH, S, 2>(lr, rec_r, h, xb2, tid);
      accn += layer_ops<SH, SOLVER, 2, NORM>(pp, lr, a1, rtol, atol, tid);
    }
    __syncthreads();  // the operands are complete
    accn += row_tiles<SH, S, NORM>(pp, xa, xb, a0, a1, rn < M, a0n, warp, lane, rtol, atol);
    if constexpr (NORM) {
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) accn += __shfl_xor_sync(0xffffffffu, accn, o);
      if (lane == 0) rsum[warp][r] = accn;
    }
    __syncthreads();  // the operands are rewritten for the next row
    r = rn;
    a0 = a0n;
    a1 = a1n;
  }
}

// Fold a finished row's a_theta into the CTA's Kahan partial.  The partial
// has the row buffers' layout (the weight blocks in fragment order in the
// tensor-core mode), so the fold is elementwise; the final reduction
// restores the flat order.
template <class SH>
__device__ __forceinline__ void fold_row(const float *a, float *psum, float *pcomp, int tid) {
  constexpr int NP = SH::NP, STEP = SH::THREADS * 4, U = 4;
  for (int e0 = tid * 4; e0 < NP; e0 += STEP * U) {
    float4 v[U], sm[U], cp[U];
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int e = e0 + u * STEP;
      if (e < NP) {
        v[u] = __ldcs(reinterpret_cast<const float4 *>(a + e));
        sm[u] = *reinterpret_cast<const float4 *>(psum + e);
        cp[u] = *reinterpret_cast<const float4 *>(pcomp + e);
      }
    }
#pragma unroll
    for (int u = 0; u < U; u++) {
      const int e = e0 + u * STEP;
      if (e < NP) {
        float sv[4] = {sm[u].x, sm[u].y, sm[u].z, sm[u].w};
        float cv[4] = {cp[u].x, cp[u].y, cp[u].z, cp[u].w};
        const float xv[4] = {v[u].x, v[u].y, v[u].z, v[u].w};
#pragma unroll
        for (int q = 0; q < 4; q++) {
          const float y = xv[q] - cv[q];
          const float t = sv[q] + y;
          cv[q] = (t - sv[q]) - y;
          sv[q] = t;
        }
        *reinterpret_cast<float4 *>(psum + e) = make_float4(sv[0], sv[1], sv[2], sv[3]);
        *reinterpret_cast<float4 *>(pcomp + e) = make_float4(cv[0], cv[1], cv[2], cv[3]);
      }
    }
  }
}

// Block-wide sum of one value per thread, returned to every thread.
template <class SH>
__device__ __forceinline__ float block_sum(float *red, float x, int tid) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  if ((tid & 31) == 0) red[tid >> 5] = x;
  __syncthreads();
  float t = 0.f;
#pragma unroll
  for (int w = 0; w < SH::WARPS; w++) t += red[w];
  __syncthreads();
  return t;
}

// ---------------------------------------------------------------------------
// Per-row scalar logic (one thread per row).
// ---------------------------------------------------------------------------
template <int M>
__device__ __forceinline__ bool bs_running(const BsRows<M> &R, int r, int max_steps) {
  return R.active[r] && order_key(R.tprev[r]) < order_key(R.te[r]) &&
         R.sres[r] == GBDX_SUCCESSFUL && R.nseg[r] < max_steps;
}

// Advance row r from segment jold to the next segment that takes a step
// (skipping empty ones): its times and the controller's initial step
// (_integrate.py:1252-1265, pid.py:316-392, constant.py:30-57).  Sets seg and
// done (no segment left).
template <int M>
__device__ void bs_next_segment(BsRows<M> &R, int r, const SolveParams &P) {
  const int64_t i = R.idx[r];
  const double *T = P.save_ts + i * P.n_save;
  const int64_t ti = i * P.time_stride;
  const double t0 = P.t0[ti];
  const int jlo = P.save_t0 ? 1 : 0;
  const int dir = R.dir[r];
  int j = R.jold[r] - 1;
  for (; j >= jlo; j--) {
    const double ts_ = dir * T[j], te = dir * (j >= 1 ? T[j - 1] : t0);
    double tn;
    if (P.controller == GBDX_PID) {
      if (R.firstseg[r] || !P.dt0) {
        double hh = P.dt0 ? fabs(P.dt0[ti]) : 0.01;
        if (P.has_dtmax) hh = fmin(hh, P.dtmax);
        if (P.has_dtmin) hh = fmax(hh, P.dtmin);
        tn = ts_ + hh;
      } else {
        tn = ts_ + fabs(P.dt0[ti]);
      }
      if (R.firstseg[r]) {
        R.hist1[r] = 0.f;
        R.hist2[r] = 0.f;
        R.at_dtmin[r] = 0;
      }
    } else {
      const double h0 = fabs(P.dt0[ti]);
      if (R.firstseg[r]) {
        R.sc[r] = 1;
        R.nc[r] = (int)ceil((te - ts_) / next_up(h0));
        R.ginv[r] = 1.0 / double(R.nc[r]);
        R.t0s[r] = ts_;
        R.t1s[r] = te;
      }
      tn = ts_ + h0;
    }
    R.firstseg[r] = 0;
    R.tprev[r] = ts_;
    R.te[r] = te;
    R.tnext[r] = fmin(tn, te);
    R.dtc[r] = R.tnext[r] - ts_;
    R.floor_te[r] = t1_clip_floor(te);
    R.nseg[r] = 0;
    R.first[r] = 1;
    R.sres[r] = GBDX_SUCCESSFUL;
    if (order_key(ts_) < order_key(te)) break;
  }
  R.seg[r] = j;
  R.done[r] = j < jlo;
}

// The controller's decision for row r (pid.py:394-567, constant.py:59-104,
// _integrate.py:410-413) on the sum of squared scaled errors R.acc over
// n_norm components.
template <int M>
__device__ void bs_row_control(BsRows<M> &R, int r, float n_norm, const SolveParams &P) {
  const double dt = R.dtc[r];
  bool keep;
  double nt0, nt1, dtn;
  if (P.controller == GBDX_PID) {
    const float acc = R.acc[r];
    keep = acc < n_norm;
    const float lg = 0.5f * (log2f(n_norm) - __log2f(acc));
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
      if (!P.force_dtmin && dtn < P.dtmin && R.sres[r] == GBDX_SUCCESSFUL)
        R.sres[r] = GBDX_DT_MIN_REACHED;
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
  }
  if (!(nt0 < R.te[r])) nt0 = R.te[r];
  if (order_key(nt1) > order_key(R.floor_te[r])) nt1 = keep ? R.te[r] : nt0 + 0.5 * (R.te[r] - nt0);
  dtn = nt1 - nt0;
  R.keep[r] = keep;
  if (keep) {
    R.nacc[r]++;
    R.first[r] = 0;
  } else {
    R.nrej[r]++;
  }
  R.nsteps[r]++;
  R.nseg[r]++;
  R.tprev[r] = nt0;
  R.tnext[r] = nt1;
  R.dtc[r] = dtn;
}

// ---------------------------------------------------------------------------
// The kernel.
// ---------------------------------------------------------------------------
template <int SOLVER, int D, int H, bool PRECISE>
__global__ void __launch_bounds__(256, 1) mlp_backsolve_kernel(SolveParams P, BsParams Q) {
  using SH = BsShape<D, H>;
  using FLD = BsField<SH, PRECISE>;
  using Sm = typename FLD::Sm;
  using TB = Tab<SOLVER>;
  constexpr int S = TB::S, NE = SH::NE, M = SH::M, REC = SH::REC, NP = SH::NP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  Sm &sm = *reinterpret_cast<Sm *>(smem_raw);
  BsRows<M> &R = sm.rows;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float *W = P.mlp;
  float *rec = Q.rec + size_t(blockIdx.x) * S * M * REC;
  float *psum = Q.psum + size_t(blockIdx.x) * NP;
  float *pcomp = Q.pcomp + size_t(blockIdx.x) * NP;
  float *ath = Q.ath + size_t(blockIdx.x) * M * 2 * NP;
  const float rtol = P.rtol_f, atol = P.atol_f;

  FLD::stage(sm, W, tid);
  if (tid < M) {
    R.active[tid] = 0;
    R.want[tid] = 1;
    R.live[tid] = 0;
  }
  __syncthreads();

  float Y0[NE], A0[NE], F0[NE], GY0[NE];
#pragma unroll
  for (int e = 0; e < NE; e++) Y0[e] = A0[e] = F0[e] = GY0[e] = 0.f;

  // Segment transitions: finished segments advance (adding the cotangents of
  // the saves they pass), finished rows write their outputs and refill.
  auto transitions = [&]() {
    while (true) {
      int need = 0;
      if (tid < M) {
        const int r = tid;
        R.trans[r] = 0;
        if (R.active[r] && !bs_running(R, r, P.max_steps)) {
          int sres = R.sres[r];
          if (sres == GBDX_SUCCESSFUL && order_key(R.tprev[r]) < order_key(R.te[r]))
            sres = GBDX_MAX_STEPS_REACHED;
          if (R.result[r] == GBDX_SUCCESSFUL) R.result[r] = sres;
          R.jold[r] = R.seg[r];
          R.trans[r] = 1;
          R.newtraj[r] = 0;
        } else if (!R.active[r] && R.want[r]) {
          const unsigned long long q = atomicAdd(P.queue, 1ull);
          if (q < (unsigned long long)P.batch) {
            const int64_t i = P.order ? (int64_t)P.order[q] : (int64_t)q;
            const int64_t ti = i * P.time_stride;
            R.idx[r] = i;
            R.dir[r] = (P.t0[ti] < P.t1[ti]) ? -1 : 1;
            R.jold[r] = P.n_save;
            R.firstseg[r] = 1;
            R.result[r] = GBDX_SUCCESSFUL;
            R.nsteps[r] = R.nacc[r] = R.nrej[r] = 0;
            R.cur[r] = 0;
            R.zero[r] = 1;
            R.active[r] = 1;
            R.trans[r] = 1;
            R.newtraj[r] = 1;
          } else {
            R.want[r] = 0;
          }
        }
        if (R.trans[r]) bs_next_segment(R, r, P);
        need = R.trans[r];
      }
      if (!__syncthreads_or(need)) break;
      // element pass: a += dL/dys over the saves passed, y from the new save
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        if (R.trans[row]) {
          const int64_t i = R.idx[row];
          if (R.newtraj[row]) A0[e] = 0.f;
          const int jn = R.seg[row] > 0 ? R.seg[row] : 0;
          for (int jj = jn; jj < R.jold[row]; jj++)
            A0[e] += *GBDX_AT(P, Q.grad_ys, (i * P.n_save + jj) * D + col, 1,
                              P.batch * P.n_save * D, GBDX_SITE_GRAD_YS);
          if (R.done[row]) {
            Q.grad_y0[i * D + col] = A0[e];
          } else {
            Y0[e] = *GBDX_AT(P, Q.ys, (i * P.n_save + R.seg[row]) * D + col, 1,
                             P.batch * P.n_save * D, GBDX_SITE_GRAD_YS);
          }
        }
      }
      __syncthreads();
      // finished rows: results, the a_theta fold, a fresh trajectory next time
      for (int r = 0; r < M; r++) {
        if (!(R.trans[r] && R.done[r])) continue;
        if (!R.zero[r]) fold_row<SH>(ath + (size_t(r) * 2 + R.cur[r]) * NP, psum, pcomp, tid);
      }
      if (tid < M && R.trans[tid] && R.done[tid]) {
        const int64_t i = R.idx[tid];
        P.result_out[i] = R.result[tid];
        P.stats_out[i * 3 + 0] = R.nsteps[tid];
        P.stats_out[i * 3 + 1] = R.nacc[tid];
        P.stats_out[i * 3 + 2] = R.nrej[tid];
        R.active[tid] = 0;
      }
      __syncthreads();
    }
  };

  transitions();
  float KY[S][NE], KA[S][NE], Yi[NE], Ai[NE], F[NE], GY[NE];
  while (__syncthreads_or(tid < M && R.active[tid])) {
    // ---- one lockstep step ---------------------------------------------------
    int first_live = 0;
    if (tid < M) {
      const int live = R.active[tid];
      first_live = live && R.first[tid];
      R.live[tid] = live;
      R.acc[tid] = 0.f;
      R.nan_y[tid] = R.nan_a[tid] = 0;
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
#pragma unroll
    for (int i = 0; i < S; i++) {
      float *rec_s = rec + size_t(i) * M * REC;
      if (i == 0) {
        if (!TB::FSAL || any_first) {
          FLD::put(sm, Y0, A0, rec_s, warp, lane);
          __syncthreads();
          FLD::eval(sm, W, Q, F, GY, rec_s, tid, warp, lane);
        } else {
#pragma unroll
          for (int e = 0; e < NE; e++) {
            F[e] = F0[e];
            GY[e] = GY0[e];
          }
        }
#pragma unroll
        for (int e = 0; e < NE; e++) {
          Yi[e] = Y0[e];
          Ai[e] = A0[e];
        }
      } else {
#pragma unroll
        for (int e = 0; e < NE; e++) {
          float a = Y0[e], b = A0[e];
#pragma unroll
          for (int j = 0; j < i; j++)
            if (TB::a(i, j) != 0.0) {
              a = fmaf(float(TB::a(i, j)), KY[j][e], a);
              b = fmaf(float(TB::a(i, j)), KA[j][e], b);
            }
          Yi[e] = a;
          Ai[e] = b;
        }
        __syncthreads();  // the previous products have finished reading X, G, R1
        FLD::put(sm, Yi, Ai, rec_s, warp, lane);
        __syncthreads();
        FLD::eval(sm, W, Q, F, GY, rec_s, tid, warp, lane);
      }
#pragma unroll
      for (int e = 0; e < NE; e++) {
        KY[i][e] = F[e] * hrow[e];
        KA[i][e] = -GY[e] * hrow[e];
      }
    }
    // y1, a1, error estimates, the (y, a) part of the error norm
    float Y1[NE], A1[NE], ErY[NE], ErA[NE];
#pragma unroll
    for (int e = 0; e < NE; e++) {
      if constexpr (TB::SSAL) {
        Y1[e] = Yi[e];
        A1[e] = Ai[e];
      } else {
        float a = Y0[e], b = A0[e];
#pragma unroll
        for (int j = 0; j < S; j++) {
          a = fmaf(float(TB::b(j)), KY[j][e], a);
          b = fmaf(float(TB::b(j)), KA[j][e], b);
        }
        Y1[e] = a;
        A1[e] = b;
      }
      float ey = 0.f, ea = 0.f;
#pragma unroll
      for (int j = 0; j < S; j++)
        if (TB::e(j) != 0.0) {
          ey = fmaf(float(TB::e(j)), KY[j][e], ey);
          ea = fmaf(float(TB::e(j)), KA[j][e], ea);
        }
      ErY[e] = isnan(ey) ? INFINITY : ey;
      ErA[e] = isnan(ea) ? INFINITY : ea;
    }
    __syncthreads();  // every warp is past its last read of the stage operands
    if (P.controller == GBDX_PID) {
#pragma unroll
      for (int e = 0; e < NE; e++) {
        int row, col;
        elem_rc<SH>(e, warp, lane, row, col);
        if (isnan(Y1[e])) R.nan_y[row] = 1;
        if (isnan(A1[e])) R.nan_a[row] = 1;
      }
      __syncthreads();
#pragma unroll
      for (int j = 0; j < SH::TPW; j++) {
#pragma unroll
        for (int half = 0; half < 2; half++) {
          int row, col;
          elem_rc<SH>(j * 4 + half * 2, warp, lane, row, col);
          const bool ny = R.nan_y[row], na = R.nan_a[row];
          float part = 0.f;
#pragma unroll
          for (int q = 0; q < 2; q++) {
            const int e = j * 4 + half * 2 + q;
            const float my = fmaxf(fabsf(Y0[e]), fabsf(ny ? Y0[e] : Y1[e]));
            const float sy = __fdividef(ErY[e], fmaf(my, rtol, atol));
            const float ma = fmaxf(fabsf(A0[e]), fabsf(na ? A0[e] : A1[e]));
            const float sa = __fdividef(ErA[e], fmaf(ma, rtol, atol));
            part = fmaf(sy, sy, part);
            part = fmaf(sa, sa, part);
          }
          part += __shfl_xor_sync(0xffffffffu, part, 1);
          part += __shfl_xor_sync(0xffffffffu, part, 2);
          if ((lane & 3) == 0) R.part[row][(warp * SH::TPW + j) % SH::NT] = part;
        }
      }
      __syncthreads();
      if (tid < M && R.live[tid]) {
        float a = 0.f;
#pragma unroll
        for (int n = 0; n < SH::NT; n++) a += R.part[tid][n];
        R.acc[tid] = a;
      }
      __syncthreads();
      // the a_theta part of the norm: one parameter pass per live row
      if (Q.track) {
        if constexpr (PRECISE) {
          for (int r = 0; r < M; r++) {
            if (!R.live[r]) continue;
            const float *a0p = R.zero[r] ? nullptr : ath + (size_t(r) * 2 + R.cur[r]) * NP;
            float *a1p = ath + (size_t(r) * 2 + (R.cur[r] ^ 1)) * NP;
            const float s = theta_pass<SH, SOLVER, true>(sm.cf, rec + size_t(r) * REC, R.h[r],
                                                         a0p, a1p, psum, pcomp, rtol, atol, tid);
            const float tot = block_sum<SH>(sm.red, s, tid);
            if (tid == 0) R.acc[r] += tot;
          }
        } else {
          theta_rows_tc<SH, SOLVER, true>(
              sm.p, sm.rsum, rec, R.h, [&](int r) { return R.live[r] != 0; },
              [&](int r, const float *&a0p, float *&a1p) {
                a0p = R.zero[r] ? nullptr : ath + (size_t(r) * 2 + R.cur[r]) * NP;
                a1p = ath + (size_t(r) * 2 + (R.cur[r] ^ 1)) * NP;
              },
              rtol, atol, tid, warp, lane);
          if (tid < M && R.live[tid]) {
            float t = 0.f;
#pragma unroll
            for (int w = 0; w < SH::WARPS; w++) t += sm.rsum[w][tid];
            R.acc[tid] += t;
          }
        }
        __syncthreads();
      }
    }
    if (tid < M && R.live[tid]) bs_row_control(R, tid, Q.n_norm, P);
    __syncthreads();
    // untracked a_theta: add the accepted increments in place
    if (!Q.track) {
      if constexpr (PRECISE) {
        for (int r = 0; r < M; r++) {
          if (!(R.live[r] && R.keep[r])) continue;
          float *ap = ath + size_t(r) * 2 * NP;
          const float *a0p = R.zero[r] ? nullptr : ap;
          theta_pass<SH, SOLVER, false>(sm.cf, rec + size_t(r) * REC, R.h[r], a0p, ap, psum,
                                        pcomp, rtol, atol, tid);
        }
      } else {
        theta_rows_tc<SH, SOLVER, false>(
            sm.p, sm.rsum, rec, R.h, [&](int r) { return R.live[r] && R.keep[r]; },
            [&](int r, const float *&a0p, float *&a1p) {
              a1p = ath + size_t(r) * 2 * NP;
              a0p = R.zero[r] ? nullptr : a1p;
            },
            rtol, atol, tid, warp, lane);
      }
    }
    // ---- accept: state, FSAL vectors and records, a_theta buffers --------------
#pragma unroll
    for (int e = 0; e < NE; e++) {
      int row, col;
      elem_rc<SH>(e, warp, lane, row, col);
      if (R.live[row] && R.keep[row]) {
        Y0[e] = Y1[e];
        A0[e] = A1[e];
        if (TB::FSAL) {
          F0[e] = F[e];
          GY0[e] = GY[e];
        }
      }
    }
    if constexpr (TB::FSAL) {
      // the last stage's records become the next step's stage 0 (all rows at
      // once: independent loads)
      for (int f = tid * 4; f < M * REC; f += SH::THREADS * 4) {
        const int r = f / REC;
        if (R.live[r] && R.keep[r])
          *reinterpret_cast<float4 *>(rec + f) =
              *reinterpret_cast<const float4 *>(rec + size_t(S - 1) * M * REC + f);
      }
    }
    __syncthreads();
    if (tid < M && R.live[tid] && R.keep[tid]) {
      if (Q.track) R.cur[tid] ^= 1;
      R.zero[tid] = 0;
    }
    __syncthreads();
    transitions();
  }
}

}  // namespace gbdx
