// gbdx_plain_bwd.cu -- the plain form of the RecursiveCheckpointAdjoint
// backward for MLP fields: one trajectory per thread, FP32 on the CUDA cores.
// The plain forward records the full tape (every accepted step's time and
// state); here each thread walks its steps in reverse, recomputes the stages
// and applies the exact VJP of the step (interpolant VJP of the saves inside
// it, then the reverse stage loop), as the reference's discretise-then-optimise
// gradient (diffrax/_adjoint.py:179-312) prescribes.  Parameter cotangents are
// added to a per-trajectory column of dP [n_params][batch] and reduced over
// the batch (compensated) at the end.  It is the baseline the fused row-tile
// backward (gbdx_mlp_bwd.cuh) is compared against.
#include "gbdx_launch.h"
#include "gbdx_mlp_bwd.cuh"
#include "gbdx_mlp_plain.cuh"
#include "gbdx_vbt.cuh"

namespace gbdx {

namespace {

template <int SOLVER, class FIELD>
__global__ void __launch_bounds__(128) plain_bwd_kernel(SolveParams P, BwdParams Q) {
  using TB = Tab<SOLVER>;
  constexpr int S = TB::S, D = FIELD::D;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= P.batch) return;
  const int64_t ti = i * P.time_stride;
  const int dir = (P.t0[ti] < P.t1[ti]) ? 1 : -1;
  const double t0 = dir * P.t0[ti], t1 = dir * P.t1[ti];
  const int N = P.tape_n[i];
  const double *tt = P.tape_t + i * int64_t(P.max_steps + 1);
  const float *ty = P.tape_y + i * int64_t(P.checkpoints) * D;
  const float *G = Q.grad_ys + i * int64_t(P.n_save) * D;
  float *dP = Q.part_sum + i;
  const int64_t stride = P.batch;
  const float *W = P.mlp;
  float gy[D];
#pragma unroll 1
  for (int n = 0; n < D; n++) gy[n] = 0.f;
  // ts saved: those <= the last accepted time (all of them unless max_steps
  // stopped the solve); the t1 save sits in the next slot
  int n_saved = 0;
  const double tN = tt[N];
  if (t0 == t1) {
    n_saved = P.n_ts;
    for (int m = 0; m < P.n_ts; m++)
      for (int n = 0; n < D; n++) gy[n] += G[(P.save_t0 + m) * D + n];
  } else {
    while (n_saved < P.n_ts && dir * P.save_ts[n_saved] <= tN) n_saved++;
  }
  if (P.save_t1)
    for (int n = 0; n < D; n++) gy[n] += G[(P.save_t0 + n_saved) * D + n];
  float ys[S][D], k[S][D], kbar[S][D], gy0[D], gy1[D], g[D], gs[D], dw[D], sg[D], f[D];
  int m_hi = t0 == t1 ? 0 : n_saved;  // saves not yet visited: [0, m_hi)
#pragma unroll 1
  for (int s = N - 1; s >= 0; s--) {
    const double ta = tt[s], tb = tt[s + 1];
    const float h = float(dir * (tb - ta));
    // recompute the stages of accepted step s from its start state
    if constexpr (FIELD::SDE) {
      for (int n = 0; n < D; n += 2) {
        const float2 wa = vbt_w_pair(P, i, ta * dir, n), wb = vbt_w_pair(P, i, tb * dir, n);
        dw[n] = wb.x - wa.x;
        dw[n + 1] = wb.y - wa.y;
      }
    }
#pragma unroll 1
    for (int st = 0; st < S; st++) {
      for (int n = 0; n < D; n++) {
        float acc = ty[s * D + n];
        for (int j = 0; j < st; j++)
          if (TB::a(st, j) != 0.0) acc = fmaf(float(TB::a(st, j)), k[j][n], acc);
        ys[st][n] = acc;
      }
      FIELD::vf(P, nullptr, ys[st], f);
      if constexpr (FIELD::SDE) {
        FIELD::sigma(P, nullptr, ys[st], sg);
        for (int n = 0; n < D; n++) k[st][n] = f[n] * h + sg[n] * dw[n];
      } else {
        for (int n = 0; n < D; n++) k[st][n] = f[n] * h;
      }
    }
    for (int st = 0; st < S; st++)
      for (int n = 0; n < D; n++) kbar[st][n] = 0.f;
    for (int n = 0; n < D; n++) {
      gy0[n] = 0.f;
      gy1[n] = gy[n];
    }
    // saves inside the step: (t_s, t_{s+1}], and [t_0, t_1] for the first
    int m_lo = m_hi;
    while (m_lo > 0 && (s == 0 || dir * P.save_ts[m_lo - 1] > ta)) m_lo--;
    for (int m = m_lo; m < m_hi; m++) {
      const double tsd = dir * P.save_ts[m];
      const float th = float(ta == tb ? 0.0 : (tsd - ta) / (tb - ta));
      float ay0, ay1, gw[7];
      interp_coeffs<SOLVER>(th, ay0, ay1, gw);
      const float *go = G + (P.save_t0 + m) * D;
      for (int n = 0; n < D; n++) {
        gy0[n] += ay0 * go[n];
        gy1[n] += ay1 * go[n];
        for (int j = 0; j < S; j++) kbar[j][n] += gw[j] * go[n];
      }
    }
    m_hi = m_lo;
    // y1 = last stage input (SSAL) or y0 + sum_j b_j k_j
    if constexpr (!TB::SSAL) {
      for (int n = 0; n < D; n++) {
        gy0[n] += gy1[n];
        for (int j = 0; j < S; j++) kbar[j][n] += float(TB::b(j)) * gy1[n];
      }
    }
#pragma unroll 1
    for (int st = S - 1; st >= 0; st--) {
      float gyi[D];
      for (int n = 0; n < D; n++) {
        gyi[n] = (TB::SSAL && st == S - 1) ? gy1[n] : 0.f;
        g[n] = kbar[st][n] * h;
        if constexpr (FIELD::SDE) gs[n] = kbar[st][n] * dw[n];
      }
      FIELD::vjp(W, ys[st], g, gs, gyi, dP, stride);
      for (int n = 0; n < D; n++) {
        gy0[n] += gyi[n];
        for (int j = 0; j < st; j++)
          if (TB::a(st, j) != 0.0) kbar[j][n] += float(TB::a(st, j)) * gyi[n];
      }
    }
    for (int n = 0; n < D; n++) gy[n] = gy0[n];
  }
  if (P.save_t0)
    for (int n = 0; n < D; n++) gy[n] += G[n];
  for (int n = 0; n < D; n++) Q.grad_y0[i * D + n] = gy[n];
}

// out[p] = sum over the batch of dP[p][:] (Kahan), one warp per parameter.
__global__ void reduce_columns_kernel(const float *dP, int64_t n_params, int64_t batch,
                                      float *out) {
  const int64_t p = int64_t(blockIdx.x) * (blockDim.x / 32) + (threadIdx.x >> 5);
  if (p >= n_params) return;
  const int lane = threadIdx.x & 31;
  float s = 0.f, c = 0.f;
  for (int64_t b = lane; b < batch; b += 32) kahan_add(&s, &c, dP[p * batch + b]);
  s -= c;
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) out[p] = s;
}

template <int SOLVER, class FIELD>
cudaError_t launch_plain_bwd(const SolveParams &P, const BwdParams &Q, int, cudaStream_t s) {
  if (P.batch <= 0) return cudaSuccess;
  plain_bwd_kernel<SOLVER, FIELD><<<unsigned((P.batch + 127) / 128), 128, 0, s>>>(P, Q);
  return cudaGetLastError();
}

cudaError_t occupancy_one(int *ctas) {
  *ctas = 1;
  return cudaSuccess;
}

}  // namespace

cudaError_t launch_reduce_columns(const float *dP, int64_t n_params, int64_t batch, float *out,
                                  cudaStream_t s) {
  if (n_params <= 0) return cudaSuccess;
  reduce_columns_kernel<<<unsigned((n_params + 7) / 8), 256, 0, s>>>(dP, n_params, batch, out);
  return cudaGetLastError();
}

BwdEntry find_mlp_plain_bwd_entry(int solver, int D, int H, bool sde) {
  using C3 = MlpPlainField<64, 128, false>;
  using C5 = MlpPlainField<32, 64, true>;
  if (!sde && D == 64 && H == 128 && solver == GBDX_TSIT5)
    return BwdEntry{&launch_plain_bwd<GBDX_TSIT5, C3>, &occupancy_one};
  if (sde && D == 32 && H == 64 && solver == GBDX_HEUN)
    return BwdEntry{&launch_plain_bwd<GBDX_HEUN, C5>, &occupancy_one};
  return BwdEntry{nullptr, nullptr};
}

}  // namespace gbdx
