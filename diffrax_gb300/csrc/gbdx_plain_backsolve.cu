// gbdx_plain_backsolve.cu -- the plain form of the BacksolveAdjoint backward
// for MLP fields: one trajectory per thread, FP32 on the CUDA cores.  Each
// thread integrates the augmented state (y, a, a_theta) of its trajectory
// backwards between the saved times (diffrax/_adjoint.py:572-734) with the
// same solver, controller, segment and norm rules as the fused kernel
// (gbdx_backsolve.cuh), but the straightforward way: every stage evaluates
// the MLP and its VJP on the CUDA cores and adds b_j K_j and e_j K_j of the
// parameter part into per-trajectory accumulators in HBM; the step's a_theta
// candidate and error norm are then formed from them.  a_theta and the two
// accumulators are [n_params][batch] arrays (coalesced across a warp); the
// final a_theta columns are reduced over the batch with compensation.  It is
// the baseline the fused row-tile backsolve is compared against.
#include "gbdx_backsolve.cuh"
#include "gbdx_launch.h"
#include "gbdx_mlp_plain.cuh"

namespace gbdx {

namespace {

template <int SOLVER, class FIELD>
__global__ void __launch_bounds__(128) plain_backsolve_kernel(SolveParams P, BsParams Q) {
  using TB = Tab<SOLVER>;
  constexpr int S = TB::S, D = FIELD::D, NP = FIELD::NP;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= P.batch) return;
  const int64_t B = P.batch;
  // per-trajectory columns: a_theta, sum_j b_j K_j, sum_j e_j K_j
  float *ath = Q.ath + i, *sb = Q.ath + int64_t(NP) * B + i, *se = Q.ath + 2 * int64_t(NP) * B + i;
  const float *W = P.mlp;
  const float rtol = float(P.rtol), atol = float(P.atol);
  BsRows<1> R;
  const int64_t ti = i * P.time_stride;
  R.idx[0] = i;
  R.dir[0] = (P.t0[ti] < P.t1[ti]) ? -1 : 1;
  R.jold[0] = P.n_save;
  R.firstseg[0] = 1;
  R.nsteps[0] = R.nacc[0] = R.nrej[0] = 0;
  int result = GBDX_SUCCESSFUL;
  bool zero = true;  // a_theta is still zero (nothing accepted yet)
  float y[D], a[D], ky[S][D], ka[S][D], yi[D], ai[D], f[D], gy[D], none[D];
  for (int n = 0; n < D; n++) a[n] = 0.f;
  const float *G = Q.grad_ys + i * int64_t(P.n_save) * D;
  const float *Ys = Q.ys + i * int64_t(P.n_save) * D;
  while (true) {
    // next non-empty segment; a += dL/dys of every save passed
    bs_next_segment(R, 0, P);
    const int jn = R.seg[0] > 0 ? R.seg[0] : 0;
    for (int jj = jn; jj < R.jold[0]; jj++)
      for (int n = 0; n < D; n++) a[n] += G[jj * D + n];
    if (R.done[0]) break;
    for (int n = 0; n < D; n++) y[n] = Ys[R.seg[0] * D + n];
    R.active[0] = 1;
    while (bs_running(R, 0, P.max_steps)) {
      const double dt = R.dtc[0];
      const float h = float(R.dir[0] > 0 ? dt : -dt);
      for (int st = 0; st < S; st++) {
        for (int n = 0; n < D; n++) {
          float p = y[n], q = a[n];
          for (int j = 0; j < st; j++)
            if (TB::a(st, j) != 0.0) {
              p = fmaf(float(TB::a(st, j)), ky[j][n], p);
              q = fmaf(float(TB::a(st, j)), ka[j][n], q);
            }
          yi[n] = p;
          ai[n] = q;
          gy[n] = 0.f;
        }
        FIELD::vf(P, nullptr, yi, f);
        const float cb = -h * float(TB::b(st)), ce = -h * float(TB::e(st));
        if (st == 0)
          FIELD::vjp_with(W, yi, ai, none, gy, [&](int p, float v) {
            sb[p * B] = cb * v;
            se[p * B] = ce * v;
          });
        else
          FIELD::vjp_with(W, yi, ai, none, gy, [&](int p, float v) {
            sb[p * B] += cb * v;
            se[p * B] += ce * v;
          });
        for (int n = 0; n < D; n++) {
          ky[st][n] = f[n] * h;
          ka[st][n] = -gy[n] * h;
        }
      }
      float y1[D], a1[D], ey[D], ea[D];
      for (int n = 0; n < D; n++) {
        if constexpr (TB::SSAL) {
          y1[n] = yi[n];
          a1[n] = ai[n];
        } else {
          float p = y[n], q = a[n];
          for (int j = 0; j < S; j++) {
            p = fmaf(float(TB::b(j)), ky[j][n], p);
            q = fmaf(float(TB::b(j)), ka[j][n], q);
          }
          y1[n] = p;
          a1[n] = q;
        }
        float e1 = 0.f, e2 = 0.f;
        for (int j = 0; j < S; j++) {
          e1 = fmaf(float(TB::e(j)), ky[j][n], e1);
          e2 = fmaf(float(TB::e(j)), ka[j][n], e2);
        }
        ey[n] = isnan(e1) ? INFINITY : e1;
        ea[n] = isnan(e2) ? INFINITY : e2;
      }
      float acc = 0.f;
      if (P.controller == GBDX_PID) {
        bool ny = false, na = false;
        for (int n = 0; n < D; n++) {
          ny |= isnan(y1[n]);
          na |= isnan(a1[n]);
        }
        for (int n = 0; n < D; n++) {
          const float my = fmaxf(fabsf(y[n]), fabsf(ny ? y[n] : y1[n]));
          const float sy = __fdividef(ey[n], fmaf(my, rtol, atol));
          const float ma = fmaxf(fabsf(a[n]), fabsf(na ? a[n] : a1[n]));
          const float sa = __fdividef(ea[n], fmaf(ma, rtol, atol));
          acc = fmaf(sy, sy, acc);
          acc = fmaf(sa, sa, acc);
        }
        if (Q.track)
          for (int p = 0; p < NP; p++) {
            const float x0 = zero ? 0.f : ath[p * B];
            acc += scaled_sq(x0, x0 + sb[p * B], se[p * B], rtol, atol);
          }
      }
      R.acc[0] = acc;
      bs_row_control(R, 0, Q.n_norm, P);
      if (R.keep[0]) {
        for (int n = 0; n < D; n++) {
          y[n] = y1[n];
          a[n] = a1[n];
        }
        for (int p = 0; p < NP; p++) ath[p * B] = (zero ? 0.f : ath[p * B]) + sb[p * B];
        zero = false;
      }
    }
    int sres = R.sres[0];
    if (sres == GBDX_SUCCESSFUL && order_key(R.tprev[0]) < order_key(R.te[0]))
      sres = GBDX_MAX_STEPS_REACHED;
    if (result == GBDX_SUCCESSFUL) result = sres;
    R.jold[0] = R.seg[0];
  }
  if (zero)
    for (int p = 0; p < NP; p++) ath[p * B] = 0.f;
  for (int n = 0; n < D; n++) Q.grad_y0[i * D + n] = a[n];
  P.result_out[i] = result;
  P.stats_out[i * 3 + 0] = R.nsteps[0];
  P.stats_out[i * 3 + 1] = R.nacc[0];
  P.stats_out[i * 3 + 2] = R.nrej[0];
}

template <int SOLVER, class FIELD>
cudaError_t launch_plain_backsolve(const SolveParams &P, const BsParams &Q, int,
                                   cudaStream_t s) {
  if (P.batch <= 0) return cudaSuccess;
  plain_backsolve_kernel<SOLVER, FIELD><<<unsigned((P.batch + 127) / 128), 128, 0, s>>>(P, Q);
  return cudaGetLastError();
}

cudaError_t occupancy_plain(int *ctas) {
  *ctas = 1;
  return cudaSuccess;
}

}  // namespace

BsEntry find_plain_backsolve_entry(int solver, int D, int H) {
  using C4 = MlpPlainField<64, 256, false>;
  if (D == 64 && H == 256 && solver == GBDX_TSIT5)
    return BsEntry{&launch_plain_backsolve<GBDX_TSIT5, C4>, &occupancy_plain, 1, Tab<GBDX_TSIT5>::S,
                   0, 0};
  return BsEntry{nullptr, nullptr, 0, 0, 0, 0};
}

}  // namespace gbdx
