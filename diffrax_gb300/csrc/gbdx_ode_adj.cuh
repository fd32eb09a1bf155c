// gbdx_ode_adj.cuh -- gradients of the analytic-field solves (Lotka-Volterra,
// Van der Pol, Ornstein-Uhlenbeck ODE and SDE) with respect to y0 and args.
//
// * RecursiveCheckpointAdjoint (diffrax/_adjoint.py:179-312): the reference
//   differentiates the discrete solve -- rejected steps get zero cotangent
//   (_integrate.py:422-424) and the controller is under stop_gradient
//   (pid.py:374, 499-501, 529-530) -- so the gradient is the VJP of the chain
//   of accepted steps on the realised time grid.  The forward (Traj with a
//   Taped field) records the time and state of every accepted step; at state
//   dimension <= 4 the whole tape is a few bytes per step, so nothing is
//   recomputed beyond the stages of the step being differentiated.  The
//   backward walks each trajectory's steps in reverse, one trajectory per
//   thread: interpolant VJP of the saves inside the step, then the reverse
//   stage loop with the field's hand-written VJP.
// * BacksolveAdjoint (_adjoint.py:538-734): per trajectory, reverse-time
//   solves of the augmented state z = (y, a, a_args) between adjacent saved
//   times, started from the saved y with a += dL/dys[j] (:646-650); the
//   augmented field is AdjointTerm.vf (_term.py:886-910): (f, -a^T df/dy,
//   -a^T df/dargs).  Solver and controller state carry over segments, every
//   segment starts with a fresh FSAL evaluation (made_jump) and with the
//   initial step of diffeqsolve given a controller state (_integrate.py:
//   1252-1265).  The error norm is rms over (y, a, a_args), or over (y, a)
//   under adjoint_rms_seminorm (_misc.py:85-116).
// The args gradient accumulates per trajectory with compensated (Kahan) sums.
#pragma once

#include "gbdx_backsolve.cuh"
#include "gbdx_traj.cuh"
#include "gbdx_vbt.cuh"

namespace gbdx {

// The field with the full gradient tape recorded by the forward kernel.
template <class F>
struct Taped : F {
  static constexpr bool TAPE = true;
};

// The local interpolant of one step as a linear map of (y0, y1, k_j):
// out = ay0 y0 + ay1 y1 + sum_j g_j k_j (tsit5.py:119-150,
// _local_interpolation.py:29-139).
template <int SOLVER, class T>
__device__ __forceinline__ void interp_coeffs_t(T th, T &ay0, T &ay1,
                                                T (&g)[Tab<SOLVER>::S]) {
  constexpr int S = Tab<SOLVER>::S;
#pragma unroll
  for (int j = 0; j < S; j++) g[j] = T(0);
  const T t2 = th * th, t3 = t2 * th, t4 = t3 * th;
  if constexpr (SOLVER == GBDX_TSIT5) {
    ay0 = T(1);
    ay1 = T(0);
#pragma unroll
    for (int j = 0; j < S; j++) g[j] = tsit5_w<T>(j, th);
  } else if constexpr (SOLVER == GBDX_DOPRI5) {
    const T Mm = T(16) * t4 - T(32) * t3 + T(16) * t2;
    ay0 = T(-8) * t4 + T(18) * t3 - T(11) * t2 + T(1) + Mm;
    ay1 = T(-8) * t4 + T(14) * t3 - T(5) * t2;
#pragma unroll
    for (int j = 0; j < S; j++) g[j] = Mm * T(Tab<GBDX_DOPRI5>::cmid(j));
    g[0] += T(-2) * t4 + T(5) * t3 - T(4) * t2 + th;
    g[6] += T(2) * t4 - T(3) * t3 + t2;
  } else if constexpr (SOLVER == GBDX_HEUN) {
    ay0 = T(2) * t3 - T(3) * t2 + T(1);
    ay1 = T(-2) * t3 + T(3) * t2;
    g[0] = t3 - T(2) * t2 + th;
    g[1] = t3 - t2;
  } else {
    ay0 = T(1) - th;
    ay1 = th;
  }
}

template <class T>
__device__ __forceinline__ void kahan_add_t(T &sum, T &comp, T x) {
  const T y = x - comp;
  const T t = sum + y;
  comp = (t - sum) - y;
  sum = t;
}

// ---------------------------------------------------------------------------
// RecursiveCheckpointAdjoint backward.
// ---------------------------------------------------------------------------
template <int SOLVER, class F, class T>
__global__ void __launch_bounds__(128) ode_rc_bwd_kernel(SolveParams P, AdjParams Q) {
  using TB = Tab<SOLVER>;
  constexpr int S = TB::S, D = F::D, NA = F::NARGS;
  // thread q takes the trajectory the forward took from queue slot q, whose
  // tape is row q (the forward's work order, when it had one): neighbouring
  // threads read neighbouring rows and have similar step counts
  const int64_t q = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= P.batch) return;
  const int64_t i = P.order ? int64_t(P.order[q]) : q;
  const int64_t ti = i * P.time_stride;
  const int dir = (P.t0[ti] < P.t1[ti]) ? 1 : -1;
  const double t0 = dir * P.t0[ti], t1 = dir * P.t1[ti];
  const int N = P.tape_n[q];
  const double *tt = P.tape_t + q * int64_t(P.max_steps + 1);
  const T *ty = reinterpret_cast<const T *>(P.tape_y) + q * int64_t(P.checkpoints) * D;
  const T *G = static_cast<const T *>(Q.grad_ys) + i * int64_t(P.n_save) * D;
  const T *ap = static_cast<const T *>(P.args) + i * P.args_stride;
  T a[NA];
#pragma unroll
  for (int p = 0; p < NA; p++) a[p] = ap[p];
  T gy[D], ga[NA], gc[NA];
#pragma unroll
  for (int n = 0; n < D; n++) gy[n] = T(0);
#pragma unroll
  for (int p = 0; p < NA; p++) ga[p] = gc[p] = T(0);
  // SaveAt(ts) points the forward reached (all of them unless max_steps
  // stopped it); the t1 save sits in the slot after them.
  int n_saved = 0;
  const double tN = *GBDX_AT(P, tt, N, 1, P.max_steps + 1, GBDX_SITE_TAPE_T);
  if (t0 == t1) {
    n_saved = P.n_ts;
    for (int m = 0; m < P.n_ts; m++)
#pragma unroll
      for (int n = 0; n < D; n++)
        gy[n] += GBDX_AT(P, G, (P.save_t0 + m) * D, D, P.n_save * D, GBDX_SITE_GRAD_YS)[n];
  } else {
    while (n_saved < P.n_ts && dir * P.save_ts[n_saved] <= tN) n_saved++;
  }
  if (P.save_t1)
#pragma unroll
    for (int n = 0; n < D; n++)
      gy[n] += GBDX_AT(P, G, (P.save_t0 + n_saved) * D, D, P.n_save * D, GBDX_SITE_GRAD_YS)[n];
  T ys[S][D], k[S][D], kbar[S][D], gy0[D], gy1[D], f[D], dw[D];
  int m_hi = t0 == t1 ? 0 : n_saved;  // saves not yet visited: [0, m_hi)
#pragma unroll 1
  for (int s = N - 1; s >= 0; s--) {
    const double *tp = GBDX_AT(P, tt, s, 2, P.max_steps + 1, GBDX_SITE_TAPE_T);
    const double ta = tp[0], tb = tp[1];
    const T *tys = GBDX_AT(P, ty, s * D, D, int64_t(P.checkpoints) * D, GBDX_SITE_TAPE_Y);
    const T h = T(dir * (tb - ta));  // the step's control
    if constexpr (F::SDE) {
#pragma unroll
      for (int n = 0; n < D; n += 2) {
        const float2 wa = vbt_w_pair(P, i, ta * dir, n), wb = vbt_w_pair(P, i, tb * dir, n);
        dw[n] = T(wb.x - wa.x);
        dw[n + 1] = T(wb.y - wa.y);
      }
    }
    // the stages of accepted step s from its start state (runge_kutta.py:
    // 1000-1160, explicit branch)
#pragma unroll
    for (int st = 0; st < S; st++) {
#pragma unroll
      for (int n = 0; n < D; n++) {
        T inc = T(0);
#pragma unroll
        for (int j = 0; j < st; j++)
          if (TB::a(st, j) != 0.0) inc += T(TB::a(st, j)) * k[j][n];
        ys[st][n] = tys[n] + inc;
      }
      F::vf(P, a, ys[st], f);
      if constexpr (F::SDE) {
        T sg[D];
        F::sigma(P, a, ys[st], sg);
#pragma unroll
        for (int n = 0; n < D; n++) k[st][n] = f[n] * h + sg[n] * dw[n];
      } else {
#pragma unroll
        for (int n = 0; n < D; n++) k[st][n] = f[n] * h;
      }
    }
#pragma unroll
    for (int st = 0; st < S; st++)
#pragma unroll
      for (int n = 0; n < D; n++) kbar[st][n] = T(0);
#pragma unroll
    for (int n = 0; n < D; n++) {
      gy0[n] = T(0);
      gy1[n] = gy[n];
    }
    // saves inside the step: (t_s, t_{s+1}], and [t_0, t_1] for the first
    int m_lo = m_hi;
    while (m_lo > 0 && (s == 0 || dir * P.save_ts[m_lo - 1] > ta)) m_lo--;
    for (int m = m_lo; m < m_hi; m++) {
      const double tsd = dir * P.save_ts[m];
      const T th = T(ta == tb ? 0.0 : (tsd - ta) / (tb - ta));
      T ay0, ay1, gw[S];
      interp_coeffs_t<SOLVER, T>(th, ay0, ay1, gw);
      const T *go = G + (P.save_t0 + m) * D;
#pragma unroll
      for (int n = 0; n < D; n++) {
        gy0[n] += ay0 * go[n];
        gy1[n] += ay1 * go[n];
#pragma unroll
        for (int j = 0; j < S; j++) kbar[j][n] += gw[j] * go[n];
      }
    }
    m_hi = m_lo;
    // y1 is the last stage input (SSAL) or y0 + sum_j b_j k_j
    if constexpr (!TB::SSAL) {
#pragma unroll
      for (int n = 0; n < D; n++) {
        gy0[n] += gy1[n];
#pragma unroll
        for (int j = 0; j < S; j++) kbar[j][n] += T(TB::b(j)) * gy1[n];
      }
    }
#pragma unroll
    for (int st = S - 1; st >= 0; st--) {
      T gyi[D], g[D], gat[NA];
#pragma unroll
      for (int n = 0; n < D; n++) {
        gyi[n] = (TB::SSAL && st == S - 1) ? gy1[n] : T(0);
        g[n] = kbar[st][n] * h;
      }
#pragma unroll
      for (int p = 0; p < NA; p++) gat[p] = T(0);
      F::vjp(a, ys[st], g, gyi, gat);
      if constexpr (F::SDE) F::sigma_vjp(a, ys[st], dw, kbar[st], gyi, gat);
#pragma unroll
      for (int p = 0; p < NA; p++) kahan_add_t(ga[p], gc[p], gat[p]);
#pragma unroll
      for (int n = 0; n < D; n++) {
        gy0[n] += gyi[n];
#pragma unroll
        for (int j = 0; j < st; j++)
          if (TB::a(st, j) != 0.0) kbar[j][n] += T(TB::a(st, j)) * gyi[n];
      }
    }
#pragma unroll
    for (int n = 0; n < D; n++) gy[n] = gy0[n];
  }
  if (P.save_t0)
#pragma unroll
    for (int n = 0; n < D; n++) gy[n] += G[n];
  T *oy = static_cast<T *>(Q.grad_y0) + i * D;
#pragma unroll
  for (int n = 0; n < D; n++) oy[n] = gy[n];
  T *oa = static_cast<T *>(Q.grad_args) + i * NA;
#pragma unroll
  for (int p = 0; p < NA; p++) oa[p] = ga[p] - gc[p];
}

// ---------------------------------------------------------------------------
// BacksolveAdjoint backward.
// ---------------------------------------------------------------------------

// The controller's decision in FP64 for the FP64-state backsolve: the PID
// update in the reference's operation order (pid.py:394-567) and the
// segment clip (_integrate.py:410-413); history in the linear domain.
__device__ __forceinline__ void bs_control_f64(BsRows<1> &R, double scaled, double &hist1,
                                               double &hist2, const SolveParams &P) {
  const double dt = R.dtc[0];
  bool keep;
  double nt0, nt1;
  if (P.controller == GBDX_PID) {
    keep = scaled < 1.0;
    if (P.has_dtmin) keep = keep || R.at_dtmin[0];
    double inv = 1.0 / scaled;
    const double f1 = (P.c1 == 0.0) ? 1.0 : pow(inv, P.c1);
    const double f2 = (P.c2 == 0.0) ? 1.0 : pow(hist1, P.c2);
    const double f3 = (P.c3 == 0.0) ? 1.0 : pow(hist2, P.c3);
    const double fmn = keep ? 1.0 : P.factormin;
    const double fmx = keep ? P.factormax : P.safety;
    double factor = P.safety * f1 * f2 * f3;
    factor = fmin(fmx, fmax(factor, fmn));
    double dtn = dt * factor;
    if (inv == 0.0 || isinf(inv)) inv = 1.0;
    if (P.has_dtmax) dtn = fmin(dtn, P.dtmax);
    if (P.has_dtmin) {
      if (!P.force_dtmin && dtn < P.dtmin && R.sres[0] == GBDX_SUCCESSFUL)
        R.sres[0] = GBDX_DT_MIN_REACHED;
      if (R.at_dtmin[0] && factor == 1.0) dtn = P.dtmin;
      R.at_dtmin[0] = dtn <= P.dtmin;
      dtn = fmax(dtn, P.dtmin);
    }
    nt0 = keep ? R.tnext[0] : R.tprev[0];
    nt1 = nt0 + dtn;
    if (keep) {
      hist2 = hist1;
      hist1 = inv;
    }
  } else {
    keep = true;
    const int s2 = R.sc[0] + 1;
    double tn = grid_time(R.t0s[0], R.t1s[0], s2, R.nc[0], R.ginv[0]);
    if (s2 == R.nc[0]) tn = R.t1s[0];
    R.sc[0] = s2;
    nt0 = R.tnext[0];
    nt1 = tn;
  }
  if (!(nt0 < R.te[0])) nt0 = R.te[0];
  if (order_key(nt1) > order_key(R.floor_te[0]))
    nt1 = keep ? R.te[0] : nt0 + 0.5 * (R.te[0] - nt0);
  R.keep[0] = keep;
  if (keep) {
    R.nacc[0]++;
    R.first[0] = 0;
  } else {
    R.nrej[0]++;
  }
  R.nsteps[0]++;
  R.nseg[0]++;
  R.tprev[0] = nt0;
  R.tnext[0] = nt1;
  R.dtc[0] = nt1 - nt0;
}

// AdjointTerm.vf: (f(y), -a^T df/dy, -a^T df/dargs) at (y, a).
template <class F, class T>
__device__ __forceinline__ void adjoint_vf(const SolveParams &P, const T *args, const T *y,
                                           const T *av, T *fy, T *fa, T *faa) {
  constexpr int D = F::D, NA = F::NARGS;
  F::vf(P, args, y, fy);
#pragma unroll
  for (int n = 0; n < D; n++) fa[n] = T(0);
#pragma unroll
  for (int p = 0; p < NA; p++) faa[p] = T(0);
  F::vjp(args, y, av, fa, faa);
#pragma unroll
  for (int n = 0; n < D; n++) fa[n] = -fa[n];
#pragma unroll
  for (int p = 0; p < NA; p++) faa[p] = -faa[p];
}

template <class T>
__device__ __forceinline__ T scaled_err(T e, T z0, T z1, T rtol, T atol) {
  const T m = fmax(Math<T>::abs_(z0), Math<T>::abs_(z1));
  const T s = e / (atol + m * rtol);
  return s * s;
}

template <int SOLVER, class F, class T>
__global__ void __launch_bounds__(128) ode_bs_kernel(SolveParams P, AdjParams Q) {
  using TB = Tab<SOLVER>;
  constexpr int S = TB::S, D = F::D, NA = F::NARGS;
  constexpr bool F64 = sizeof(T) == 8;
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= P.batch) return;
  const T rtol = T(P.rtol), atol = T(P.atol);
  BsRows<1> R;
  const int64_t ti = i * P.time_stride;
  R.idx[0] = i;
  R.dir[0] = (P.t0[ti] < P.t1[ti]) ? -1 : 1;  // every segment runs against the forward
  R.jold[0] = P.n_save;
  R.firstseg[0] = 1;
  R.nsteps[0] = R.nacc[0] = R.nrej[0] = 0;
  R.sres[0] = GBDX_SUCCESSFUL;
  R.at_dtmin[0] = 0;
  double hist1 = 1.0, hist2 = 1.0;  // FP64 PID history (pid.py:388-392)
  const int n_norm = Q.track_args ? 2 * D + NA : 2 * D;
  const T *ap = static_cast<const T *>(P.args) + i * P.args_stride;
  T args[NA];
#pragma unroll
  for (int p = 0; p < NA; p++) args[p] = ap[p];
  const T *G = static_cast<const T *>(Q.grad_ys) + i * int64_t(P.n_save) * D;
  const T *Ys = static_cast<const T *>(Q.ys) + i * int64_t(P.n_save) * D;
  T y[D], av[D], aa[NA];
#pragma unroll
  for (int n = 0; n < D; n++) av[n] = T(0);
#pragma unroll
  for (int p = 0; p < NA; p++) aa[p] = T(0);
  int result = GBDX_SUCCESSFUL;
  T ky[S][D], ka[S][D], kaa[S][NA];
  T f0y[D], f0a[D], f0aa[NA], fny[D], fna[D], fnaa[NA];
  while (true) {
    // next non-empty segment; a += dL/dys of every save passed
    bs_next_segment(R, 0, P);
    const int jn = R.seg[0] > 0 ? R.seg[0] : 0;
    for (int jj = jn; jj < R.jold[0]; jj++)
#pragma unroll
      for (int n = 0; n < D; n++)
        av[n] += GBDX_AT(P, G, jj * D, D, P.n_save * D, GBDX_SITE_GRAD_YS)[n];
    if (R.done[0]) break;
#pragma unroll
    for (int n = 0; n < D; n++)
      y[n] = GBDX_AT(P, Ys, R.seg[0] * D, D, P.n_save * D, GBDX_SITE_GRAD_YS)[n];
    R.active[0] = 1;
    bool have_f0 = false;  // made_jump: the segment's first step evaluates f afresh
    while (bs_running(R, 0, P.max_steps)) {
      const double dt = R.dtc[0];
      const T h = T(R.dir[0] > 0 ? dt : -dt);
      T zy[D], za[D];
#pragma unroll
      for (int st = 0; st < S; st++) {
#pragma unroll
        for (int n = 0; n < D; n++) {
          T iy = T(0), ia = T(0);
#pragma unroll
          for (int j = 0; j < st; j++)
            if (TB::a(st, j) != 0.0) {
              iy += T(TB::a(st, j)) * ky[j][n];
              ia += T(TB::a(st, j)) * ka[j][n];
            }
          zy[n] = y[n] + iy;
          za[n] = av[n] + ia;
        }
        T fy[D], fa[D], faa[NA];
        if (TB::FSAL && st == 0 && have_f0) {
#pragma unroll
          for (int n = 0; n < D; n++) {
            fy[n] = f0y[n];
            fa[n] = f0a[n];
          }
#pragma unroll
          for (int p = 0; p < NA; p++) faa[p] = f0aa[p];
        } else {
          adjoint_vf<F, T>(P, args, zy, za, fy, fa, faa);
        }
        if (TB::FSAL && st == S - 1) {
#pragma unroll
          for (int n = 0; n < D; n++) {
            fny[n] = fy[n];
            fna[n] = fa[n];
          }
#pragma unroll
          for (int p = 0; p < NA; p++) fnaa[p] = faa[p];
        }
#pragma unroll
        for (int n = 0; n < D; n++) {
          ky[st][n] = fy[n] * h;
          ka[st][n] = fa[n] * h;
        }
#pragma unroll
        for (int p = 0; p < NA; p++) kaa[st][p] = faa[p] * h;
      }
      // proposal and embedded error (_integrate.py:386: NaN -> inf)
      T y1[D], a1[D], aa1[NA], ey[D], ea[D], eaa[NA];
#pragma unroll
      for (int n = 0; n < D; n++) {
        if constexpr (TB::SSAL) {
          y1[n] = zy[n];
          a1[n] = za[n];
        } else {
          T iy = T(0), ia = T(0);
#pragma unroll
          for (int j = 0; j < S; j++) {
            iy += T(TB::b(j)) * ky[j][n];
            ia += T(TB::b(j)) * ka[j][n];
          }
          y1[n] = y[n] + iy;
          a1[n] = av[n] + ia;
        }
        T e1 = T(0), e2 = T(0);
#pragma unroll
        for (int j = 0; j < S; j++) {
          e1 += T(TB::e(j)) * ky[j][n];
          e2 += T(TB::e(j)) * ka[j][n];
        }
        ey[n] = isnan(e1) ? T(INFINITY) : e1;
        ea[n] = isnan(e2) ? T(INFINITY) : e2;
      }
#pragma unroll
      for (int p = 0; p < NA; p++) {
        T ip = T(0), e3 = T(0);
#pragma unroll
        for (int j = 0; j < S; j++) {
          ip += T(TB::b(j)) * kaa[j][p];
          e3 += T(TB::e(j)) * kaa[j][p];
        }
        aa1[p] = aa[p] + ip;
        eaa[p] = isnan(e3) ? T(INFINITY) : e3;
      }
      if (P.controller == GBDX_PID) {
        // rms over the leaves y, a (and a_args); a leaf with a NaN in its
        // proposal is measured against its old value (pid.py:475-481)
        bool ny = false, na = false, naa = false;
#pragma unroll
        for (int n = 0; n < D; n++) {
          ny |= isnan(y1[n]);
          na |= isnan(a1[n]);
        }
#pragma unroll
        for (int p = 0; p < NA; p++) naa |= isnan(aa1[p]);
        T acc = T(0);
#pragma unroll
        for (int n = 0; n < D; n++) acc += scaled_err(ey[n], y[n], ny ? y[n] : y1[n], rtol, atol);
#pragma unroll
        for (int n = 0; n < D; n++) acc += scaled_err(ea[n], av[n], na ? av[n] : a1[n], rtol, atol);
        if (Q.track_args)
#pragma unroll
          for (int p = 0; p < NA; p++)
            acc += scaled_err(eaa[p], aa[p], naa ? aa[p] : aa1[p], rtol, atol);
        if constexpr (F64) {
          bs_control_f64(R, sqrt(double(acc)) / sqrt(double(n_norm)), hist1, hist2, P);
        } else {
          R.acc[0] = float(acc);
          bs_row_control(R, 0, float(n_norm), P);
        }
      } else {
        if constexpr (F64) {
          bs_control_f64(R, 0.0, hist1, hist2, P);
        } else {
          R.acc[0] = 0.f;
          bs_row_control(R, 0, float(n_norm), P);
        }
      }
      if (R.keep[0]) {
#pragma unroll
        for (int n = 0; n < D; n++) {
          y[n] = y1[n];
          av[n] = a1[n];
        }
#pragma unroll
        for (int p = 0; p < NA; p++) aa[p] = aa1[p];
        if (TB::FSAL) {
          // the solver state of a rejected step is kept (_integrate.py:424)
#pragma unroll
          for (int n = 0; n < D; n++) {
            f0y[n] = fny[n];
            f0a[n] = fna[n];
          }
#pragma unroll
          for (int p = 0; p < NA; p++) f0aa[p] = fnaa[p];
          have_f0 = true;
        }
      }
    }
    int sres = R.sres[0];
    if (sres == GBDX_SUCCESSFUL && order_key(R.tprev[0]) < order_key(R.te[0]))
      sres = GBDX_MAX_STEPS_REACHED;
    if (result == GBDX_SUCCESSFUL) result = sres;
    R.jold[0] = R.seg[0];
  }
  T *oy = static_cast<T *>(Q.grad_y0) + i * D;
#pragma unroll
  for (int n = 0; n < D; n++) oy[n] = av[n];
  T *oa = static_cast<T *>(Q.grad_args) + i * NA;
#pragma unroll
  for (int p = 0; p < NA; p++) oa[p] = aa[p];
  P.result_out[i] = result;
  P.stats_out[i * 3 + 0] = R.nsteps[0];
  P.stats_out[i * 3 + 1] = R.nacc[0];
  P.stats_out[i * 3 + 2] = R.nrej[0];
}

}  // namespace gbdx
