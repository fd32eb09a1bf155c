// gbdx_traj.cuh -- one trajectory of a vmapped diffeqsolve, held in registers.
//
// Traj<SOLVER, FIELD, T>::step() is one iteration of the reference's outer
// while-loop body (diffrax/_integrate.py:365-662): an explicit RK step (or,
// for the additive-noise SRKs, the stochastic step of srk.py:335-671), the
// NaN->inf error guard (:386), the controller (pid.py:394-567 or
// constant.py:59-104), clip-to-end (:410-413, 278-284), the keep/reject select
// (:422-430), the step counters (:433-437) and the SaveAt(ts) loop (:456-487).
// init() follows diffeqsolve's set-up (:1036-1305) and finish() the t1 save and
// max_steps_reached result (:847-883).
#pragma once

#include "gbdx_common.cuh"
#include "gbdx_f64i.cuh"
#include "gbdx_vbt.cuh"

namespace gbdx {

// 1/x to the MUFU reciprocal's accuracy (the reciprocal inside __fdividef),
// for normal x.
__device__ __forceinline__ float rcp_approx(float x) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
  return r;
}

template <class T>
__device__ __forceinline__ T tsit5_w(int j, T t) {
  // Tsit5 dense-output weights b_j(theta) (tsit5.py:119-150).
  switch (j) {
    case 0:
      return T(-1.0530884977290216) * t * (t - T(1.3299890189751412)) *
             (t * t - T(1.4364028541716351) * t + T(0.7139816917074209));
    case 1:
      return T(0.1017) * t * t * (t * t - T(2.1966568338249754) * t + T(1.2949852507374631));
    case 2:
      return T(2.490627285651252793) * t * t *
             (t * t - T(2.38535645472061657) * t + T(1.57803468208092486));
    case 3:
      return T(-16.54810288924490272) * (t - T(1.21712927295533244)) *
             (t - T(0.61620406037800089)) * t * t;
    case 4:
      return T(47.37952196281928122) * (t - T(1.203071208372362603)) *
             (t - T(0.658047292653547382)) * t * t;
    case 5:
      return T(-34.87065786149660974) * (t - T(1.2)) * (t - T(0.666666666666666667)) * t * t;
    default:
      return T(2.5) * (t - T(1)) * (t - T(0.6)) * t * t;
  }
}

// Dopri8 dense-output weights theta P_j(theta) and their theta-derivative
// P_j + theta P_j' (Tab<GBDX_DOPRI8>::p, dopri8.py:192-303).
template <class T>
__device__ __forceinline__ T dopri8_w(int j, T t) {
  using TB = Tab<GBDX_DOPRI8>;
  const T p = ((((T(TB::p(j, 0)) * t + T(TB::p(j, 1))) * t + T(TB::p(j, 2))) * t +
                T(TB::p(j, 3))) * t + T(TB::p(j, 4))) * t + T(TB::p(j, 5));
  return t * p;
}
template <class T>
__device__ __forceinline__ T dopri8_dw(int j, T t) {
  using TB = Tab<GBDX_DOPRI8>;
  const T p = ((((T(TB::p(j, 0)) * t + T(TB::p(j, 1))) * t + T(TB::p(j, 2))) * t +
                T(TB::p(j, 3))) * t + T(TB::p(j, 4))) * t + T(TB::p(j, 5));
  const T dp = (((T(5 * TB::p(j, 0)) * t + T(4 * TB::p(j, 1))) * t + T(3 * TB::p(j, 2))) * t +
                T(2 * TB::p(j, 3))) * t + T(TB::p(j, 4));
  return p + t * dp;
}

// d/dtheta of the Tsit5 dense-output weights b_j(theta) of tsit5_w (product
// rule on the same factored polynomials).
template <class T>
__device__ __forceinline__ T tsit5_dw(int j, T t) {
  auto quad = [](T c, T a, T e, T t) {  // c t^2 (t^2 - a t + e)
    const T q = t * t - a * t + e;
    return c * (T(2) * t * q + t * t * (T(2) * t - a));
  };
  auto cub = [](T c, T a, T b, T t) {  // c (t - a)(t - b) t^2
    const T u = t - a, v = t - b;
    return c * (v * t * t + u * t * t + T(2) * t * u * v);
  };
  switch (j) {
    case 0: {  // c t (t - a)(t^2 - p t + q)
      const T c = T(-1.0530884977290216), a = T(1.3299890189751412);
      const T p = T(1.4364028541716351), q = T(0.7139816917074209);
      const T g = t * t - p * t + q;
      return c * ((t - a) * g + t * g + t * (t - a) * (T(2) * t - p));
    }
    case 1: return quad(T(0.1017), T(2.1966568338249754), T(1.2949852507374631), t);
    case 2:
      return quad(T(2.490627285651252793), T(2.38535645472061657), T(1.57803468208092486), t);
    case 3:
      return cub(T(-16.54810288924490272), T(1.21712927295533244), T(0.61620406037800089), t);
    case 4:
      return cub(T(47.37952196281928122), T(1.203071208372362603), T(0.658047292653547382), t);
    case 5: return cub(T(-34.87065786149660974), T(1.2), T(0.666666666666666667), t);
    default: return cub(T(2.5), T(1), T(0.6), t);
  }
}

// ClipStepSizeController (diffrax/_step_size_controller/clip.py) works in the
// loop's direction-flipped time, where the caller's sorted times become
// sort(ts * direction) (clip.py:203-213).  clip_get is the i-th of those, +inf
// past the end (_get_t, clip.py:55-62); clip_find the first index whose time
// is strictly greater than t, searched from a hint (_find_idx_with_hint,
// clip.py:102-118).
// The comparisons run on order keys (integer pipes; GB300 issues FP64
// compares at ~1/64 of the FP32 rate), with -0 keyed as +0 so that key
// equality and order are the FP64 ones; the sign flip is an integer XOR.
__device__ __forceinline__ long long ckey(double x) {
  const long long k = order_key(x);
  return k == -1 ? 0 : k;
}
__device__ __forceinline__ double clip_get(const double *ts, int n, int i, int dir) {
  if (i >= n) return INFINITY;
  if (dir > 0) return __ldg(ts + i);
  return __longlong_as_double(__double_as_longlong(__ldg(ts + n - 1 - i)) ^
                              (long long)0x8000000000000000ULL);
}
__device__ __forceinline__ int clip_find(const double *ts, int n, int dir, double t, int hint) {
  const long long kt = ckey(t);
  int i = hint;
  while (i < n && ckey(clip_get(ts, n, i, dir)) <= kt) i++;
  while (i > 0 && ckey(clip_get(ts, n, i - 1, dir)) > kt) i--;
  return i;
}

// ClipStepSizeController.init (clip.py:215-276): the first step ends no
// later than the first step time after t0, and just before the first jump.
// sidx / jidx: the trajectory's search hints into step_ts / jump_ts.
__device__ __forceinline__ double clip_start(const SolveParams &P, int dir, int &sidx,
                                             int &jidx, double a, double tn) {
  sidx = jidx = 0;
  if (P.n_step_ts > 0) {
    sidx = clip_find(P.step_ts, P.n_step_ts, dir, a, 0);
    const double st = clip_get(P.step_ts, P.n_step_ts, sidx, dir);
    if (ckey(st) < ckey(tn)) tn = st;
  }
  if (P.n_jump_ts > 0) {
    jidx = clip_find(P.jump_ts, P.n_jump_ts, dir, a, 0);
    const double jt = next_down(clip_get(P.jump_ts, P.n_jump_ts, jidx, dir));
    if (ckey(jt) < ckey(tn)) tn = jt;
  }
  return tn;
}

// ClipStepSizeController.adapt_step_size after the PID controller
// (clip.py:330-389).  A step that ended at x or just before x, for x a
// jump time, restarts past x (_bump_next_t0, clip.py:79-99: the sorted
// times equal to nt0 or to nextafter(nt0) sit just below and at the first
// index above nt0); the next step ends no later than the next step time and
// just before the next jump.  Returns made_jump.
__device__ __forceinline__ bool clip_next(const SolveParams &P, int dir, int &sidx, int &jidx,
                                          double &nt0, double &nt1) {
  bool made = false;
  if (P.n_step_ts > 0) {
    const int n = P.n_step_ts;
    const int i = clip_find(P.step_ts, n, dir, nt0, sidx);
    const double n1 = next_up(nt0);
    double b0 = nt0;
    if (i < n && ckey(clip_get(P.step_ts, n, i, dir)) == ckey(n1)) b0 = next_up(n1);
    if (i > 0 && ckey(clip_get(P.step_ts, n, i - 1, dir)) == ckey(nt0)) b0 = n1;
    sidx = clip_find(P.step_ts, n, dir, b0, i);
    const double st = clip_get(P.step_ts, n, sidx, dir);
    if (ckey(st) < ckey(nt1)) nt1 = st;
  }
  if (P.n_jump_ts > 0) {
    const int n = P.n_jump_ts;
    const int i = clip_find(P.jump_ts, n, dir, nt0, jidx);
    const double n1 = next_up(nt0);
    const bool m1 = i < n && ckey(clip_get(P.jump_ts, n, i, dir)) == ckey(n1);
    const bool m2 = i > 0 && ckey(clip_get(P.jump_ts, n, i - 1, dir)) == ckey(nt0);
    if (m1) nt0 = next_up(n1);
    if (m2) nt0 = n1;
    made = m1 || m2;
    const double lo = next_up(nt0);  // never an empty interval (clip.py:354-372)
    if (ckey(lo) > ckey(nt1)) nt1 = lo;
    jidx = clip_find(P.jump_ts, n, dir, nt0, i);
    const double jt = next_down(clip_get(P.jump_ts, n, jidx, dir));
    if (ckey(jt) < ckey(nt1)) nt1 = jt;
  }
  return made;
}

// LAT selects the form of the FP32 copy of dt for the FP32-state kernels: the
// hardware conversion (shortest latency; the fused kernel, whose time is set
// by the step latency of its longest trajectories) or the integer-pipe one
// (no FP64-pipe issue; the plain kernel, which keeps every trajectory
// resident and is bound by FP64 issue).  Both give the same value.  XO
// (extended outputs) adds SaveAt(steps=n) and SaveAt(dense=True)
// (_integrate.py:492-540); the kernels without them keep the shorter step.
template <int SOLVER, class FIELD, class T, bool LAT = false, bool XO = false>
struct Traj {
  using TB = Tab<SOLVER>;
  static constexpr int D = FIELD::D;
  static constexpr int S = TB::S;
  static constexpr int NA = FIELD::NARGS > 0 ? FIELD::NARGS : 1;
  static constexpr bool F32 = sizeof(T) == 4;
  static constexpr bool LEVY = FieldLevy<FIELD>::value;
  static_assert(!is_srk(SOLVER) || LEVY, "the SRKs need the space-time Levy area");

  T y[D];
  T f0[D];  // FSAL: f(t_n, y_n) from the last stage of the previous step
  T args[NA];
  double tprev, tnext, t1, floor1;
  double dtc;  // FP32 mode: tnext - tprev carried from the controller (saves a DADD)
  // FP32 mode: the clip of tnext against t1 (_integrate.py:410-413) of the
  // previous step is checked after this step's stages rather than before them
  // (pend); a step that ran with a size the check would have changed is
  // discarded and run again.  pkeep is that previous step's keep.
  bool pend, pkeep;
  bool live;  // tprev < t1, maintained without an FP64 comparison
  // PID history (pid.py:388-392).  FP32 keeps log2 of the inverse scaled
  // errors so the factor is one exp2 of a weighted sum; FP64 keeps the values.
  T h1, h2;
  int at_dtmin;
  int sc, nc;  // ConstantStepSize state (constant.py:41-57)
  double t0s, t1s;
  double ginv;  // RN(1 / nc), for the grid fraction
  int first, dir, save_index, ts_index, nsteps, nacc, nrej, result;
  int sdown;  // XO: accepted steps left until the next SaveAt(steps=n) save
  int sidx, jidx;  // XO: ClipStepSizeController step / jump indices (hints)
  // XO events: the conditions' last values, the condition that fired (-1
  // none) and, with a root finder, the event time
  double evv[GBDX_MAX_EVENTS];
  int evi;
  double tfin;
  int64_t idx;
  // the trajectory's row of the gradient tape: its queue slot, so that the
  // rows a warp writes together are neighbours however the work order
  // permutes the trajectories (scattered rows cost page-translation misses)
  int64_t trow;
  T wb[FIELD::SDE ? D : 1];  // SDE: W(tprev) of every component (FP32 fields only)
  // Levy area tree: wb holds W_unit(r) and hb bar H_unit(r) at the unit time
  // rb of tprev (unscaled, for Chen's relation)
  T hb[LEVY ? D : 1];
  float rb;

  __device__ __forceinline__ bool running(const SolveParams &P) const {
    return live && result == GBDX_SUCCESSFUL && nsteps < P.max_steps;
  }

  __device__ __forceinline__ T *ys_row(const SolveParams &P, int slot) const {
    return GBDX_AT(P, reinterpret_cast<T *>(P.ys_out), (idx * P.n_save + slot) * D, D,
                   P.batch * P.n_save * D, GBDX_SITE_YS);
  }
  __device__ __forceinline__ double *ts_at(const SolveParams &P, int slot) const {
    return GBDX_AT(P, P.ts_out, idx * P.n_save + slot, 1, P.batch * P.n_save, GBDX_SITE_TS);
  }

  __device__ void init(const SolveParams &P, int64_t i, int64_t row) {
    idx = i;
    trow = row;
    const int64_t ti = i * P.time_stride;
    double a = P.t0[ti], b = P.t1[ti];
    dir = (a < b) ? 1 : -1;  // _integrate.py:1160
    a *= dir;
    b *= dir;
    t1 = b;
    const T *y0 = reinterpret_cast<const T *>(P.y0) + i * D;
#pragma unroll
    for (int n = 0; n < D; n++) y[n] = y0[n];
    const T *ag = reinterpret_cast<const T *>(P.args) + i * P.args_stride;
#pragma unroll
    for (int n = 0; n < FIELD::NARGS; n++) args[n] = ag[n];
    double tn;
    if (P.controller == GBDX_PID) {
      // Terms are wrapped before PIDController.init (_integrate.py:1172-1176,
      // 1254), so dt0=None selects 0.01 (pid.py:48-49).
      double h = P.dt0 ? P.dt0[ti] * dir : 0.01;
      if (P.has_dtmax) h = fmin(h, P.dtmax);
      if (P.has_dtmin) h = fmax(h, P.dtmin);
      tn = a + h;
      if constexpr (XO) tn = clip_init(P, a, tn);
      h1 = F32 ? T(0) : T(1);
      h2 = h1;
      at_dtmin = 0;
    } else {
      double h = P.dt0[ti] * dir;
      sc = 1;
      // an infinite t1 is marked by nc = -1: the grid keeps adding dt0
      // (constant.py:48-55, 94-97)
      const bool fin = isfinite(b);
      nc = fin ? (int)ceil((b - a) / next_up(h)) : -1;
      t0s = a;
      t1s = fin ? b : h;
      tn = a + h;
    }
    // A controller state passed from a previous solve replaces the init
    // above; its first step is then t0 + dt0, unclipped (dt0=None keeps the
    // controller's initial step) (_integrate.py:1252-1265).
    // (the extended-output kernels only: the others keep their shorter init)
    const double *st_in =
        (XO && P.state_in)
            ? GBDX_AT(P, P.state_in, i * int64_t(GBDX_STATE_HEAD + D), GBDX_STATE_HEAD + D,
                      P.batch * (GBDX_STATE_HEAD + D), GBDX_SITE_STATE)
            : nullptr;
    if (st_in && st_in[4] != 0.0) {
      if (P.controller == GBDX_PID) {
        h1 = F32 ? T(log2(st_in[0])) : T(st_in[0]);  // FP32 keeps the log2 domain
        h2 = F32 ? T(log2(st_in[1])) : T(st_in[1]);
        at_dtmin = st_in[2] != 0.0;
        if (P.dt0) tn = a + P.dt0[ti] * dir;
      } else {
        sc = int(st_in[0]);
        nc = int(st_in[1]);
        t0s = st_in[2];
        t1s = st_in[3];
      }
    }
    if (P.controller != GBDX_PID) ginv = 1.0 / double(nc);
    tnext = fmin(tn, b);
    dtc = tnext - a;
    pend = false;
    pkeep = true;
    live = a < b;
    tprev = a;
    floor1 = t1_clip_floor(b);
    if constexpr (LEVY) {
      rb = float((a * dir - P.vbt_t0) * P.vbt_inv_len);
#pragma unroll
      for (int n = 0; n < D; n += 2) {
        float2 w, hh;
        vbt_levy_pair(P, i, rb, n, w, hh);
        wb[n] = w.x;
        wb[n + 1] = w.y;
        hb[n] = hh.x;
        hb[n + 1] = hh.y;
      }
    } else if constexpr (FIELD::SDE) {
#pragma unroll
      for (int n = 0; n < D; n += 2) {
        const float2 w = vbt_w_pair(P, i, a * dir, n);
        wb[n] = w.x;
        wb[n + 1] = w.y;
      }
    }
    first = 1;
    // a passed solver state (first_step, f0) and made_jump: FSAL solvers
    // reuse f0 unless first_step or made_jump (runge_kutta.py:684-700)
    if (XO && st_in && TB::FSAL && st_in[5] == 0.0 && st_in[6] == 0.0) {
      first = 0;
#pragma unroll
      for (int n = 0; n < D; n++) f0[n] = T(st_in[GBDX_STATE_HEAD + n]);
    }
    save_index = 0;
    ts_index = 0;
    nsteps = nacc = nrej = 0;
    result = GBDX_SUCCESSFUL;
    if constexpr (FIELD::TAPE) {
      // full gradient tape: the time and state at every accepted step
      if (P.tape_t) {
        *GBDX_AT(P, P.tape_t, row * (P.max_steps + 1), 1, P.batch * (P.max_steps + 1),
                 GBDX_SITE_TAPE_T) = a;
        T *o = GBDX_AT(P, reinterpret_cast<T *>(P.tape_y), row * int64_t(P.checkpoints) * D, D,
                       P.batch * P.checkpoints * D, GBDX_SITE_TAPE_Y);
#pragma unroll
        for (int n = 0; n < D; n++) o[n] = y[n];
      }
    }
    if (P.save_t0) {
      T *o = ys_row(P, 0);
#pragma unroll
      for (int n = 0; n < D; n++) o[n] = y[n];
      *ts_at(P, 0) = a * dir;
      save_index = 1;
    }
    if constexpr (XO) {
      sdown = P.save_steps;
      // dense_ts[0] = t0 in the loop's time (_integrate.py:1315-1323); the
      // rest of the buffers was filled with +inf before the launch.
      if (P.dense_ts)
        *GBDX_AT(P, P.dense_ts, i * (P.max_steps + 1), 1, P.batch * (P.max_steps + 1),
                 GBDX_SITE_DENSE_TS) = a;
      // Event values at (t0, y0) (_integrate.py:1333-1426): a boolean
      // condition that already holds ends the solve before its first step.
      evi = -1;
      tfin = a;
      if (P.n_event > 0) {
        T f[D];
        FIELD::vf(P, args, y, f);
        // unrolled over the condition slots: constant indices keep evv in
        // registers and the parameter arrays in the constant bank
#pragma unroll
        for (int e = 0; e < GBDX_MAX_EVENTS; e++) {
          if (e < P.n_event) {
            evv[e] = ev_value(P, e, a, y, f);
            if (evi < 0 && P.ev_kind[e] != GBDX_EV_LINEAR && evv[e] != 0.0) evi = e;
          }
        }
        if (evi >= 0) result = GBDX_EVENT_OCCURRED;
      }
    }
  }

  // Value of event condition e at the loop's time t and state yv, with f the
  // field there (steady_state_event); booleans are 0 / 1 (_event.py:120-175).
  __device__ __forceinline__ double ev_value(const SolveParams &P, int e, double t, const T *yv,
                             const T *f) const {
    const int c0 = 6 * e;  // coefficients P.ev_coef[c0 ..]
    if (P.ev_kind[e] == GBDX_EV_STEADY) {
      double sf = 0.0, sy = 0.0;
#pragma unroll
      for (int n = 0; n < D; n++) {
        sf += double(f[n]) * double(f[n]);
        sy += double(yv[n]) * double(yv[n]);
      }
      return sqrt(sf / D) < P.ev_coef[c0 + 1] + P.ev_coef[c0 + 0] * sqrt(sy / D) ? 1.0 : 0.0;
    }
    double v = 0.0;
#pragma unroll
    for (int n = 0; n < (D < 4 ? D : 4); n++) v += P.ev_coef[c0 + n] * double(yv[n]);
    v += P.ev_coef[c0 + 4] * t;
    v += P.ev_coef[c0 + 5];
    if (P.ev_kind[e] == GBDX_EV_LINEAR_BOOL) return v > 0 ? 1.0 : 0.0;
    return v;
  }

  // Whether condition e triggers between its values vo and vn: a boolean when
  // it holds, a real value on the chosen sign change (_integrate.py:585-602).
  __device__ __forceinline__ static bool ev_trig(const SolveParams &P, int e, double vo,
                                                 double vn) {
    if (P.ev_kind[e] != GBDX_EV_LINEAR) return vn != 0.0;
    const double so = isnan(vo) ? vo : double((vo > 0) - (vo < 0));
    const double sn = isnan(vn) ? vn : double((vn > 0) - (vn < 0));
    if (P.ev_dir[e] == GBDX_EV_UP) return so <= 0 && sn > 0;
    if (P.ev_dir[e] == GBDX_EV_DOWN) return so > 0 && sn <= 0;
    return so != sn;
  }

  // d/dtheta of the local interpolant inside the step, component n.
  __device__ __forceinline__ T interp_d(T th, int n, const T (&k)[S][D], const T (&y1)[D]) const {
    if constexpr (SOLVER == GBDX_DOPRI8) {
      T acc = T(0);
#pragma unroll
      for (int j = 0; j < S; j++) acc += dopri8_dw<T>(j, th) * k[j][n];
      return acc;
    } else if constexpr (SOLVER == GBDX_TSIT5) {
      T acc = T(0);
#pragma unroll
      for (int j = 0; j < 7; j++) acc += tsit5_dw<T>(j, th) * k[j < S ? j : 0][n];
      return acc;
    } else if constexpr (SOLVER == GBDX_DOPRI5) {
      T cm = T(0);
#pragma unroll
      for (int j = 0; j < S; j++) cm += T(Tab<GBDX_DOPRI5>::cmid(j < 7 ? j : 0)) * k[j][n];
      const T y0 = y[n], yy1 = y1[n], ymid = y0 + cm;
      const T fa = k[0][n], fb = k[S - 1][n];
      const T a = T(2) * (fb - fa) - T(8) * (yy1 + y0) + T(16) * ymid;
      const T b = T(5) * fa - T(3) * fb + T(18) * y0 + T(14) * yy1 - T(32) * ymid;
      const T c = fb - T(4) * fa - T(11) * y0 - T(5) * yy1 + T(16) * ymid;
      return ((T(4) * a * th + T(3) * b) * th + T(2) * c) * th + fa;
    } else if constexpr (SOLVER == GBDX_HEUN) {
      const T y0 = y[n], yy1 = y1[n], ka = k[0][n], kb = k[S - 1][n];
      const T a = ka + kb + T(2) * y0 - T(2) * yy1;
      const T b = T(-2) * ka - kb - T(3) * y0 + T(3) * yy1;
      return (T(3) * a * th + T(2) * b) * th + ka;
    } else {
      return y1[n] - y[n];
    }
  }

  // The event's root find (_integrate.py:704-779): Newton's method (the
  // restated optimistix.Newton with cauchy termination) on
  // g(t) = w . interp(t) + wt t + c over the step [tp, tn] from t = tn, each
  // iterate clipped to the step; it stops once the step was below
  // atol + rtol |t| and |g| at the previous iterate below atol, from the
  // second iteration on, or fails after 256 iterations.  A boolean condition's
  // root is the end of the step.  y holds the step's y0.
  __device__ __forceinline__ double ev_root(const SolveParams &P, int kind, const double (&cf)[6],
                                            const T (&k)[S][D], const T (&y1)[D], double tp,
                                            double tn, bool &ok) const {
    ok = true;
    if (kind != GBDX_EV_LINEAR) return tn;
    const double span = tn - tp;
    double t = tn;
    for (int it = 1; it <= 256; it++) {
      const T th = T(span == 0.0 ? 0.0 : (t - tp) / span);
      double g = 0.0, gp = 0.0;
#pragma unroll
      for (int n = 0; n < (D < 4 ? D : 4); n++) {
        g += cf[n] * double(interp(th, n, k, y1));
        gp += cf[n] * (span == 0.0 ? 0.0 : double(interp_d(th, n, k, y1)) / span);
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

  __device__ double clip_init(const SolveParams &P, double a, double tn) {
    return clip_start(P, dir, sidx, jidx, a, tn);
  }
  __device__ __forceinline__ bool clip_adapt(const SolveParams &P, double &nt0, double &nt1) {
    return clip_next(P, dir, sidx, jidx, nt0, nt1);
  }

  // One loop iteration.
  __device__ void step(const SolveParams &P) {
    const double dt = F32 ? dtc : tnext - tprev;
    // control = dir * dt (WrapTerm, _term.py:742-745); a sign flip in FP32 mode
    T h;
    if constexpr (F32) {
      const float hm = LAT ? float(dt) : f64i_to_f32(dt);
      h = dir > 0 ? hm : -hm;
    } else {
      h = T(dir * dt);
    }
    T k[S][D];
    T f[D], yi[D], y1[D], err[D], flast[D];
    T dw[FIELD::SDE ? D : 1], wn[FIELD::SDE ? D : 1], sg[FIELD::SDE ? D : 1];
    T dh[LEVY ? D : 1], hn[LEVY ? D : 1];
    float rn = 0.f;
    if constexpr (LEVY) {
      // (W, H) over the loop's step from the tree's values at its two ends
      // by Chen's relation (_levy_diff, tree.py:94-126), scaled by sqrt(T)
      // (tree.py:303-323).  The WrapTerm evaluates the forward real interval
      // and multiplies W and H by the direction (_term.py:742-745): W_b - W_a
      // either way, and H is dir times the relation's value for (a, b).
      rn = float((tnext * dir - P.vbt_t0) * P.vbt_inv_len);
      const float su = rn - rb;
      const float inv = fabsf(su) < 1.1920929e-7f ? 0.f : 1.0f / su;
      const float sq = P.vbt_sqrt_len, sqh = dir > 0 ? sq : -sq;
#pragma unroll
      for (int n = 0; n < D; n += 2) {
        float2 w, hh;
        vbt_levy_pair(P, idx, rn, n, w, hh);
        wn[n] = w.x;
        wn[n + 1] = w.y;
        hn[n] = hh.x;
        hn[n + 1] = hh.y;
      }
#pragma unroll
      for (int n = 0; n < D; n++) {
        const float u_bb_s = rn * wb[n] - rb * wn[n];
        const float bhh_su = hn[n] - hb[n] - 0.5f * u_bb_s;
        dw[n] = sq * (wn[n] - wb[n]);
        dh[n] = sqh * (inv * bhh_su);
      }
    } else if constexpr (FIELD::SDE) {
      // Brownian increment over [tprev, tnext] (ControlTerm, _term.py:420-427)
#pragma unroll
      for (int n = 0; n < D; n += 2) {
        const float2 w = vbt_w_pair(P, idx, tnext * dir, n);
        wn[n] = w.x;
        wn[n + 1] = w.y;
        dw[n] = w.x - wb[n];
        dw[n + 1] = w.y - wb[n + 1];
      }
    }
    if constexpr (is_srk(SOLVER)) {
      // ShARK / SRA1 / SEA, the additive-noise branch of AbstractSRK.step
      // (srk.py:335-671):
      //   z_j = (y0 + sum_i a_ji h f_i) + g (aw_j W + ah_j H),
      //   y1 = (y0 + sum_j b_j h f_j) + g (bw W + bh H),  err = sum_j e_j h f_j,
      // with g = g(t0) (the Ornstein-Uhlenbeck diffusion is constant, so the
      // correction 0.5 (g(t1) - g(t0)) (W - 2H) of srk.py:607-618 is zero).
      // The drift's control is the loop's step t1 - t0 (srk.py:364, given to
      // vf_prod, which the WrapTerm does not flip).
      const T hl = dir > 0 ? h : -h;
      T gw[D], gh[D];
      FIELD::sigma(P, args, y, sg);
#pragma unroll
      for (int n = 0; n < D; n++) {
        gw[n] = sg[n] * dw[n];
        gh[n] = sg[n] * dh[n];
      }
#pragma unroll
      for (int j = 0; j < S; j++) {
#pragma unroll
        for (int n = 0; n < D; n++) {
          T drift = T(0);
#pragma unroll
          for (int i = 0; i < j; i++)
            if (TB::a(j, i) != 0.0) drift += T(TB::a(j, i)) * k[i][n];
          T noise = T(0);
          if (TB::aw(j) != 0.0) noise += T(TB::aw(j)) * gw[n];
          if (TB::ah(j) != 0.0) noise += T(TB::ah(j)) * gh[n];
          yi[n] = (y[n] + drift) + noise;
        }
        FIELD::vf(P, args, yi, f);
#pragma unroll
        for (int n = 0; n < D; n++) k[j][n] = f[n] * hl;
      }
#pragma unroll
      for (int n = 0; n < D; n++) {
        T drift = T(0), e = T(0);
#pragma unroll
        for (int j = 0; j < S; j++) {
          drift += T(TB::b(j)) * k[j][n];
          if (TB::e(j) != 0.0) e += T(TB::e(j)) * k[j][n];
        }
        T noise = T(0);
        if (TB::BW != 0.0) noise += T(TB::BW) * gw[n];
        if (TB::BH != 0.0) noise += T(TB::BH) * gh[n];
        y1[n] = (y[n] + drift) + noise;
        err[n] = is_nan_(e) ? T(INFINITY) : e;
      }
    } else {
      // Stage 0: FSAL reuse except on the first step (runge_kutta.py:684-700).
      if (TB::FSAL && !first) {
#pragma unroll
        for (int n = 0; n < D; n++) f[n] = f0[n];
      } else {
        FIELD::vf(P, args, y, f);
      }
      if constexpr (FIELD::SDE) {
        FIELD::sigma(P, args, y, sg);
#pragma unroll
        for (int n = 0; n < D; n++) k[0][n] = f[n] * h + sg[n] * dw[n];
      } else {
#pragma unroll
        for (int n = 0; n < D; n++) k[0][n] = f[n] * h;
      }
#pragma unroll
      for (int i = 1; i < S; i++) {
#pragma unroll
        for (int n = 0; n < D; n++) {
          if constexpr (F32) {
            // y0 first, newest stage last: only one FMA waits on k_{i-1}.
            T acc = y[n];
#pragma unroll
            for (int j = 0; j < i; j++)
              if (TB::a(i, j) != 0.0) acc = fmaf(T(TB::a(i, j)), k[j][n], acc);
            yi[n] = acc;
          } else {
            // Reference order: increment first, then y0 (runge_kutta.py:866-871).
            T inc = T(0);
#pragma unroll
            for (int j = 0; j < i; j++)
              if (TB::a(i, j) != 0.0) inc += T(TB::a(i, j)) * k[j][n];
            yi[n] = y[n] + inc;
          }
        }
        FIELD::vf(P, args, yi, f);
        if constexpr (FIELD::SDE) {
          FIELD::sigma(P, args, yi, sg);
#pragma unroll
          for (int n = 0; n < D; n++) k[i][n] = f[n] * h + sg[n] * dw[n];
        } else {
#pragma unroll
          for (int n = 0; n < D; n++) k[i][n] = f[n] * h;
        }
        if (i == S - 1) {
#pragma unroll
          for (int n = 0; n < D; n++) flast[n] = f[n];
        }
      }
      // y1 (SSAL: the last stage's input, runge_kutta.py:1177-1185) and the
      // embedded error estimate (:1186-1197).
#pragma unroll
      for (int n = 0; n < D; n++) {
        if constexpr (TB::SSAL) {
          y1[n] = yi[n];
        } else {
          T inc = T(0);
#pragma unroll
          for (int j = 0; j < S; j++) inc += T(TB::b(j)) * k[j][n];
          y1[n] = y[n] + inc;
        }
        T e = T(0);
#pragma unroll
        for (int j = 0; j < S; j++)
          if (TB::e(j) != 0.0) e += T(TB::e(j)) * k[j][n];
        err[n] = is_nan_(e) ? T(INFINITY) : e;
      }
    }  // explicit RK stages

    if constexpr (F32) {
      if (pend) {
        pend = false;
        if (order_key(tnext) > order_key(floor1)) {
          tnext = pkeep ? t1 : tprev + 0.5 * (t1 - tprev);
          dtc = tnext - tprev;
          return;  // run the step again with the clipped size
        }
      }
    }
    // tnext never exceeds t1 here (it is min(t0 + dt0, t1) or clipped), so
    // after the step tprev < t1 unless this step is kept and ends at t1
    // (keys: a +0 tnext against a -0 t1 also ends).
    const bool at_end = order_key(tnext) >= order_key(t1);
    bool keep;
    double nt0, nt1, dt_next;  // dt_next == nt1 - nt0 (FP32 mode carries it)
    if (P.controller == GBDX_PID) {
      // scaled = rms(err / (atol + rtol max(|y0|, |y1|))), y1 -> y0 if NaN
      // (pid.py:466-492).
      bool any_nan = false;
#pragma unroll
      for (int n = 0; n < D; n++) any_nan |= is_nan_(y1[n]);
      const double prev_dt = dt;
      T factor;
      T hnew;
      if constexpr (F32) {
        // Sum of squares of err / (atol + rtol max(|y0|, |y1|)); keep <=> RMS < 1
        // <=> acc < D.  log2(1 / rms) = 0.5 (log2 D - log2 acc), so the factor
        // safety * inv^c1 * prev^c2 * prev2^c3 is one exp2 of a weighted sum.
        // The reciprocal of the tolerance scale depends on y1 only, so it is
        // formed while the last stage's field evaluation (which the error
        // estimate waits for) is in flight.
        T acc = T(0);
#pragma unroll
        for (int n = 0; n < D; n++) {
          T ym = fmaxf(fabsf(y[n]), fabsf(any_nan ? y[n] : y1[n]));
          T s = err[n] * rcp_approx(fmaf(ym, P.rtol_f, P.atol_f));
          acc = fmaf(s, s, acc);
        }
        keep = acc < T(D);
        const T lg = T(0.5) * (Math<T>::log2_(T(D)) - __log2f(acc));
        T ex = T(0);
        if (P.c1_f != 0.f) ex += P.c1_f * lg;
        if (P.c2_f != 0.f) ex += P.c2_f * h1;
        if (P.c3_f != 0.f) ex += P.c3_f * h2;
        factor = P.safety_f * exp2f(ex);
        hnew = isinf(lg) ? T(0) : lg;  // inv in {0, inf} -> 1 (pid.py:536-538)
      } else {
        T acc = T(0);
#pragma unroll
        for (int n = 0; n < D; n++) {
          T ym = fmax(Math<T>::abs_(y[n]), Math<T>::abs_(any_nan ? y[n] : y1[n]));
          T s = err[n] / (T(P.atol) + ym * T(P.rtol));
          acc += s * s;
        }
        const T scaled = Math<T>::sqrt_(acc) / Math<T>::sqrt_(T(D));
        keep = scaled < T(1);
        T inv = T(1) / scaled;
        T f1 = (P.c1 == 0.0) ? T(1) : T(pow(double(inv), P.c1));
        T f2 = (P.c2 == 0.0) ? T(1) : T(pow(double(h1), P.c2));
        T f3 = (P.c3 == 0.0) ? T(1) : T(pow(double(h2), P.c3));
        factor = T(P.safety) * f1 * f2 * f3;
        hnew = (inv == T(0) || isinf(inv)) ? T(1) : inv;
      }
      if (P.has_dtmin) keep = keep || at_dtmin;
      const T fmn = keep ? T(1) : (F32 ? T(P.factormin_f) : T(P.factormin));
      const T fmx = keep ? (F32 ? T(P.factormax_f) : T(P.factormax))
                         : (F32 ? T(P.safety_f) : T(P.safety));
      factor = F32 ? fminf(fmaxf(factor, fmn), fmx) : fmin(fmax(factor, fmn), fmx);
      // FP32 mode: the widening of the factor and the comparisons run on the
      // integer pipes (dt, dtmin and dtmax are never NaN); GB300's FP64
      // conversions take as long as its FP64 multiply.
      double dtn;
      if constexpr (F32) {
        dtn = prev_dt * f64i_from_f32(factor);
      } else {
        dtn = prev_dt * double(factor);
      }
      if (P.has_dtmax && order_key(dtn) > order_key(P.dtmax)) dtn = P.dtmax;
      if (P.has_dtmin) {
        const bool below = order_key(dtn) < order_key(P.dtmin);
        if (!P.force_dtmin && below && result == GBDX_SUCCESSFUL) result = GBDX_DT_MIN_REACHED;
        if (at_dtmin && factor == T(1)) dtn = P.dtmin;
        at_dtmin = order_key(dtn) <= order_key(P.dtmin);
        if (at_dtmin) dtn = P.dtmin;
      }
      nt0 = keep ? tnext : tprev;
      nt1 = nt0 + dtn;
      dt_next = dtn;
      if (keep) {
        h2 = h1;
        h1 = hnew;
      }
    } else {
      keep = true;
      const int s2 = sc + 1;
      double tn = grid_time(t0s, t1s, s2, nc, ginv);
      if (s2 == nc) tn = t1s;
      if (nc < 0) tn = tnext + t1s;
      sc = s2;
      nt0 = tnext;
      nt1 = tn;
      dt_next = F32 ? tn - nt0 : 0.0;
    }
    bool made_jump = false;
    if constexpr (XO) {
      if (P.controller == GBDX_PID && (P.n_step_ts > 0 || P.n_jump_ts > 0)) {
        made_jump = clip_adapt(P, nt0, nt1);
        dt_next = nt1 - nt0;
      }
    }
    // Book-keeping (_integrate.py:410-413).  tprev and tnext never exceed t1
    // (tnext starts at min(t0 + dt0, t1) and is clipped), so the minimum with
    // t1 is the identity; FP32 mode skips it and defers the clip to the next
    // step (pend).
    if constexpr (F32) {
      dtc = dt_next;
      pend = true;
      pkeep = keep;
    } else {
      nt0 = fmin(nt0, t1);
      if (nt1 > floor1) nt1 = keep ? t1 : nt0 + 0.5 * (t1 - nt0);
    }

    if (keep) {
      // Events at the new state (_integrate.py:542-633): the first condition
      // (in order) that triggers ends the solve; with a root finder the final
      // time is the root inside this step, and the saves after it are not
      // made (the reference deletes them, :796-821).
      double tsave = tnext;
      T yfin[XO ? D : 1];
      if constexpr (XO) {
        if (P.n_event > 0) {
          T fn[D];
          if constexpr (TB::FSAL) {
#pragma unroll
            for (int n = 0; n < D; n++) fn[n] = flast[n];
          } else {
            bool steady = false;
#pragma unroll
            for (int e = 0; e < GBDX_MAX_EVENTS; e++)
              steady |= e < P.n_event && P.ev_kind[e] == GBDX_EV_STEADY;
            if (steady) FIELD::vf(P, args, y1, fn);
          }
          int fired = -1;
#pragma unroll
          for (int e = 0; e < GBDX_MAX_EVENTS; e++) {
            if (e < P.n_event) {
              const double v = ev_value(P, e, tnext, y1, fn);
              if (fired < 0 && ev_trig(P, e, evv[e], v)) fired = e;
              evv[e] = v;
            }
          }
          if (fired >= 0) {
            evi = fired;
            result = GBDX_EVENT_OCCURRED;
            tfin = tnext;
            if (P.event_root) {
              bool ok = true;
              // the fired condition's kind and coefficients, selected with
              // constant indices
              int kind = GBDX_EV_LINEAR;
              double cf[6];
#pragma unroll
              for (int e = 0; e < GBDX_MAX_EVENTS; e++) {
                if (e == fired) {
                  kind = P.ev_kind[e];
#pragma unroll
                  for (int n = 0; n < 6; n++) cf[n] = P.ev_coef[6 * e + n];
                }
              }
              tfin = ev_root(P, kind, cf, k, y1, tprev, tnext, ok);
              if (!ok) result = GBDX_NONLINEAR_MAX_STEPS;
              const double span = tnext - tprev;
              const T th = T(span == 0.0 ? 0.0 : (tfin - tprev) / span);
#pragma unroll
              for (int n = 0; n < D; n++) yfin[n] = interp(th, n, k, y1);
              tsave = tfin;
            }
          }
        }
      }
      // SaveAt(ts): every ts <= tnext of the step just taken, interpolated
      // inside [tprev, tnext] (_integrate.py:456-487).
      while (ts_index < P.n_ts) {
        const double tsv = __ldg(P.save_ts + ts_index);
        const double tsd = dir > 0 ? tsv : -tsv;
        if (order_key(tsd) > order_key(tsave)) break;  // save times are never NaN
        const double thd = (tprev == tnext) ? 0.0 : (tsd - tprev) / (tnext - tprev);
        const T th = T(thd);
        T *o = ys_row(P, save_index);
#pragma unroll
        for (int n = 0; n < D; n++) o[n] = interp(th, n, k, y1);
        *ts_at(P, save_index) = tsv;
        ts_index++;
        save_index++;
      }
      if constexpr (XO) {
        // SaveAt(steps=n): (tnext, y1) of every n-th accepted step, after the
        // step's ts saves (_integrate.py:492-527).
        if (P.save_steps > 0 && --sdown == 0) {
          sdown = P.save_steps;
          if (order_key(tnext) <= order_key(tsave)) {  // not past an event's root
            T *o = ys_row(P, save_index);
#pragma unroll
            for (int n = 0; n < D; n++) o[n] = y1[n];
            *ts_at(P, save_index) = dir > 0 ? tnext : -tnext;
            save_index++;
          }
        }
        // SaveAt(dense=True): the step's end time and (y0, y1, k_0..k_{S-1})
        // (_integrate.py:529-540).
        if (P.dense_ts) {
          *GBDX_AT(P, P.dense_ts, idx * (P.max_steps + 1) + nacc + 1, 1,
                   P.batch * (P.max_steps + 1), GBDX_SITE_DENSE_TS) = tnext;
          T *r = GBDX_AT(P, reinterpret_cast<T *>(P.dense_info),
                         (idx * P.max_steps + nacc) * int64_t((2 + S) * D), (2 + S) * D,
                         P.batch * P.max_steps * int64_t((2 + S) * D), GBDX_SITE_DENSE_INFO);
#pragma unroll
          for (int n = 0; n < D; n++) {
            r[n] = y[n];
            r[D + n] = y1[n];
          }
#pragma unroll
          for (int j = 0; j < S; j++)
#pragma unroll
            for (int n = 0; n < D; n++) r[(2 + j) * D + n] = k[j][n];
        }
      }
#pragma unroll
      for (int n = 0; n < D; n++) y[n] = y1[n];
      if constexpr (XO) {
        if (evi >= 0 && P.event_root) {
#pragma unroll
          for (int n = 0; n < D; n++) y[n] = yfin[n];
        }
      }
      if constexpr (FIELD::TAPE) {
        if (P.tape_t) {
          *GBDX_AT(P, P.tape_t, trow * (P.max_steps + 1) + nacc + 1, 1,
                   P.batch * (P.max_steps + 1), GBDX_SITE_TAPE_T) = tnext;
          T *o = GBDX_AT(P, reinterpret_cast<T *>(P.tape_y),
                         (trow * int64_t(P.checkpoints) + nacc + 1) * D, D,
                         P.batch * P.checkpoints * D, GBDX_SITE_TAPE_Y);
#pragma unroll
          for (int n = 0; n < D; n++) o[n] = y1[n];
        }
      }
      if constexpr (FIELD::SDE) {
#pragma unroll
        for (int n = 0; n < D; n++) wb[n] = wn[n];
      }
      if constexpr (LEVY) {
#pragma unroll
        for (int n = 0; n < D; n++) hb[n] = hn[n];
        rb = rn;
      }
      if (TB::FSAL) {
#pragma unroll
        for (int n = 0; n < D; n++) f0[n] = flast[n];
        first = 0;
      }
      // after a jump the FSAL solvers evaluate the first stage afresh
      // (runge_kutta.py:684-700); a rejected step keeps the flag
      // (_integrate.py:425)
      if constexpr (XO) {
        if (made_jump) first = 1;
      }
      nacc++;
    } else {
      nrej++;
    }
    nsteps++;
    tprev = nt0;
    tnext = nt1;
    live = !(keep && at_end);
  }

  // Dense output inside the step, component n.  y holds y0 of the step.
  __device__ __forceinline__ T interp(T th, int n, const T (&k)[S][D], const T (&y1)[D]) const {
    if constexpr (SOLVER == GBDX_DOPRI8) {
      T acc = T(0);
#pragma unroll
      for (int j = 0; j < S; j++) acc += dopri8_w<T>(j, th) * k[j][n];
      return y[n] + acc;
    } else if constexpr (SOLVER == GBDX_TSIT5) {
      T acc = T(0);
#pragma unroll
      for (int j = 0; j < 7; j++) acc += tsit5_w<T>(j, th) * k[j < S ? j : 0][n];
      return y[n] + acc;
    } else if constexpr (SOLVER == GBDX_DOPRI5) {
      // FourthOrderPolynomialInterpolation (_local_interpolation.py:95-139)
      T cm = T(0);
#pragma unroll
      for (int j = 0; j < S; j++) cm += T(Tab<GBDX_DOPRI5>::cmid(j < 7 ? j : 0)) * k[j][n];
      const T y0 = y[n], yy1 = y1[n], ymid = y0 + cm;
      const T fa = k[0][n], fb = k[S - 1][n];
      const T a = T(2) * (fb - fa) - T(8) * (yy1 + y0) + T(16) * ymid;
      const T b = T(5) * fa - T(3) * fb + T(18) * y0 + T(14) * yy1 - T(32) * ymid;
      const T c = fb - T(4) * fa - T(11) * y0 - T(5) * yy1 + T(16) * ymid;
      return (((a * th + b) * th + c) * th + fa) * th + y0;
    } else if constexpr (SOLVER == GBDX_HEUN) {
      // ThirdOrderHermitePolynomialInterpolation.from_k (:50-92)
      const T y0 = y[n], yy1 = y1[n], ka = k[0][n], kb = k[S - 1][n];
      const T a = ka + kb + T(2) * y0 - T(2) * yy1;
      const T b = T(-2) * ka - kb - T(3) * y0 + T(3) * yy1;
      return ((a * th + b) * th + ka) * th + y0;
    } else {
      return y[n] + th * (y1[n] - y[n]);  // LocalLinearInterpolation (:29-47)
    }
  }

  __device__ void finish(const SolveParams &P) {
    const double t0 = P.t0[idx * P.time_stride] * dir;
    // t0 == t1: the ts outputs are y0 (_integrate.py:823-845).
    if (t0 == t1) {
      for (int m = 0; m < P.n_ts; m++) {
        T *o = ys_row(P, save_index);
#pragma unroll
        for (int n = 0; n < D; n++) o[n] = y[n];
        *ts_at(P, save_index) = t0 * dir;
        save_index++;
      }
    }
    // The t1 value is already saved when SaveAt(steps=n) saved the last step:
    // always for n = 1, for n > 1 when n divides the accepted steps
    // (_integrate.py:847-877).
    // With an event root finder the final value is saved whenever the steps
    // saved the t1 value, as that save fell after the event (:860-872); the
    // final time is then the event's.
    bool t1_via_steps = false, save_final = P.save_t1;
    double tf = tprev;
    if constexpr (XO) {
      t1_via_steps = P.save_steps > 0 && sdown == P.save_steps;
      const bool root = P.n_event > 0 && P.event_root;
      save_final = root ? (P.save_t1 || t1_via_steps) : (P.save_t1 && !t1_via_steps);
      if (root && evi >= 0) tf = tfin;
    }
    if (save_final) {
      T *o = ys_row(P, save_index);
#pragma unroll
      for (int n = 0; n < D; n++) o[n] = y[n];
      *ts_at(P, save_index) = tf * dir;
      save_index++;
    }
    if (!P.saves_prefilled) {
      for (int m = save_index; m < P.n_save; m++) {
        T *o = ys_row(P, m);
#pragma unroll
        for (int n = 0; n < D; n++) o[n] = T(INFINITY);
        *ts_at(P, m) = dir > 0 ? INFINITY : -INFINITY;  // direction * inf
      }
    }
    if constexpr (XO) {
      if (P.dense_n) P.dense_n[idx] = nacc + 1;
      if (P.event_index) P.event_index[idx] = evi;
    }
    int r = result;
    if (r == GBDX_SUCCESSFUL && tprev < t1) r = GBDX_MAX_STEPS_REACHED;  // :883
    P.result_out[idx] = r;
    if constexpr (FIELD::TAPE) {
      if (P.tape_n) {
        P.tape_n[trow] = nacc;
        P.tape_stride[trow] = 1;
      }
    }
    P.stats_out[idx * 3 + 0] = nsteps;
    P.stats_out[idx * 3 + 1] = nacc;
    P.stats_out[idx * 3 + 2] = nrej;
    if (XO && P.state_out) {
      // SaveAt(controller_state=, solver_state=, made_jump=) (_integrate.py:
      // 1489-1500): the record gbdx_fwd_extras documents
      double *so = GBDX_AT(P, P.state_out, idx * int64_t(GBDX_STATE_HEAD + D),
                           GBDX_STATE_HEAD + D, P.batch * (GBDX_STATE_HEAD + D),
                           GBDX_SITE_STATE);
      if (P.controller == GBDX_PID) {
        so[0] = F32 ? exp2(double(h1)) : double(h1);
        so[1] = F32 ? exp2(double(h2)) : double(h2);
        so[2] = at_dtmin ? 1.0 : 0.0;
        so[3] = 0.0;
      } else {
        so[0] = sc;
        so[1] = nc;
        so[2] = t0s;
        so[3] = t1s;
      }
      const bool fsal_valid = TB::FSAL && !first;
      so[4] = 1.0;
      so[5] = fsal_valid ? 0.0 : 1.0;
      so[6] = 0.0;  // made_jump: set by a ClipStepSizeController only
#pragma unroll
      for (int n = 0; n < D; n++) so[GBDX_STATE_HEAD + n] = fsal_valid ? double(f0[n]) : 0.0;
    }
  }
};

// ---------------------------------------------------------------------------
// K0: the plain form -- one trajectory per thread, one launch, no refill.
// ---------------------------------------------------------------------------
template <int SOLVER, class FIELD, class T, bool XO = false>
__global__ void __launch_bounds__(128) plain_kernel(SolveParams P) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= P.batch) return;
  Traj<SOLVER, FIELD, T, false, XO> tr;
  tr.init(P, i, i);
  while (tr.running(P)) tr.step(P);
  tr.finish(P);
}

// ---------------------------------------------------------------------------
// K1: the fused persistent form.  A grid sized to the SM count keeps every lane
// busy: when a lane's trajectory finishes it takes the next trajectory index
// from a device counter (one warp-aggregated atomicAdd per refill), so warps
// never idle on the longest lane of a fixed group.
// ---------------------------------------------------------------------------
template <int SOLVER, class FIELD, class T, bool XO = false>
__global__ void __launch_bounds__(256) fused_kernel(SolveParams P) {
  Traj<SOLVER, FIELD, T, true, XO> tr;
  const unsigned lane = threadIdx.x & 31u;
  const unsigned lt_mask = (1u << lane) - 1u;
  bool active = false;
  bool drained = false;  // warp-uniform: the queue has no more work
  while (true) {
    if (!drained) {
      const unsigned need = __ballot_sync(0xffffffffu, !active);
      if (need) {
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(P.queue, (unsigned long long)__popc(need));
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base + __popc(need) >= (unsigned long long)P.batch) drained = true;
        if (!active) {
          const unsigned long long mine = base + __popc(need & lt_mask);
          if (mine < (unsigned long long)P.batch) {
            tr.init(P, P.order ? (int64_t)P.order[mine] : (int64_t)mine, (int64_t)mine);
            active = true;
          }
        }
      }
    }
    if (!__any_sync(0xffffffffu, active)) break;
    if (active) {
      if (tr.running(P)) {
        tr.step(P);
      } else {
        tr.finish(P);
        active = false;
      }
    }
  }
}

}  // namespace gbdx
