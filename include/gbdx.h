/*
 * gbdx.h -- C ABI of the GB300-native batched diffeqsolve library (libgbdx.so).
 *
 * One problem handle describes a vmapped Diffrax solve: the solver, the step
 * size controller, the registered vector field, what to save and how to
 * differentiate.  Every array argument is a caller-owned CUDA device pointer
 * (device memory, or page-locked host memory through the address
 * gbdx_host_device_pointer gives); the library performs no allocation inside a solve and never synchronises the
 * host (results, including per-trajectory RESULTS codes, stay on the device).
 * Every call returns 0 on success or a negative gbdx_status; the message of the
 * last failure on the calling thread is available from gbdx_last_error().
 *
 * Reference interfaces replaced (paths inside the Diffrax v0.7.2 tree):
 *   gbdx_problem_create   <- the static arguments of diffeqsolve
 *                            (diffrax/_integrate.py:888-911) and their checks
 *                            (diffrax/_integrate.py:1036-1265)
 *   gbdx_solve_fwd        <- jax.vmap(diffeqsolve) forward:
 *                            AbstractAdjoint.loop (diffrax/_adjoint.py:121-143)
 *                            driving loop() (diffrax/_integrate.py:302-885)
 *   gbdx_solve_fwd_ex     <- the same with SaveAt(dense=True) (the dense_ts /
 *                            dense_infos buffers of loop(),
 *                            diffrax/_integrate.py:529-540, 1315-1323) and
 *                            events (event_mask, diffrax/_integrate.py:542-821)
 *   gbdx_dense_evaluate   <- DenseInterpolation.evaluate / .derivative
 *                            (diffrax/_global_interpolation.py:315-393)
 *   gbdx_solve_bwd        <- the VJP of that solve under
 *                            RecursiveCheckpointAdjoint (diffrax/_adjoint.py:179-312)
 *   gbdx_backsolve_bwd    <- BacksolveAdjoint's backward pass
 *   gbdx_backsolve_bwd_ex    (diffrax/_adjoint.py:572-734, AdjointTerm
 *                            diffrax/_term.py:767-910)
 */
#ifndef GBDX_H_
#define GBDX_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Solvers (diffrax/_solver/{euler,heun,dopri5,tsit5,dopri8,shark,sra1,sea}.py);
 * Dopri8 on the analytic fields; ShARK, SRA1 and SEA (the additive-noise
 * stochastic Runge--Kutta methods, srk.py:335-671) on the Ornstein--Uhlenbeck
 * SDE with a space-time Levy area tree (SEA: constant steps). */
enum gbdx_solver {
  GBDX_EULER = 0,
  GBDX_HEUN = 1,
  GBDX_DOPRI5 = 2,
  GBDX_TSIT5 = 3,
  GBDX_DOPRI8 = 4,
  GBDX_SHARK = 5,
  GBDX_SRA1 = 6,
  GBDX_SEA = 7
};
/* Levy area drawn by the virtual Brownian tree (diffrax/_custom_types.py). */
enum gbdx_levy_area { GBDX_LEVY_NONE = 0, GBDX_LEVY_SPACE_TIME = 1 };
/* Step size controllers (diffrax/_step_size_controller/{constant,pid}.py). */
enum gbdx_controller { GBDX_CONSTANT = 0, GBDX_PID = 1 };
/* Registered vector fields. */
enum gbdx_field {
  GBDX_LOTKA_VOLTERRA = 0,     /* args (a, b, c, d) */
  GBDX_VAN_DER_POL = 1,        /* args (mu) */
  GBDX_ORNSTEIN_UHLENBECK = 2, /* args (theta, mu, sigma); drift theta (mu - y) */
  GBDX_MLP = 3,                /* eqx.nn.MLP, tanh hidden, identity output */
  GBDX_LINEAR = 4              /* y' = A y, A in params */
};
/* Diagonal diffusion of a ControlTerm driven by a VirtualBrownianTree. */
enum gbdx_diffusion { GBDX_DIFF_NONE = 0, GBDX_DIFF_OU = 1, GBDX_DIFF_TANH_DIAG = 2 };
enum gbdx_dtype { GBDX_F32 = 0, GBDX_F64 = 1 };
/* Kernel family: PLAIN is one trajectory per thread launched once per
 * trajectory; FUSED is the persistent work-stealing integrator; TC is the
 * MLP-field forward on the fifth-generation tensor cores (tcgen05.mma with the
 * accumulators and the Runge--Kutta stages in tensor memory; 64 -> 128 -> 128
 * -> 64 fields, Tsit5, BF16 products, forward solves). */
enum gbdx_kernel {
  GBDX_KERNEL_AUTO = 0,
  GBDX_KERNEL_PLAIN = 1,
  GBDX_KERNEL_FUSED = 2,
  GBDX_KERNEL_TC = 3
};
enum gbdx_adjoint { GBDX_ADJ_NONE = 0, GBDX_ADJ_RECURSIVE = 1, GBDX_ADJ_BACKSOLVE = 2 };
enum gbdx_norm { GBDX_NORM_RMS = 0, GBDX_NORM_ADJOINT_SEMI = 1 };
/* Work order of the fused kernels.  AUTO hands out trajectories by decreasing
 * |t1 - t0| when t0/t1 are per trajectory (time_stride 1), else in index order.
 * The order never changes results, only how busy the lanes stay. */
/* Arithmetic of the MLP field: BF16 operands on the tensor cores with FP32
 * accumulation (the product path), or FP32 SIMT products (parity mode). */
enum gbdx_mlp_precision { GBDX_MLP_BF16 = 0, GBDX_MLP_FP32 = 1 };
enum gbdx_schedule { GBDX_SCHED_AUTO = 0, GBDX_SCHED_INDEX = 1, GBDX_SCHED_LONGEST_FIRST = 2 };

/* RESULTS codes written per trajectory (diffrax/_solution.py:13-31). */
enum gbdx_result {
  GBDX_SUCCESSFUL = 0,
  GBDX_MAX_STEPS_REACHED = 1,
  GBDX_DT_MIN_REACHED = 2,
  GBDX_EVENT_OCCURRED = 3,
  GBDX_MAX_STEPS_REJECTED = 4,
  GBDX_INTERNAL_ERROR = 5,
  GBDX_NONLINEAR_MAX_STEPS = 6 /* the event's root find did not converge */
};

/* Registered event conditions (diffrax/_event.py:13-175).  A condition is
 * evaluated at the loop's time t (time runs forward: t * sign(t1 - t0), the
 * time the reference hands to cond_fn) and state y:
 *   LINEAR       value = sum_n w_n y_n + wt t + c  (real-valued; n < min(dim, 4))
 *   LINEAR_BOOL  value > 0 of the same form      (boolean)
 *   STEADY       rms(f(t, y)) < atol + rtol rms(y) (steady_state_event)  */
enum gbdx_event_kind { GBDX_EV_LINEAR = 0, GBDX_EV_LINEAR_BOOL = 1, GBDX_EV_STEADY = 2 };
/* Event direction of a real-valued condition: either sign change, up-crossings
 * only (direction=True), down-crossings only (direction=False). */
enum gbdx_event_dir { GBDX_EV_EITHER = 0, GBDX_EV_UP = 1, GBDX_EV_DOWN = 2 };
#define GBDX_MAX_EVENTS 4

enum gbdx_status {
  GBDX_OK = 0,
  GBDX_ERR_INVALID = -1,     /* a ValueError in the reference */
  GBDX_ERR_UNSUPPORTED = -2, /* combination outside this library's scope */
  GBDX_ERR_CUDA = -3,        /* a CUDA runtime error */
  GBDX_ERR_WORKSPACE = -4,   /* workspace too small */
  GBDX_ERR_BOUNDS = -5       /* bounds-checked build: a kernel index left its buffer */
};

/* Bounds-checked build (libgbdx_bounds.so: the same sources compiled with
 * -DGBDX_BOUNDS).  Every kernel index into a caller buffer or a workspace
 * region (saved ys / ts, the checkpoint tape, the dense records, the resume
 * records, the backward's segment scratch) is checked against the extent the
 * call defines.  An index outside it records (site, index) -- the first one
 * of the launch -- and the access goes to a scratch sink in the workspace
 * instead, so the launch completes.  The call then synchronizes its stream
 * (unless the stream is capturing a graph) and returns GBDX_ERR_BOUNDS with
 * the site and index in gbdx_last_error().  The workspace grows by
 * GBDX_BOUNDS_BYTES.  In the release build gbdx_bounds_checked() is 0 and
 * no check is compiled. */
enum gbdx_bounds_site {
  GBDX_SITE_YS = 1,          /* ys_out */
  GBDX_SITE_TS = 2,          /* ts_out */
  GBDX_SITE_TAPE_T = 3,      /* the tape's accepted-step times */
  GBDX_SITE_TAPE_Y = 4,      /* the tape's checkpoint states */
  GBDX_SITE_DENSE_TS = 5,    /* dense_ts */
  GBDX_SITE_DENSE_INFO = 6,  /* dense_info */
  GBDX_SITE_STATE = 7,       /* state_in / state_out */
  GBDX_SITE_SCRATCH = 8,     /* the backward's segment recompute states */
  GBDX_SITE_GRAD_YS = 9      /* grad_ys / the saved ys read by a backward */
};
#define GBDX_BOUNDS_BYTES (256 + 65536)
int gbdx_bounds_checked(void);

/* Problem descriptor.  The leading block is shared with the FP64 oracle's
 * descriptor; the trailing block selects precision and kernels. */
typedef struct gbdx_problem_desc {
  int32_t solver, controller, field, dim;
  double rtol, atol, pcoeff, icoeff, dcoeff, safety, factormin, factormax;
  double dtmin, dtmax; /* NaN means None */
  int32_t force_dtmin;
  double error_order;  /* 0 means the solver's own (diffrax/_solver/base.py:97-120) */
  int32_t n_ts, save_t0, save_t1;
  int32_t max_steps;     /* INT32_MAX: max_steps=None (no SaveAt(steps / dense), no
                            RecursiveCheckpointAdjoint) */
  int32_t n_args;
  int32_t mlp_depth;     /* number of linear layers */
  int32_t mlp_widths[9]; /* widths[0] = dim, widths[mlp_depth] = dim */
  int32_t diffusion;     /* gbdx_diffusion */
  double vbt_t0, vbt_t1, vbt_tol;
  uint64_t seed;
  int32_t norm;          /* backsolve adjoint norm (gbdx_norm) */
  int32_t schedule;      /* gbdx_schedule: work order of the fused kernels */
  /* GB300 execution policy */
  int32_t dtype;         /* gbdx_dtype of y, args and params */
  int32_t kernel;        /* gbdx_kernel */
  int32_t adjoint;       /* gbdx_adjoint */
  int32_t checkpoints;   /* RecursiveCheckpointAdjoint(checkpoints=...) slots */
  int32_t block_threads; /* 0 = autotuned */
  int32_t ctas_per_sm;   /* 0 = autotuned */
  int32_t mlp_precision; /* gbdx_mlp_precision of the MLP field's products */
  int32_t save_steps;    /* SaveAt(steps=n): save every n-th accepted step; 0 = off */
  int32_t save_dense;    /* SaveAt(dense=True): record the dense output (solve with
                            gbdx_solve_fwd_ex) */
  /* ClipStepSizeController(PIDController(...), step_ts, jump_ts)
   * (diffrax/_step_size_controller/clip.py:120-427; store_rejected_steps is not
   * available): the numbers of step and jump times, passed after the n_ts
   * SaveAt times in the solve's save_ts array.  PID controller only. */
  int32_t n_step_ts, n_jump_ts;
  /* Event(cond_fn=[...], root_finder, direction) (diffrax/_event.py:13-51,
   * diffrax/_integrate.py:542-633, 686-877): n_event conditions (0 = none,
   * at most GBDX_MAX_EVENTS) of kind ev_kind (gbdx_event_kind) and direction
   * ev_dir (gbdx_event_dir).  Coefficients of condition i: LINEAR(_BOOL)
   * ev_coef[6 i + n] = w_n (n < dim), [6 i + 4] = wt, [6 i + 5] = c; STEADY
   * [6 i] = rtol, [6 i + 1] = atol.  event_root = 1 locates the event time by
   * Newton's method (optimistix.Newton(newton_rtol, newton_atol)) on the last
   * step's interpolant.  Forward solves of the analytic fields (ODEs and the
   * Ornstein--Uhlenbeck SDE); solve with gbdx_solve_fwd_ex to read which
   * condition fired. */
  int32_t n_event, event_root;
  int32_t ev_kind[GBDX_MAX_EVENTS], ev_dir[GBDX_MAX_EVENTS];
  /* The VirtualBrownianTree's levy_area (gbdx_levy_area): SPACE_TIME draws the
   * space-time Levy area H beside W (diffrax/_brownian/tree.py:562-603,
   * 727-750); GBDX_SHARK needs it, Euler and Heun use its W. */
  int32_t levy_area;
  double newton_rtol, newton_atol;
  double ev_coef[6 * GBDX_MAX_EVENTS];
} gbdx_problem_desc;

/* Optional outputs of gbdx_solve_fwd_ex (NULL where not wanted). */
typedef struct gbdx_fwd_extras {
  /* SaveAt(dense=True) (diffrax/_integrate.py:529-540, 1315-1323):
   *   dense_ts   : device f64 [batch, max_steps + 1]: t0 then the end time of
   *                every accepted step, in the loop's direction-flipped time
   *                (t * sign(t1 - t0)); +inf where unused.
   *   dense_info : device [batch, max_steps, (2 + stages) * dim] in desc.dtype:
   *                per accepted step (y0, y1, k_0 .. k_{stages-1}), each dim
   *                long, with k_j the stage increments f_j * control; +inf
   *                where unused.  stages = 1 Euler, 2 Heun, 7 Dopri5 and Tsit5.
   *   dense_n    : device int32 [batch]: accepted steps + 1. */
  double *dense_ts;
  void *dense_info;
  int32_t *dense_n;
  /* Event: device int32 [batch], the index of the condition that ended the
   * solve (the reference's event_mask), -1 where none did. */
  int32_t *event_index;
  /* Resuming a solve (diffeqsolve's solver_state / controller_state /
   * made_jump inputs and SaveAt(solver_state=, controller_state=,
   * made_jump=) outputs, diffrax/_integrate.py:1252-1271, 1309, 1489-1500):
   * device f64 [batch, GBDX_STATE_HEAD + dim] records of
   *   [0..3] the controller state: PID (prev_inv_scaled_error,
   *          prev_prev_inv_scaled_error, at_dtmin, 0); ConstantStepSize
   *          (steps_completed, num_steps, t0, t1 or dt0) in the loop's
   *          direction-flipped time;
   *   [4]    1 when [0..3] holds a controller state (state_in: the first step
   *          is then t0 + dt0 unclipped, or the controller's initial step for
   *          dt0 = NULL);
   *   [5]    the solver state's first_step (1: no FSAL value yet);
   *   [6]    made_jump;
   *   [7..]  the FSAL value f0 (Tsit5, Dopri5, Dopri8).
   * state_in resumes from such a record, state_out receives the final one.
   * Analytic fields without a ClipStepSizeController. */
  const double *state_in;
  double *state_out;
} gbdx_fwd_extras;

#define GBDX_STATE_HEAD 7

typedef struct gbdx_problem gbdx_problem;

/* Validates the descriptor and builds a handle.  Errors mirror the reference's
 * ValueErrors (adaptive Euler, Euler with an SDE and an adaptive controller,
 * ConstantStepSize without dt0 is checked at solve time, and so on). */
int gbdx_problem_create(const gbdx_problem_desc *desc, gbdx_problem **out);
int gbdx_problem_destroy(gbdx_problem *problem);

/* Number of saved points per trajectory (diffrax/_integrate.py:1273-1293):
 * save_t0 + n_ts + max_steps / save_steps (when save_steps > 0) + save_t1
 * (unless save_steps divides max_steps, when the t1 value is a step save). */
int gbdx_num_saves(const gbdx_problem *problem);

/* Device workspace (bytes) a forward solve over `batch` trajectories needs. */
size_t gbdx_workspace_size(const gbdx_problem *problem, int64_t batch);

/*
 * Forward solve of `batch` independent trajectories.
 *   t0, t1, dt0 : device f64 [batch] (time_stride 1) or [1] (time_stride 0);
 *                 dt0 may be NULL, meaning dt0=None.
 *   y0          : device [batch, dim] in desc.dtype.
 *   args        : device [batch, n_args] (args_stride n_args) or [n_args]
 *                 (args_stride 0) in desc.dtype; NULL when n_args == 0.
 *   params      : device MLP / linear / diffusion parameters in desc.dtype
 *                 (layout in gbdx_param_count); NULL for analytic fields.
 *   save_ts     : device f64 [n_ts + n_step_ts + n_jump_ts]: the SaveAt(ts)
 *                 times (monotone in the direction of integration, inside
 *                 [t0, t1]), then the step_ts and the jump_ts of a
 *                 ClipStepSizeController, each sorted increasing.
 *   ys_out      : device [batch, n_saves, dim] in desc.dtype (unsaved = +inf).
 *   ts_out      : device f64 [batch, n_saves].
 *   result_out  : device int32 [batch] gbdx_result codes.
 *   stats_out   : device int32 [batch, 3] (num_steps, accepted, rejected).
 *   workspace   : device scratch of gbdx_workspace_size bytes.
 *   stream      : cudaStream_t (NULL = legacy default stream).
 */
int gbdx_solve_fwd(const gbdx_problem *problem, int64_t batch, const double *t0,
                   const double *t1, const double *dt0, int64_t time_stride,
                   const void *y0, const void *args, int64_t args_stride,
                   const void *params, const double *save_ts, void *ys_out,
                   double *ts_out, int32_t *result_out, int32_t *stats_out,
                   void *workspace, size_t workspace_bytes, void *stream);

/*
 * Backward of a solve under RecursiveCheckpointAdjoint: the
 * discretise-then-optimise VJP of the accepted-step map (the controller is
 * stop-gradient, as in the reference).  Call it after gbdx_solve_fwd on the
 * same problem, inputs and workspace: the forward recorded its accepted-step
 * time grid and state checkpoints there (every accepted state for the
 * analytic fields).
 *   grad_ys     : device [batch, n_saves, dim] cotangent of ys (desc.dtype).
 *   grad_y0     : device [batch, dim] output, dL/dy0.
 *   grad_params : MLP fields: device [gbdx_param_count] FP32 output,
 *                 dL/dparams summed over the batch with compensated (Kahan)
 *                 accumulation.  Analytic fields (Lotka-Volterra, Van der
 *                 Pol, Ornstein-Uhlenbeck ODE and SDE; Euler, Heun, Dopri5,
 *                 Tsit5): dL/dargs in desc.dtype, [batch, n_args] when args
 *                 has a row per trajectory (args_stride = n_args), else
 *                 [n_args] summed over the batch (compensated).
 */
int gbdx_solve_bwd(const gbdx_problem *problem, int64_t batch, const double *t0,
                   const double *t1, const double *dt0, int64_t time_stride,
                   const void *y0, const void *args, int64_t args_stride,
                   const void *params, const double *save_ts, const void *grad_ys,
                   void *grad_y0, void *grad_params, void *workspace,
                   size_t workspace_bytes, void *stream);

/*
 * Backward of a solve under BacksolveAdjoint (MLP field ODEs): reverse-time
 * solves of the augmented state (y, a, a_theta) between adjacent saved times
 * (diffrax/_adjoint.py:572-734) with the problem's solver and controller --
 * create the problem with adjoint = GBDX_ADJ_BACKSOLVE and the backward's
 * solver, controller and norm (desc.norm: GBDX_NORM_RMS runs the error norm
 * over every a_theta component as the reference's default does,
 * GBDX_NORM_ADJOINT_SEMI over (y, a) only), and the forward's SaveAt.
 *   t0, t1, dt0, time_stride : the forward's (dt0 may be NULL for PID).
 *   save_ts     : device [batch, n_saves] FP64, the forward's ts_out.
 *   ys          : device [batch, n_saves, dim] FP32, the forward's ys_out.
 *   grad_ys     : device [batch, n_saves, dim] FP32 cotangent of ys.
 *   params      : device FP32 field parameters (flat layout).
 *   grad_y0     : device [batch, dim] FP32 output, dL/dy0.
 *   grad_params : device [gbdx_param_count] FP32 output, dL/dparams summed
 *                 over the batch with compensated (Kahan) accumulation.
 *   result_out  : device [batch] int32, the first failing RESULTS code of the
 *                 backward's solves (0 = successful).
 *   stats_out   : device [batch, 3] int32, backward steps / accepted /
 *                 rejected over all segments.
 * The workspace is gbdx_workspace_size(problem, batch) bytes.
 */
int gbdx_backsolve_bwd(const gbdx_problem *problem, int64_t batch, const double *t0,
                       const double *t1, const double *dt0, int64_t time_stride,
                       const double *save_ts, const void *ys, const void *grad_ys,
                       const void *params, void *grad_y0, void *grad_params,
                       int32_t *result_out, int32_t *stats_out, void *workspace,
                       size_t workspace_bytes, void *stream);

/*
 * gbdx_backsolve_bwd with the field's args: the same backward pass
 * (diffrax/_adjoint.py:572-734) for every field, including the analytic ones
 * (Lotka-Volterra, Van der Pol, Ornstein-Uhlenbeck ODEs; Euler, Heun, Dopri5,
 * Tsit5), whose augmented state is (y, a, a_args) -- AdjointTerm.vf
 * (diffrax/_term.py:886-910) with the args as the differentiable leaves.
 * GBDX_NORM_RMS runs the error norm over (y, a, a_args), GBDX_NORM_ADJOINT_SEMI
 * over (y, a).  ys, grad_ys and grad_y0 are in desc.dtype.
 *   args, args_stride : as for gbdx_solve_fwd (NULL, 0 for MLP fields).
 *   grad_params : MLP fields as gbdx_backsolve_bwd; analytic fields dL/dargs,
 *                 [batch, n_args] for per-trajectory args, else [n_args]
 *                 summed over the batch (compensated).
 */
int gbdx_backsolve_bwd_ex(const gbdx_problem *problem, int64_t batch, const double *t0,
                          const double *t1, const double *dt0, int64_t time_stride,
                          const double *save_ts, const void *ys, const void *grad_ys,
                          const void *args, int64_t args_stride, const void *params,
                          void *grad_y0, void *grad_params, int32_t *result_out,
                          int32_t *stats_out, void *workspace, size_t workspace_bytes,
                          void *stream);

/*
 * Forward solve with the optional outputs of gbdx_fwd_extras: the arguments of
 * gbdx_solve_fwd plus `extras`.  Problems with save_dense or events must be
 * solved here (dense_ts, dense_info and dense_n are then required; event_index
 * may be NULL).  With n_saves = 0 (SaveAt(dense=True) alone) ys_out and ts_out
 * may be NULL.
 */
int gbdx_solve_fwd_ex(const gbdx_problem *problem, int64_t batch, const double *t0,
                      const double *t1, const double *dt0, int64_t time_stride,
                      const void *y0, const void *args, int64_t args_stride,
                      const void *params, const double *save_ts, void *ys_out,
                      double *ts_out, int32_t *result_out, int32_t *stats_out,
                      const gbdx_fwd_extras *extras, void *workspace,
                      size_t workspace_bytes, void *stream);

/*
 * DenseInterpolation.evaluate (order 0) and .derivative (order 1) of a dense
 * solve (diffrax/_global_interpolation.py:315-393 with the solver's local
 * interpolant, diffrax/_solver/tsit5.py:103-156,
 * diffrax/_local_interpolation.py:29-139): out[b, q] = y_b(t) or dy_b/dt at
 * t = query[b * query_stride + q] in the caller's time (query_stride 0: one
 * set of Q times shared by the batch; Q: Q times per trajectory).
 *   t0, t1, time_stride : the solve's (only the direction sign(t1 - t0) is read).
 *   y0                  : device [batch, dim], the solve's initial state.
 *   dense_ts, dense_info, dense_n : gbdx_solve_fwd_ex's dense outputs.
 *   left    : which side's step a query on a step boundary takes (1 = left).
 *   out     : device [batch, Q, dim] in desc.dtype; NaN outside [t0, t1].
 */
int gbdx_dense_evaluate(const gbdx_problem *problem, int64_t batch, const double *t0,
                        const double *t1, int64_t time_stride, const void *y0,
                        const double *dense_ts, const void *dense_info,
                        const int32_t *dense_n, int64_t Q, const double *query,
                        int64_t query_stride, int left, int order, void *out, void *stream);

/*
 * Forward solve for callers that cannot allocate device memory.  It has no
 * counterpart in the reference.  Callers such as real-time or embedded hosts
 * that reserve all device memory at start-up, or plugin hosts that only hand
 * the solver its input and output buffers, cannot allocate the workspace of
 * gbdx_solve_fwd; this entry point takes the same
 * arguments without it and runs the same solve, using instead a fixed 4 MiB
 * scratch array that every GPU loading the library holds until the process
 * exits.  Batches whose workspace would exceed it (more than 1,047,360
 * trajectories on the fused kernels) are rejected with GBDX_ERR_WORKSPACE,
 * and problems created with an adjoint with GBDX_ERR_UNSUPPORTED (their tape
 * must outlive the call in a workspace that gbdx_solve_bwd reads).
 * The first call on a device (and the first after the device's context was
 * replaced, e.g. by cudaDeviceReset) looks up the array's device address in
 * that context; make that first call before any stream capture.  All calls
 * share the one array (the solve clears what must start at zero), so calls
 * that overlap on the GPU race: serialise them on one stream.
 */
int gbdx_solve_fwd_noalloc(const gbdx_problem *problem, int64_t batch, const double *t0,
                           const double *t1, const double *dt0, int64_t time_stride,
                           const void *y0, const void *args, int64_t args_stride,
                           const void *params, const double *save_ts, void *ys_out,
                           double *ts_out, int32_t *result_out, int32_t *stats_out,
                           void *stream);

/*
 * Diagnostic of the fifth-generation tensor-core path on the current GPU (no
 * counterpart in the reference): one CTA computes D = A B^T for A, B device
 * FP32 [128, 64] rounded to BF16, with tcgen05.mma (operands in shared memory,
 * FP32 accumulator in tensor memory), into D device FP32 [128, 128];
 * status (device int32) is 0, or 1 if the products did not complete.
 */
int gbdx_selftest_tcgen05(const float *A, const float *B, float *D, int32_t *status,
                          void *stream);

/* Number of parameters of the MLP / linear field plus diffusion, in the flat
 * layout [W_0 (out x in, row-major), b_0, W_1, b_1, ..., W_sigma, b_sigma]. */
int64_t gbdx_param_count(const gbdx_problem *problem);

/* sizeof(gbdx_problem_desc), for bindings to check their struct layout. */
size_t gbdx_problem_desc_size(void);

/* The device address of page-locked host memory (no counterpart in the
 * reference, where jax.device_put moves a host array to the device): on
 * success *device is the address under which kernels read and write the
 * host buffer at `host` directly (over NVLink-C2C on a Grace system), and it
 * may be passed as any array argument of a solve -- a solve then moves its
 * inputs and results itself, with no copy before or after it.  The buffer
 * must stay allocated while such a solve runs.  GBDX_ERR_INVALID when `host`
 * is not page-locked host memory mapped for the current device. */
int gbdx_host_device_pointer(const void *host, void **device);

/* Library version and the message of the last error on this thread. */
int gbdx_version(void);
const char *gbdx_last_error(void);

#ifdef __cplusplus
}
#endif

#endif /* GBDX_H_ */
