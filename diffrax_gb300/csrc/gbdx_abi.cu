// gbdx_abi.cu -- the extern "C" boundary of libgbdx.so.
//
// Validation mirrors the ValueErrors that diffeqsolve raises at trace time
// (diffrax/_integrate.py:1036-1154, pid.py:437-447, constant.py:42-46).  A
// solve never allocates: scratch comes from the caller's workspace.
#include <cuda_runtime.h>
#include <math.h>
#include <nvtx3/nvToolsExt.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <string>

#include "../../include/gbdx.h"
#include "gbdx_launch.h"
#include "gbdx_sched.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const char *fmt, ...) __attribute__((format(printf, 2, 3)));
int fail(int code, const char *fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  g_last_error = buf;
  return code;
}

int cuda_fail(cudaError_t e, const char *what) {
  return fail(GBDX_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
}

constexpr size_t kQueueBytes = 256;

// An NVTX range over one C-ABI call, so a profiler's timeline shows which
// solve issued which launches (no cost when no profiler is attached).
struct NvtxRange {
  explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange &) = delete;
  NvtxRange &operator=(const NvtxRange &) = delete;
};

}  // namespace

namespace gbdx {
// Records `msg` as this thread's last error and returns `code` (for the other
// translation units of the library).
int set_last_error(int code, const char *msg) { return fail(code, "%s", msg); }
}  // namespace gbdx

struct gbdx_problem {
  gbdx_problem_desc d;
  int n_save;
  double c1, c2, c3;  // PID exponents
  gbdx::OdeEntry ode;
  // the extended-output form of an analytic-field forward: it also reads and
  // writes the resume records (gbdx_fwd_extras state_in / state_out)
  gbdx::OdeEntry ode_xo;
  gbdx::BwdEntry bwd;  // RecursiveCheckpointAdjoint backward (MLP fields)
  gbdx::BsEntry bs;    // BacksolveAdjoint backward (MLP fields)
  gbdx::AdjEntry adj;  // gradients of the analytic fields (y0 and args)
  bool mlp;            // MLP-field row-tile integrator
  int rows_per_cta;
  int mlp_block;       // threads per CTA of the MLP integrator
};

namespace gbdx {
// The adjoint the problem was created with (GBDX_ADJ_*), for the other
// translation units of the library.
int problem_adjoint(const gbdx_problem *p) { return p->d.adjoint; }
}  // namespace gbdx

namespace {

// Workspace of one solve: the work counter, the work order, and (recursive
// adjoint) the tape the backward reads plus its scratch.
struct WsLayout {
  size_t order, ffrag, tape_t, tape_y, tape_n, tape_s, scratch, psum, pcomp, bounds, total;
  bool has_ffrag;  // width-256 MLP forward: W0 / W2 fragments at ffrag
  size_t frag, rec, ath;  // backsolve: B fragments, stage records, a_theta
  int seg_max, n_cta;
  bool track;
};

// Backsolve tracks a_theta per row when its PID error norm runs over it.
bool bs_tracks(const gbdx_problem_desc &d) {
  return d.controller == GBDX_PID && d.norm == GBDX_NORM_RMS;
}

size_t up256(size_t x) { return (x + 255) / 256 * 256; }

int ws_layout(const gbdx_problem *p, int64_t batch, WsLayout *L) {
  const gbdx_problem_desc &d = p->d;
  const size_t B = size_t(batch > 0 ? batch : 1);
  size_t off = kQueueBytes;
  L->order = off;
  if (d.kernel != GBDX_KERNEL_PLAIN && d.schedule != GBDX_SCHED_INDEX)
    off += up256(gbdx::schedule_workspace_bytes(int64_t(B)));
  // The width-256 MLP integrator reads W0 and W2 as BF16 mma fragments.
  L->ffrag = off;
  L->has_ffrag = p->mlp && d.kernel != GBDX_KERNEL_TC && d.mlp_widths[1] >= 256 &&
                 d.mlp_precision != GBDX_MLP_FP32;
  if (L->has_ffrag) off += 2 * up256(size_t(d.dim) * d.mlp_widths[1] * 2);
  L->tape_t = L->tape_y = L->tape_n = L->tape_s = L->scratch = L->psum = L->pcomp = off;
  L->seg_max = 0;
  L->n_cta = 0;
  L->frag = L->rec = L->ath = off;
  L->track = false;
  if (d.adjoint == GBDX_ADJ_BACKSOLVE && p->bs.launch && d.kernel == GBDX_KERNEL_PLAIN) {
    // the plain backsolve: a_theta and two stage accumulators per trajectory
    L->n_cta = int(B);
    L->track = bs_tracks(d);
    L->frag = L->rec = L->psum = L->pcomp = L->ath = off;
    off += up256(3 * B * size_t(gbdx_param_count(p)) * sizeof(float));
  } else if (d.adjoint == GBDX_ADJ_BACKSOLVE && p->bs.launch) {
    int dev = 0, sms = 0, occ = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = p->bs.occupancy(&occ);
    if (e != cudaSuccess) return cuda_fail(e, "backsolve launch shape");
    if (occ < 1) occ = 1;
    int64_t grid = int64_t(sms) * occ;
    const int64_t needed = (int64_t(B) + p->bs.rows - 1) / p->bs.rows;
    if (grid > needed) grid = needed;
    L->n_cta = int(grid);
    const size_t np = size_t(gbdx_param_count(p));
    const size_t D = size_t(d.dim), H = size_t(d.mlp_widths[1]);
    L->frag = off;
    if (p->bs.gfrag) off += 4 * up256(D * H * 2);
    L->rec = off;
    off += up256(size_t(L->n_cta) * p->bs.stages * p->bs.rows * p->bs.rec * sizeof(float));
    L->psum = off;
    off += up256(size_t(L->n_cta) * np * sizeof(float));
    L->pcomp = off;
    off += up256(size_t(L->n_cta) * np * sizeof(float));
    L->track = bs_tracks(d);
    L->ath = off;
    off += up256(size_t(L->n_cta) * p->bs.rows * 2 * np * sizeof(float));
  }
  if (d.adjoint == GBDX_ADJ_RECURSIVE && p->bwd.launch && d.kernel == GBDX_KERNEL_PLAIN) {
    // the plain backward: full tape, per-trajectory cotangents dP [P][B]
    const size_t C = size_t(d.max_steps) + 1;
    L->tape_t = off;
    off += up256(B * C * sizeof(double));
    L->tape_y = off;
    off += up256(B * C * d.dim * sizeof(float));
    L->tape_n = off;
    off += up256(B * sizeof(int32_t));
    L->tape_s = off;
    off += up256(B * sizeof(int32_t));
    L->scratch = off;
    L->psum = off;
    off += up256(B * size_t(gbdx_param_count(p)) * sizeof(float));
    L->pcomp = off;
    L->n_cta = int(B);
  } else if (d.adjoint == GBDX_ADJ_RECURSIVE && p->bwd.launch) {
    const int C = d.checkpoints > 1 ? d.checkpoints : 2;
    L->tape_t = off;
    off += up256(B * size_t(d.max_steps + 1) * sizeof(double));
    L->tape_y = off;
    off += up256(B * size_t(C) * d.dim * sizeof(float));
    L->tape_n = off;
    off += up256(B * sizeof(int32_t));
    L->tape_s = off;
    off += up256(B * sizeof(int32_t));
    // With C slots the checkpoint stride stays below 2 max_steps / C + 1.
    int seg = (2 * d.max_steps + C - 1) / C + 1;
    if (seg > d.max_steps + 1) seg = d.max_steps + 1;
    L->seg_max = seg;
    L->scratch = off;
    off += up256(B * size_t(seg) * d.dim * sizeof(float));
    int dev = 0, sms = 0, occ = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = p->bwd.occupancy(&occ);
    if (e != cudaSuccess) return cuda_fail(e, "backward launch shape");
    if (occ < 1) occ = 1;
    int64_t grid = int64_t(sms) * occ;
    const int64_t needed = (int64_t(B) + p->rows_per_cta - 1) / p->rows_per_cta;
    if (grid > needed) grid = needed;
    L->n_cta = int(grid);
    const size_t np = size_t(gbdx_param_count(p));
    L->psum = off;
    off += up256(size_t(L->n_cta) * np * sizeof(float));
    L->pcomp = off;
    off += up256(size_t(L->n_cta) * np * sizeof(float));
  }
  if (d.adjoint == GBDX_ADJ_RECURSIVE && p->adj.rc_bwd) {
    // the analytic fields: the full tape (time and state of every accepted
    // step) and the per-trajectory args gradients
    const size_t esz = d.dtype == GBDX_F32 ? 4 : 8, C = size_t(d.max_steps) + 1;
    L->tape_t = off;
    off += up256(B * C * sizeof(double));
    L->tape_y = off;
    off += up256(B * C * d.dim * esz);
    L->tape_n = off;
    off += up256(B * sizeof(int32_t));
    L->tape_s = off;
    off += up256(B * sizeof(int32_t));
    L->scratch = off;
    off += up256(B * size_t(p->adj.n_args) * esz);
  } else if (d.adjoint == GBDX_ADJ_BACKSOLVE && p->adj.bs_bwd) {
    const size_t esz = d.dtype == GBDX_F32 ? 4 : 8;
    L->scratch = off;
    off += up256(B * size_t(p->adj.n_args) * esz);
    L->track = bs_tracks(d);
  }
  L->bounds = off;
#ifdef GBDX_BOUNDS
  off += GBDX_BOUNDS_BYTES;
#endif
  L->total = off;
  return GBDX_OK;
}

// Bounds-checked builds: clear the launch's record before its kernels and
// read it after them (include/gbdx.h, GBDX_ERR_BOUNDS).
int bounds_clear(const gbdx::SolveParams &P, cudaStream_t s) {
#ifdef GBDX_BOUNDS
  cudaError_t e = cudaMemsetAsync(P.bounds, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return cuda_fail(e, "bounds record reset");
#else
  (void)P;
  (void)s;
#endif
  return GBDX_OK;
}

const char *bounds_site_name(int site) {
  switch (site) {
    case GBDX_SITE_YS: return "ys";
    case GBDX_SITE_TS: return "ts";
    case GBDX_SITE_TAPE_T: return "tape times";
    case GBDX_SITE_TAPE_Y: return "tape states";
    case GBDX_SITE_DENSE_TS: return "dense_ts";
    case GBDX_SITE_DENSE_INFO: return "dense_info";
    case GBDX_SITE_STATE: return "state records";
    case GBDX_SITE_SCRATCH: return "segment scratch";
    case GBDX_SITE_GRAD_YS: return "grad_ys / saved ys";
    default: return "unknown";
  }
}

int bounds_report(const gbdx::SolveParams &P, cudaStream_t s, const char *call) {
#ifdef GBDX_BOUNDS
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  cudaError_t e = cudaStreamIsCapturing(s, &cap);
  if (e != cudaSuccess) return cuda_fail(e, "bounds capture query");
  if (cap != cudaStreamCaptureStatusNone) return GBDX_OK;
  unsigned long long rec = 0;
  e = cudaMemcpyAsync(&rec, P.bounds, sizeof rec, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return cuda_fail(e, "bounds record read");
  if (rec != 0) {
    long long idx = static_cast<long long>(rec << 8) >> 8;  // sign-extend 56 bits
    const int site = int(rec >> 56);
    return fail(GBDX_ERR_BOUNDS, "%s: index %lld outside the %s buffer (site %d)", call, idx,
                bounds_site_name(site), site);
  }
#else
  (void)P;
  (void)s;
  (void)call;
#endif
  return GBDX_OK;
}

}  // namespace

extern "C" {

int gbdx_version(void) { return 1; }

int gbdx_bounds_checked(void) {
#ifdef GBDX_BOUNDS
  return 1;
#else
  return 0;
#endif
}

size_t gbdx_problem_desc_size(void) { return sizeof(gbdx_problem_desc); }

int gbdx_host_device_pointer(const void *host, void **device) {
  if (!host || !device) return fail(GBDX_ERR_INVALID, "gbdx_host_device_pointer: null argument");
  *device = nullptr;
  cudaPointerAttributes a;
  cudaError_t e = cudaPointerGetAttributes(&a, host);
  if (e != cudaSuccess || a.type != cudaMemoryTypeHost) {
    cudaGetLastError();
    return fail(GBDX_ERR_INVALID, "gbdx_host_device_pointer: %p is not page-locked host memory",
                host);
  }
  void *d = nullptr;
  e = cudaHostGetDevicePointer(&d, const_cast<void *>(host), 0);
  if (e != cudaSuccess || !d) {
    cudaGetLastError();
    return fail(GBDX_ERR_INVALID,
                "gbdx_host_device_pointer: %p is not mapped for the current device (%s)", host,
                cudaGetErrorString(e));
  }
  *device = d;
  return GBDX_OK;
}

const char *gbdx_last_error(void) { return g_last_error.c_str(); }

static int solver_order(int solver) {
  switch (solver) {
    case GBDX_EULER: return 1;
    case GBDX_HEUN: return 2;
    case GBDX_DOPRI8: return 8;
    case GBDX_SHARK: return 2;
    case GBDX_SRA1: return 2;
    case GBDX_SEA: return 1;
    default: return 5;
  }
}
// Stages of a solver: the k vectors of its dense-output record.
static int solver_stages(int solver) {
  switch (solver) {
    case GBDX_EULER: return 1;
    case GBDX_HEUN: return 2;
    case GBDX_DOPRI8: return 14;
    case GBDX_SHARK: return 2;
    case GBDX_SRA1: return 2;
    case GBDX_SEA: return 1;
    default: return 7;
  }
}
static double solver_strong_order(int solver) {
  if (solver == GBDX_SHARK || solver == GBDX_SRA1) return 1.5;
  if (solver == GBDX_SEA) return 1.0;
  return (solver == GBDX_EULER || solver == GBDX_HEUN) ? 0.5 : 0.0;
}

int gbdx_problem_create(const gbdx_problem_desc *desc, gbdx_problem **out) {
  if (!desc || !out) return fail(GBDX_ERR_INVALID, "null descriptor or output handle");
  *out = nullptr;
  const gbdx_problem_desc &d = *desc;
  if (d.solver < GBDX_EULER || d.solver > GBDX_SEA)
    return fail(GBDX_ERR_INVALID, "unknown solver %d", d.solver);
  if (d.controller != GBDX_CONSTANT && d.controller != GBDX_PID)
    return fail(GBDX_ERR_INVALID, "unknown step size controller %d", d.controller);
  if (d.dtype != GBDX_F32 && d.dtype != GBDX_F64)
    return fail(GBDX_ERR_INVALID, "unknown dtype %d", d.dtype);
  if (d.dim < 1) return fail(GBDX_ERR_INVALID, "state dimension must be positive");
  if (d.kernel < GBDX_KERNEL_AUTO || d.kernel > GBDX_KERNEL_TC)
    return fail(GBDX_ERR_INVALID, "unknown kernel family %d", d.kernel);
  if (d.kernel == GBDX_KERNEL_TC && d.field != GBDX_MLP)
    return fail(GBDX_ERR_UNSUPPORTED, "the tensor-core (TC) kernel integrates MLP fields");
  if (d.max_steps < 1) return fail(GBDX_ERR_INVALID, "max_steps must be a positive integer");
  // the tape and the step-indexed outputs are sized by max_steps: an unbounded
  // solve (max_steps=None, passed as INT32_MAX) has none of them
  if (d.max_steps > (1 << 30) &&
      (d.adjoint == GBDX_ADJ_RECURSIVE || d.save_dense || d.save_steps > 0))
    return fail(GBDX_ERR_INVALID,
                "max_steps above 2^30 (an unbounded solve) takes neither SaveAt(steps=n), "
                "SaveAt(dense=True) nor RecursiveCheckpointAdjoint");
  if (d.n_ts < 0) return fail(GBDX_ERR_INVALID, "negative number of SaveAt(ts=...) points");
  if (d.save_steps < 0) return fail(GBDX_ERR_INVALID, "SaveAt(steps=n) needs n >= 0");
  // Output length (_integrate.py:1273-1293): SaveAt(steps=n) reserves
  // max_steps // n slots, and the t1 slot only when n does not divide max_steps.
  int n_save = (d.save_t0 ? 1 : 0) + d.n_ts;
  if (d.save_steps > 0) n_save += d.max_steps / d.save_steps;
  if (d.save_t1 && (d.save_steps == 0 || d.max_steps % d.save_steps != 0)) n_save += 1;
  if (n_save < 1 && !d.save_dense)
    return fail(GBDX_ERR_INVALID, "Empty saveat -- nothing will be saved.");
  const bool sde = d.diffusion != GBDX_DIFF_NONE;
  if (d.levy_area != GBDX_LEVY_NONE && d.levy_area != GBDX_LEVY_SPACE_TIME)
    return fail(GBDX_ERR_INVALID, "unknown levy_area %d", d.levy_area);
  if (d.levy_area != GBDX_LEVY_NONE && !sde)
    return fail(GBDX_ERR_INVALID, "levy_area belongs to the Brownian tree of an SDE");
  // srk.py:374-379: the SRKs take the space-time Levy area of an SDE's tree
  if (gbdx::is_srk(d.solver) && (!sde || d.levy_area != GBDX_LEVY_SPACE_TIME))
    return fail(GBDX_ERR_INVALID,
                "ShARK, SRA1 and SEA solve SDEs whose Brownian tree has "
                "levy_area=SpaceTimeLevyArea");
  // pid.py:437-447: adaptive stepping needs an error estimate.
  if (d.controller == GBDX_PID && (d.solver == GBDX_EULER || d.solver == GBDX_SEA))
    return fail(GBDX_ERR_INVALID,
                "Cannot use adaptive step sizes with a solver that does not provide error "
                "estimates.");
  // _integrate.py:1145-1151
  if (sde && d.controller == GBDX_PID && d.solver == GBDX_EULER)
    return fail(GBDX_ERR_INVALID,
                "An SDE should not be solved with adaptive step sizes with Euler's method.");
  if (d.controller == GBDX_PID) {
    if (!(d.rtol >= 0) || !(d.atol >= 0))
      return fail(GBDX_ERR_INVALID, "rtol and atol must be non-negative");
    if (!(d.factormin > 0) || !(d.factormax > 0) || !(d.safety > 0))
      return fail(GBDX_ERR_INVALID, "factormin, factormax and safety must be positive");
  }

  gbdx_problem *p = new gbdx_problem();
  p->d = d;
  p->n_save = n_save;
  double order = d.error_order > 0 ? d.error_order
                                   : (sde ? solver_strong_order(d.solver) + 0.5
                                          : (double)solver_order(d.solver));
  p->c1 = (d.icoeff + d.pcoeff + d.dcoeff) / order;
  p->c2 = -(d.pcoeff + 2 * d.dcoeff) / order;
  p->c3 = d.dcoeff / order;
  p->ode = gbdx::OdeEntry{nullptr, nullptr};
  p->bwd = gbdx::BwdEntry{nullptr, nullptr};
  p->bs = gbdx::BsEntry{nullptr, nullptr, 0, 0, 0, 0};
  p->adj = gbdx::AdjEntry{};
  p->mlp = false;
  p->rows_per_cta = 1;
  p->mlp_block = 256;
  if (d.n_step_ts < 0 || d.n_jump_ts < 0) {
    delete p;
    return fail(GBDX_ERR_INVALID, "negative number of step_ts or jump_ts");
  }
  const bool clip = d.n_step_ts > 0 || d.n_jump_ts > 0;
  // clip.py:195-199
  if (clip && d.controller != GBDX_PID) {
    delete p;
    return fail(GBDX_ERR_INVALID,
                "Can only apply `ClipStepSizeController` to adaptive step size controllers.");
  }
  if (d.n_event < 0 || d.n_event > GBDX_MAX_EVENTS) {
    delete p;
    return fail(GBDX_ERR_INVALID, "an event has 0 to %d conditions", GBDX_MAX_EVENTS);
  }
  for (int e = 0; e < d.n_event; e++) {
    if (d.ev_kind[e] < GBDX_EV_LINEAR || d.ev_kind[e] > GBDX_EV_STEADY ||
        d.ev_dir[e] < GBDX_EV_EITHER || d.ev_dir[e] > GBDX_EV_DOWN) {
      delete p;
      return fail(GBDX_ERR_INVALID, "unknown event condition kind or direction");
    }

  }
  if (d.n_event > 0 && d.event_root && !(d.newton_rtol >= 0 && d.newton_atol > 0)) {
    delete p;
    return fail(GBDX_ERR_INVALID, "the root finder needs rtol >= 0 and atol > 0");
  }
  const bool xo = d.save_steps > 0 || d.save_dense || clip || d.n_event > 0;
  // The MLP integrator (K2) records step saves and dense steps, runs the clip
  // controller and the events; the plain and tensor-core MLP kernels do not.
  const bool xo_mlp = d.field == GBDX_MLP && d.adjoint == GBDX_ADJ_NONE &&
                      d.kernel != GBDX_KERNEL_PLAIN && d.kernel != GBDX_KERNEL_TC;
  if (xo && !xo_mlp &&
      (d.field == GBDX_MLP || d.adjoint != GBDX_ADJ_NONE ||
       (sde && d.diffusion != GBDX_DIFF_OU))) {
    delete p;
    return fail(GBDX_ERR_UNSUPPORTED,
                "SaveAt(steps=...), SaveAt(dense=True), ClipStepSizeController and events "
                "are available for forward solves of the analytic fields (ODEs and the "
                "Ornstein-Uhlenbeck SDE) and of the MLP fields on the fused kernel");
  }
  if (!sde && (d.field == GBDX_LOTKA_VOLTERRA || d.field == GBDX_VAN_DER_POL ||
               d.field == GBDX_ORNSTEIN_UHLENBECK)) {
    p->ode_xo = d.dtype == GBDX_F32 ? gbdx::find_ode_entry_f32_xo(d.solver, d.field, d.dim)
                                    : gbdx::find_ode_entry_f64_xo(d.solver, d.field, d.dim);
    if (xo)
      p->ode = p->ode_xo;
    else
      p->ode = d.dtype == GBDX_F32 ? gbdx::find_ode_entry_f32(d.solver, d.field, d.dim)
                                   : gbdx::find_ode_entry_f64(d.solver, d.field, d.dim);
    if (!p->ode.launch) {
      delete p;
      return fail(GBDX_ERR_UNSUPPORTED, "no kernel for field %d with state dimension %d",
                  d.field, d.dim);
    }
    if (d.adjoint != GBDX_ADJ_NONE) {
      p->adj = d.dtype == GBDX_F32 ? gbdx::find_ode_adj_entry_f32(d.solver, d.field, d.dim, false)
                                   : gbdx::find_ode_adj_entry_f64(d.solver, d.field, d.dim);
      if (!p->adj.rc_bwd) {
        delete p;
        return fail(GBDX_ERR_UNSUPPORTED,
                    "gradients of the analytic fields take Euler, Heun, Dopri5 or Tsit5");
      }
      if (d.adjoint == GBDX_ADJ_RECURSIVE) p->ode = p->adj.fwd;
      if (d.adjoint == GBDX_ADJ_BACKSOLVE && d.norm != GBDX_NORM_RMS &&
          d.norm != GBDX_NORM_ADJOINT_SEMI) {
        delete p;
        return fail(GBDX_ERR_INVALID, "unknown norm %d", d.norm);
      }
    }
  } else if (sde && d.field == GBDX_ORNSTEIN_UHLENBECK && d.diffusion == GBDX_DIFF_OU) {
    if (d.dtype != GBDX_F32) {
      delete p;
      return fail(GBDX_ERR_UNSUPPORTED,
                  "the Ornstein-Uhlenbeck SDE runs with FP32 state (FP32 Brownian tree)");
    }
    p->ode_xo = d.levy_area == GBDX_LEVY_SPACE_TIME
                    ? gbdx::find_ode_sde_levy_entry_f32_xo(d.solver, d.dim)
                    : gbdx::find_ode_sde_entry_f32_xo(d.solver, d.dim);
    p->ode = xo ? p->ode_xo
                : (d.levy_area == GBDX_LEVY_SPACE_TIME
                       ? gbdx::find_ode_sde_levy_entry_f32(d.solver, d.dim)
                       : gbdx::find_ode_sde_entry_f32(d.solver, d.dim));
    if (!p->ode.launch) {
      delete p;
      return fail(GBDX_ERR_UNSUPPORTED,
                  "no SDE kernel for state dimension %d (the Ornstein-Uhlenbeck SDE takes "
                  "dim 2 or 4) or solver %d", d.dim, d.solver);
    }
    if (d.adjoint == GBDX_ADJ_BACKSOLVE) {
      delete p;
      return fail(GBDX_ERR_UNSUPPORTED, "BacksolveAdjoint is available for ODEs");
    }
    if (d.adjoint == GBDX_ADJ_RECURSIVE) {
      if (d.levy_area != GBDX_LEVY_NONE) {
        delete p;
        return fail(GBDX_ERR_UNSUPPORTED,
                    "gradients of the Ornstein-Uhlenbeck SDE take the W-only Brownian tree");
      }
      p->adj = gbdx::find_ode_adj_entry_f32(d.solver, d.field, d.dim, true);
      if (!p->adj.rc_bwd) {
        delete p;
        return fail(GBDX_ERR_UNSUPPORTED,
                    "gradients of the Ornstein-Uhlenbeck SDE take Euler or Heun");
      }
      p->ode = p->adj.fwd;
    }
  } else if (d.field == GBDX_MLP) {
    const int *w = d.mlp_widths;
    if (d.solver == GBDX_DOPRI8) {
      delete p;
      return fail(GBDX_ERR_UNSUPPORTED, "Dopri8 is available for the analytic fields");
    }
    if (d.levy_area != GBDX_LEVY_NONE) {
      delete p;
      return fail(GBDX_ERR_UNSUPPORTED,
                  "the space-time Levy area tree (and ShARK) drive the Ornstein-Uhlenbeck SDE");
    }
    if (d.mlp_depth != 3 || w[0] != d.dim || w[3] != d.dim || w[1] != w[2]) {
      delete p;
      return fail(GBDX_ERR_UNSUPPORTED,
                  "MLP fields must be dim -> width -> width -> dim (got depth %d)",
                  d.mlp_depth);
    }
    if (d.dtype != GBDX_F32) {
      delete p;
      return fail(GBDX_ERR_UNSUPPORTED, "MLP fields run with FP32 state");
    }
    if (sde && d.diffusion != GBDX_DIFF_TANH_DIAG) {
      delete p;
      return fail(GBDX_ERR_UNSUPPORTED, "MLP drifts take the tanh diagonal diffusion");
    }
    const bool precise = d.mlp_precision == GBDX_MLP_FP32;
    const int D = d.dim, H = w[1];
    if (d.kernel == GBDX_KERNEL_TC) {
      // the tcgen05 forward: BF16 products, no gradient tape
      if (precise || d.adjoint != GBDX_ADJ_NONE) {
        delete p;
        return fail(GBDX_ERR_UNSUPPORTED,
                    "the tensor-core (TC) kernel runs BF16 forward solves without an adjoint");
      }
      p->ode = gbdx::find_mlp_tc_entry(d.solver, D, H, sde);
      if (!p->ode.launch) {
        delete p;
        return fail(GBDX_ERR_UNSUPPORTED,
                    "the tensor-core (TC) kernel takes 64 -> 128 -> 128 -> 64 ODE fields with "
                    "Tsit5 or Dopri5 (got dim %d, width %d, solver %d%s)", D, H, d.solver,
                    sde ? ", SDE" : "");
      }
      p->mlp = true;
      p->rows_per_cta = 128;
      p->mlp_block = 512;  // four threads per trajectory
      *out = p;
      return GBDX_OK;
    }
    if (d.kernel == GBDX_KERNEL_PLAIN) {
      // The plain form: one trajectory per thread, FP32 CUDA-core products.
      if (d.adjoint == GBDX_ADJ_BACKSOLVE) {
        p->bs = sde ? gbdx::BsEntry{nullptr, nullptr, 0, 0, 0, 0}
                    : gbdx::find_plain_backsolve_entry(d.solver, D, H);
        if (!p->bs.launch) {
          delete p;
          return fail(GBDX_ERR_UNSUPPORTED,
                      "no plain backsolve for dim %d, width %d, solver %d", D, H, d.solver);
        }
      }
      if (d.adjoint == GBDX_ADJ_RECURSIVE) {
        p->bwd = gbdx::find_mlp_plain_bwd_entry(d.solver, D, H, sde);
        if (!p->bwd.launch) {
          delete p;
          return fail(GBDX_ERR_UNSUPPORTED, "no plain backward for dim %d, width %d, solver %d",
                      D, H, d.solver);
        }
      }
      p->ode = gbdx::find_mlp_plain_entry(d.solver, D, H, sde);
      if (!p->ode.launch) {
        delete p;
        return fail(GBDX_ERR_UNSUPPORTED, "no plain kernel for dim %d, width %d, solver %d",
                    D, H, d.solver);
      }
      *out = p;
      return GBDX_OK;
    }
    if (D == 64 && H == 128) {
      p->ode_xo = gbdx::find_mlp_xo_entry_d64h128(d.solver, precise, sde);
      p->ode = xo ? p->ode_xo : gbdx::find_mlp_entry_d64h128(d.solver, precise, sde);
    }
    if (D == 64 && H == 256) {
      p->ode_xo = gbdx::find_mlp_xo_entry_d64h256(d.solver, precise, sde);
      p->ode = xo ? p->ode_xo : gbdx::find_mlp_entry_d64h256(d.solver, precise, sde);
    }
    if (D == 32 && H == 64) {
      p->ode_xo = gbdx::find_mlp_xo_entry_d32h64(d.solver, precise, sde);
      p->ode = xo ? p->ode_xo : gbdx::find_mlp_entry_d32h64(d.solver, precise, sde);
    }
    if (!p->ode.launch) {
      delete p;
      return fail(GBDX_ERR_UNSUPPORTED,
                  "no MLP kernel for dim %d, width %d, solver %d%s", D, H, d.solver,
                  sde ? " (SDE)" : "");
    }
    p->mlp = true;
    p->rows_per_cta = H >= 256 ? 16 : 32;
    if (d.adjoint == GBDX_ADJ_RECURSIVE) {
      if (D == 64 && H == 128) p->bwd = gbdx::find_mlp_bwd_entry_d64h128(d.solver, precise, sde);
      // (width 256 does not fit the backward's weights and operands in
      // shared memory; that shape is differentiated by BacksolveAdjoint)
      if (D == 32 && H == 64) p->bwd = gbdx::find_mlp_bwd_entry_d32h64(d.solver, precise, sde);
      if (!p->bwd.launch) {
        delete p;
        return fail(GBDX_ERR_UNSUPPORTED, "no backward kernel for this MLP problem");
      }
    }
    if (d.adjoint == GBDX_ADJ_BACKSOLVE) {
      if (sde) {
        delete p;
        return fail(GBDX_ERR_UNSUPPORTED, "BacksolveAdjoint is available for MLP ODEs");
      }
      if (D == 64 && H == 256) p->bs = gbdx::find_backsolve_entry_d64h256(d.solver, precise);
      if (D == 64 && H == 128) p->bs = gbdx::find_backsolve_entry_d64h128(d.solver, precise);
      if (D == 32 && H == 64) p->bs = gbdx::find_backsolve_entry_d32h64(d.solver, precise);
      if (!p->bs.launch) {
        delete p;
        return fail(GBDX_ERR_UNSUPPORTED,
                    "no backsolve kernel for dim %d, width %d, solver %d%s", D, H, d.solver,
                    precise ? " (FP32 products)" : "");
      }
      if (d.norm != GBDX_NORM_RMS && d.norm != GBDX_NORM_ADJOINT_SEMI) {
        delete p;
        return fail(GBDX_ERR_INVALID, "unknown norm %d", d.norm);
      }
    }
  } else {
    delete p;
    return fail(GBDX_ERR_UNSUPPORTED, "field %d (diffusion %d) is not available", d.field,
                d.diffusion);
  }
  *out = p;
  return GBDX_OK;
}

int gbdx_problem_destroy(gbdx_problem *problem) {
  delete problem;
  return GBDX_OK;
}

int gbdx_num_saves(const gbdx_problem *problem) { return problem ? problem->n_save : -1; }

int64_t gbdx_param_count(const gbdx_problem *problem) {
  if (!problem) return -1;
  const gbdx_problem_desc &d = problem->d;
  int64_t n = 0;
  if (d.field == GBDX_MLP)
    for (int l = 0; l < d.mlp_depth; l++)
      n += (int64_t)d.mlp_widths[l] * d.mlp_widths[l + 1] + d.mlp_widths[l + 1];
  if (d.field == GBDX_LINEAR) n += (int64_t)d.dim * d.dim;
  if (d.diffusion == GBDX_DIFF_TANH_DIAG) n += (int64_t)d.dim * d.dim + d.dim;
  return n;
}

size_t gbdx_workspace_size(const gbdx_problem *problem, int64_t batch) {
  if (!problem) return 0;
  WsLayout L;
  if (ws_layout(problem, batch, &L) != GBDX_OK) return 0;
  return L.total;
}

static int device_sm_count(int *sms) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  e = cudaDeviceGetAttribute(sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaDeviceGetAttribute");
  return GBDX_OK;
}

// Checks shared by the solve entry points and the kernel parameters they share.
static int prepare(const gbdx_problem *problem, int64_t batch, const double *t0,
                   const double *t1, const double *dt0, int64_t time_stride, const void *y0,
                   const void *args, int64_t args_stride, const void *params,
                   const double *save_ts, void *workspace, size_t workspace_bytes,
                   gbdx::SolveParams *out, WsLayout *L) {
  const gbdx_problem_desc &d = problem->d;
  if (!t0 || !t1 || !y0) return fail(GBDX_ERR_INVALID, "null input pointer");
  if (time_stride != 0 && time_stride != 1)
    return fail(GBDX_ERR_INVALID, "time_stride must be 0 or 1");
  if (d.controller == GBDX_CONSTANT && !dt0)
    return fail(GBDX_ERR_INVALID,
                "Constant step size solvers cannot select step size automatically; please "
                "pass a value for `dt0`.");
  if (d.n_ts + d.n_step_ts + d.n_jump_ts > 0 && !save_ts)
    return fail(GBDX_ERR_INVALID, "SaveAt(ts=...) or step_ts/jump_ts without times");
  if (d.n_args > 0 && !args) return fail(GBDX_ERR_INVALID, "field arguments missing");
  if (problem->mlp && !params) return fail(GBDX_ERR_INVALID, "MLP parameters missing");
  const int rc = ws_layout(problem, batch, L);
  if (rc != GBDX_OK) return rc;
  if (workspace_bytes < L->total || !workspace)
    return fail(GBDX_ERR_WORKSPACE, "workspace of %zu bytes is smaller than %zu",
                workspace_bytes, L->total);
  gbdx::SolveParams &P = *out;
  memset(&P, 0, sizeof P);
#ifdef GBDX_BOUNDS
  P.bounds = reinterpret_cast<unsigned long long *>(static_cast<char *>(workspace) + L->bounds);
  P.bounds_sink = static_cast<char *>(workspace) + L->bounds + 256;
#endif
  P.batch = batch;
  P.t0 = t0;
  P.t1 = t1;
  P.dt0 = dt0;
  P.time_stride = time_stride;
  P.y0 = y0;
  P.args = args;
  P.args_stride = args_stride;
  P.params = params;
  P.save_ts = save_ts;
  P.n_step_ts = d.n_step_ts;
  P.n_jump_ts = d.n_jump_ts;
  P.step_ts = save_ts ? save_ts + d.n_ts : nullptr;
  P.jump_ts = save_ts ? save_ts + d.n_ts + d.n_step_ts : nullptr;
  P.n_event = d.n_event;
  P.event_root = d.event_root ? 1 : 0;
  for (int e = 0; e < GBDX_MAX_EVENTS; e++) {
    P.ev_kind[e] = d.ev_kind[e];
    P.ev_dir[e] = d.ev_dir[e];
  }
  memcpy(P.ev_coef, d.ev_coef, sizeof P.ev_coef);
  P.newton_rtol = d.newton_rtol;
  P.newton_atol = d.newton_atol;
  P.controller = d.controller;
  P.rtol = d.rtol;
  P.atol = d.atol;
  P.safety = d.safety;
  P.factormin = d.factormin;
  P.factormax = d.factormax;
  P.has_dtmin = !isnan(d.dtmin);
  P.has_dtmax = !isnan(d.dtmax);
  P.dtmin = d.dtmin;
  P.dtmax = d.dtmax;
  P.force_dtmin = d.force_dtmin;
  P.c1 = problem->c1;
  P.c2 = problem->c2;
  P.c3 = problem->c3;
  P.rtol_f = float(d.rtol);
  P.atol_f = float(d.atol);
  P.safety_f = float(d.safety);
  P.factormin_f = float(d.factormin);
  P.factormax_f = float(d.factormax);
  P.c1_f = float(problem->c1);
  P.c2_f = float(problem->c2);
  P.c3_f = float(problem->c3);
  P.n_ts = d.n_ts;
  P.save_t0 = d.save_t0 ? 1 : 0;
  P.save_t1 = d.save_t1 ? 1 : 0;
  P.n_save = problem->n_save;
  P.max_steps = d.max_steps;
  P.queue = reinterpret_cast<unsigned long long *>(workspace);
  P.mlp = static_cast<const float *>(params);
  P.seed = d.seed;
  P.vbt_t0 = d.vbt_t0;
  P.vbt_len = d.vbt_t1 - d.vbt_t0;
  P.vbt_tol_unit = d.vbt_tol / (d.vbt_t1 - d.vbt_t0);
  // GB300 issues FP64 at ~1/64 of the FP32 rate: the per-evaluation division
  // and square root of the tree's time scaling are done once here.
  P.vbt_inv_len = 1.0 / (d.vbt_t1 - d.vbt_t0);
  P.vbt_sqrt_len = float(sqrt(d.vbt_t1 - d.vbt_t0));
  if (d.adjoint == GBDX_ADJ_RECURSIVE && (problem->bwd.launch || problem->adj.rc_bwd)) {
    char *w = static_cast<char *>(workspace);
    P.tape_t = reinterpret_cast<double *>(w + L->tape_t);
    P.tape_y = reinterpret_cast<float *>(w + L->tape_y);
    P.tape_n = reinterpret_cast<int32_t *>(w + L->tape_n);
    P.tape_stride = reinterpret_cast<int32_t *>(w + L->tape_s);
    // An even slot count keeps the online thinning exact: when the slots
    // fill at step n = C s, n is a multiple of the doubled stride 2 s.  The
    // plain form tapes every accepted step.
    P.checkpoints = (d.kernel == GBDX_KERNEL_PLAIN || problem->adj.rc_bwd)
                        ? d.max_steps + 1
                        : (d.checkpoints >= 4 ? (d.checkpoints / 2) * 2 : 2);
  }
  return GBDX_OK;
}

// Reset the work counter and (per-trajectory intervals) build the
// longest-first order, both on stream s.
// Whether the fused kernels take the trajectories longest-first: per-trajectory
// intervals and the schedule allowing it.
static bool longest_first_order(const gbdx_problem_desc &d, int64_t time_stride) {
  return time_stride == 1 && (d.schedule == GBDX_SCHED_LONGEST_FIRST ||
                              d.schedule == GBDX_SCHED_AUTO);
}

static int start_queue(const gbdx_problem *problem, gbdx::SolveParams &P, void *workspace,
                       cudaStream_t s) {
  const gbdx_problem_desc &d = problem->d;
  cudaError_t e = cudaMemsetAsync(workspace, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return cuda_fail(e, "queue reset");
  if (longest_first_order(d, P.time_stride)) {
    int32_t *order = nullptr;
    e = gbdx::build_longest_first_order(P.t0, P.t1, P.batch,
                                        static_cast<char *>(workspace) + kQueueBytes, &order,
                                        s);
    if (e != cudaSuccess) return cuda_fail(e, "work order");
    P.order = order;
  }
  return GBDX_OK;
}

}  // extern "C"

// The forward solve behind gbdx_solve_fwd and gbdx_solve_fwd_ex.
static int solve_fwd(const gbdx_problem *problem, int64_t batch, const double *t0,
                     const double *t1, const double *dt0, int64_t time_stride, const void *y0,
                     const void *args, int64_t args_stride, const void *params,
                     const double *save_ts, void *ys_out, double *ts_out, int32_t *result_out,
                     int32_t *stats_out, const gbdx_fwd_extras *ex, void *workspace,
                     size_t workspace_bytes, void *stream) {
  NvtxRange nvtx("gbdx_solve_fwd");
  double *dense_ts = ex ? ex->dense_ts : nullptr;
  void *dense_info = ex ? ex->dense_info : nullptr;
  int32_t *dense_n = ex ? ex->dense_n : nullptr;
  const gbdx_problem_desc &d = problem->d;
  const bool resume = ex && (ex->state_in || ex->state_out);
  if (resume && (d.n_step_ts > 0 || d.n_jump_ts > 0 || d.adjoint != GBDX_ADJ_NONE ||
                 !problem->ode_xo.launch))
    return fail(GBDX_ERR_UNSUPPORTED,
                "solver and controller states are available for forward solves without a "
                "ClipStepSizeController on the trajectory kernels and the fused MLP kernel");
  if (batch < 0) return fail(GBDX_ERR_INVALID, "negative batch");
  if (batch == 0) return GBDX_OK;
  if ((problem->n_save > 0 && (!ys_out || !ts_out)) || !result_out || !stats_out)
    return fail(GBDX_ERR_INVALID, "null output pointer");
  gbdx::SolveParams P;
  WsLayout L;
  int rc = prepare(problem, batch, t0, t1, dt0, time_stride, y0, args, args_stride, params,
                   save_ts, workspace, workspace_bytes, &P, &L);
  if (rc != GBDX_OK) return rc;
  P.ys_out = ys_out;
  P.ts_out = ts_out;
  P.result_out = result_out;
  P.stats_out = stats_out;
  P.save_steps = d.save_steps;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  rc = bounds_clear(P, s);
  if (rc != GBDX_OK) return rc;
  if (d.save_dense) {
    // The reference's dense buffers start full of +inf (_integrate.py:1315-1323);
    // the solve overwrites the recorded steps.
    const int stages = solver_stages(d.solver);
    const int64_t rec = int64_t(2 + stages) * d.dim;
    cudaError_t e = gbdx::launch_fill_inf_f64(dense_ts, batch * (int64_t(d.max_steps) + 1), s);
    if (e == cudaSuccess) {
      const int64_t n = batch * int64_t(d.max_steps) * rec;
      e = d.dtype == GBDX_F32 ? gbdx::launch_fill_inf_f32(static_cast<float *>(dense_info), n, s)
                              : gbdx::launch_fill_inf_f64(static_cast<double *>(dense_info), n, s);
    }
    if (e != cudaSuccess) return cuda_fail(e, "dense buffer fill");
    P.dense_ts = dense_ts;
    P.dense_info = dense_info;
    P.dense_n = dense_n;
  }
  if (d.n_event > 0) P.event_index = ex ? ex->event_index : nullptr;
  if (resume) {
    P.state_in = ex->state_in;
    P.state_out = ex->state_out;
  }
  if (d.save_steps > 0 && problem->n_save > 0) {
    // SaveAt(steps=n) reserves max_steps / n slots per trajectory, most of
    // them unused: fill them all in one pass before the solve
    cudaError_t e =
        d.dtype == GBDX_F32
            ? gbdx::launch_fill_saves_f32(static_cast<float *>(ys_out), ts_out, batch,
                                          problem->n_save, d.dim, t0, t1, time_stride, s)
            : gbdx::launch_fill_saves_f64(static_cast<double *>(ys_out), ts_out, batch,
                                          problem->n_save, d.dim, t0, t1, time_stride, s);
    if (e != cudaSuccess) return cuda_fail(e, "save buffer fill");
    P.saves_prefilled = 1;
  }

  if (L.has_ffrag) {
    // W0 (B[k][n] = W0[n][k], K = D, N = H) and W2 (K = H, N = D) as BF16
    // mma fragments for this launch
    const int D = d.dim, H = d.mlp_widths[1];
    const float *W = static_cast<const float *>(params);
    uint2 *f0 = reinterpret_cast<uint2 *>(static_cast<char *>(workspace) + L.ffrag);
    uint2 *f2 = reinterpret_cast<uint2 *>(static_cast<char *>(workspace) + L.ffrag +
                                          up256(size_t(D) * H * 2));
    cudaError_t e = gbdx::launch_frag_prep(W, D, D, H, 1, f0, s);
    if (e == cudaSuccess)
      e = gbdx::launch_frag_prep(W + size_t(H) * D + H + size_t(H) * H + H, H, H, D, 1, f2, s);
    if (e != cudaSuccess) return cuda_fail(e, "weight fragments");
    P.w0f = f0;
    P.w2f = f2;
  }
  gbdx::LaunchCfg cfg;
  cfg.kernel = d.kernel == GBDX_KERNEL_PLAIN ? GBDX_KERNEL_PLAIN : GBDX_KERNEL_FUSED;
  cfg.block = problem->mlp ? problem->mlp_block : (d.block_threads > 0 ? d.block_threads : 64);
  if (!problem->mlp && (cfg.block % 32 != 0 || cfg.block > 256))
    return fail(GBDX_ERR_INVALID, "block_threads must be a multiple of 32 up to 256");
  cfg.grid = 1;
  if (cfg.kernel == GBDX_KERNEL_FUSED) {
    int sms = 0;
    rc = device_sm_count(&sms);
    if (rc != GBDX_OK) return rc;
    int occ = 0;
    cudaError_t e = (resume ? problem->ode_xo : problem->ode).occupancy(cfg.block, &occ);
    if (e != cudaSuccess) return cuda_fail(e, "occupancy query");
    if (occ < 1) occ = 1;
    int per_sm = d.ctas_per_sm;
    if (per_sm <= 0 && problem->mlp) per_sm = occ;
    if (per_sm <= 0) {
      // Keep about B / 1.7 lanes resident: enough warps to hide the step's
      // dependency latency, few enough that lanes refill from the queue and
      // the longest trajectories (started first) meet little contention
      // (measured on the uneven Van der Pol batch).
      per_sm = (int)((double)batch / (1.7 * cfg.block * sms) + 0.5);
      if (per_sm < 1) per_sm = 1;
      if (per_sm > occ) per_sm = occ;
    }
    int64_t grid = (int64_t)sms * per_sm;
    const int rows = problem->mlp ? problem->rows_per_cta : cfg.block;
    const int64_t needed = (batch + rows - 1) / rows;
    if (grid > needed) grid = needed;
    cfg.grid = (int)grid;
    rc = start_queue(problem, P, workspace, s);
    if (rc != GBDX_OK) return rc;
  }
  // resume records are read and written by the extended-output form
  cudaError_t e = (resume ? problem->ode_xo : problem->ode).launch(P, cfg, s);
  if (e != cudaSuccess) return cuda_fail(e, "kernel launch");
  return bounds_report(P, s, "gbdx_solve_fwd");
}

extern "C" {

int gbdx_solve_fwd(const gbdx_problem *problem, int64_t batch, const double *t0,
                   const double *t1, const double *dt0, int64_t time_stride,
                   const void *y0, const void *args, int64_t args_stride,
                   const void *params, const double *save_ts, void *ys_out,
                   double *ts_out, int32_t *result_out, int32_t *stats_out,
                   void *workspace, size_t workspace_bytes, void *stream) {
  if (!problem) return fail(GBDX_ERR_INVALID, "null problem");
  if (problem->d.save_dense || problem->d.n_event > 0)
    return fail(GBDX_ERR_INVALID,
                "the problem saves the dense output or has an event: solve it with "
                "gbdx_solve_fwd_ex");
  return solve_fwd(problem, batch, t0, t1, dt0, time_stride, y0, args, args_stride, params,
                   save_ts, ys_out, ts_out, result_out, stats_out, nullptr, workspace,
                   workspace_bytes, stream);
}

int gbdx_solve_fwd_ex(const gbdx_problem *problem, int64_t batch, const double *t0,
                      const double *t1, const double *dt0, int64_t time_stride,
                      const void *y0, const void *args, int64_t args_stride,
                      const void *params, const double *save_ts, void *ys_out,
                      double *ts_out, int32_t *result_out, int32_t *stats_out,
                      const gbdx_fwd_extras *extras, void *workspace, size_t workspace_bytes,
                      void *stream) {
  if (!problem) return fail(GBDX_ERR_INVALID, "null problem");
  if (problem->d.save_dense && batch > 0 &&
      (!extras || !extras->dense_ts || !extras->dense_info || !extras->dense_n))
    return fail(GBDX_ERR_INVALID,
                "the problem saves the dense output: dense_ts, dense_info and dense_n are "
                "required");
  return solve_fwd(problem, batch, t0, t1, dt0, time_stride, y0, args, args_stride, params,
                   save_ts, ys_out, ts_out, result_out, stats_out, extras, workspace,
                   workspace_bytes, stream);
}

int gbdx_dense_evaluate(const gbdx_problem *problem, int64_t batch, const double *t0,
                        const double *t1, int64_t time_stride, const void *y0,
                        const double *dense_ts, const void *dense_info,
                        const int32_t *dense_n, int64_t Q, const double *query,
                        int64_t query_stride, int left, int order, void *out, void *stream) {
  NvtxRange nvtx("gbdx_dense_evaluate");
  if (!problem) return fail(GBDX_ERR_INVALID, "null problem");
  const gbdx_problem_desc &d = problem->d;
  if (!d.save_dense)
    return fail(GBDX_ERR_INVALID, "the problem was not created with SaveAt(dense=True)");
  if (batch < 0 || Q < 0) return fail(GBDX_ERR_INVALID, "negative batch or query count");
  if (time_stride != 0 && time_stride != 1)
    return fail(GBDX_ERR_INVALID, "time_stride must be 0 or 1");
  if (query_stride != 0 && query_stride != Q)
    return fail(GBDX_ERR_INVALID, "query_stride must be 0 (shared) or Q (per trajectory)");
  if (order != 0 && order != 1)
    return fail(GBDX_ERR_INVALID, "order must be 0 (evaluate) or 1 (derivative)");
  if (batch == 0 || Q == 0) return GBDX_OK;
  if (!t0 || !t1 || !y0 || !dense_ts || !dense_info || !dense_n || !query || !out)
    return fail(GBDX_ERR_INVALID, "null pointer argument");
  gbdx::DenseEvalArgs A;
  A.batch = batch;
  A.Q = Q;
  A.q_stride = query_stride;
  A.time_stride = time_stride;
  A.dim = d.dim;
  A.max_steps = d.max_steps;
  A.left = left ? 1 : 0;
  A.order = order;
  A.t0 = t0;
  A.t1 = t1;
  A.query = query;
  A.dense_ts = dense_ts;
  A.y0 = y0;
  A.dense_info = dense_info;
  A.dense_n = dense_n;
  A.out = out;
  cudaError_t e = gbdx::launch_dense_evaluate(d.solver, d.dtype, A,
                                              reinterpret_cast<cudaStream_t>(stream));
  if (e != cudaSuccess) return cuda_fail(e, "dense evaluation launch");
  return GBDX_OK;
}

int gbdx_solve_bwd(const gbdx_problem *problem, int64_t batch, const double *t0,
                   const double *t1, const double *dt0, int64_t time_stride,
                   const void *y0, const void *args, int64_t args_stride,
                   const void *params, const double *save_ts, const void *grad_ys,
                   void *grad_y0, void *grad_params, void *workspace,
                   size_t workspace_bytes, void *stream) {
  NvtxRange nvtx("gbdx_solve_bwd");
  if (!problem) return fail(GBDX_ERR_INVALID, "null problem");
  if (problem->d.adjoint != GBDX_ADJ_RECURSIVE ||
      (!problem->bwd.launch && !problem->adj.rc_bwd))
    return fail(GBDX_ERR_UNSUPPORTED,
                "the problem was not created with RecursiveCheckpointAdjoint");
  if (batch < 0) return fail(GBDX_ERR_INVALID, "negative batch");
  if (!grad_ys || !grad_y0 || !grad_params)
    return fail(GBDX_ERR_INVALID, "null gradient pointer");
  gbdx::SolveParams P;
  WsLayout L;
  int rc = prepare(problem, batch, t0, t1, dt0, time_stride, y0, args, args_stride, params,
                   save_ts, workspace, workspace_bytes, &P, &L);
  if (rc != GBDX_OK) return rc;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  rc = bounds_clear(P, s);
  if (rc != GBDX_OK) return rc;
  if (problem->adj.rc_bwd) {
    // analytic fields: grad_params receives dL/dargs, per trajectory
    // [batch, n_args] when args has a row per trajectory, else [n_args].  The
    // tape rows are the forward's queue slots: its work order (left in the
    // workspace by the forward) maps them back to trajectories.
    if (problem->d.kernel != GBDX_KERNEL_PLAIN && longest_first_order(problem->d, time_stride))
      P.order = reinterpret_cast<const int32_t *>(static_cast<char *>(workspace) + kQueueBytes);
    gbdx::AdjParams A;
    memset(&A, 0, sizeof A);
    A.grad_ys = grad_ys;
    A.grad_y0 = grad_y0;
    A.grad_args = args_stride != 0 ? grad_params : static_cast<char *>(workspace) + L.scratch;
    cudaError_t e = problem->adj.rc_bwd(P, A, s);
    if (e != cudaSuccess) return cuda_fail(e, "backward launch");
    if (args_stride == 0) {
      e = problem->d.dtype == GBDX_F32
              ? gbdx::launch_reduce_arg_rows_f32(A.grad_args, batch, problem->adj.n_args,
                                                 grad_params, s)
              : gbdx::launch_reduce_arg_rows_f64(A.grad_args, batch, problem->adj.n_args,
                                                 grad_params, s);
      if (e != cudaSuccess) return cuda_fail(e, "gradient reduction");
    }
    return bounds_report(P, s, "gbdx_solve_bwd");
  }
  const int np = int(gbdx_param_count(problem));
  char *w = static_cast<char *>(workspace);
  gbdx::BwdParams Q;
  Q.grad_ys = static_cast<const float *>(grad_ys);
  Q.grad_y0 = static_cast<float *>(grad_y0);
  Q.part_sum = reinterpret_cast<float *>(w + L.psum);
  Q.part_comp = reinterpret_cast<float *>(w + L.pcomp);
  Q.scratch = reinterpret_cast<float *>(w + L.scratch);
  Q.seg_max = L.seg_max;
  Q.n_params = np;
  cudaError_t e = cudaMemsetAsync(w + L.psum, 0, L.bounds - L.psum, s);
  if (e != cudaSuccess) return cuda_fail(e, "gradient partial reset");
  const bool plain = problem->d.kernel == GBDX_KERNEL_PLAIN;
  if (batch > 0) {
    if (!plain) {
      rc = start_queue(problem, P, workspace, s);
      if (rc != GBDX_OK) return rc;
    }
    e = problem->bwd.launch(P, Q, L.n_cta, s);
    if (e != cudaSuccess) return cuda_fail(e, "backward launch");
  }
  if (plain)
    e = gbdx::launch_reduce_columns(Q.part_sum, np, batch, static_cast<float *>(grad_params), s);
  else if (problem->d.mlp_precision == GBDX_MLP_FP32)
    e = gbdx::launch_reduce_partials(Q.part_sum, Q.part_comp, batch > 0 ? L.n_cta : 0, np,
                                     static_cast<float *>(grad_params), s);
  else  // the tensor-core mode keeps the weight blocks in fragment order
    e = gbdx::launch_reduce_partials_frag(
        Q.part_sum, Q.part_comp, batch > 0 ? L.n_cta : 0, problem->d.dim,
        problem->d.mlp_widths[1], problem->d.diffusion != GBDX_DIFF_NONE,
        static_cast<float *>(grad_params), s);
  if (e != cudaSuccess) return cuda_fail(e, "gradient reduction");
  return bounds_report(P, s, "gbdx_solve_bwd");
}

int gbdx_backsolve_bwd(const gbdx_problem *problem, int64_t batch, const double *t0,
                       const double *t1, const double *dt0, int64_t time_stride,
                       const double *save_ts, const void *ys, const void *grad_ys,
                       const void *params, void *grad_y0, void *grad_params,
                       int32_t *result_out, int32_t *stats_out, void *workspace,
                       size_t workspace_bytes, void *stream) {
  return gbdx_backsolve_bwd_ex(problem, batch, t0, t1, dt0, time_stride, save_ts, ys, grad_ys,
                               nullptr, 0, params, grad_y0, grad_params, result_out,
                               stats_out, workspace, workspace_bytes, stream);
}

int gbdx_backsolve_bwd_ex(const gbdx_problem *problem, int64_t batch, const double *t0,
                          const double *t1, const double *dt0, int64_t time_stride,
                          const double *save_ts, const void *ys, const void *grad_ys,
                          const void *args, int64_t args_stride, const void *params,
                          void *grad_y0, void *grad_params, int32_t *result_out,
                          int32_t *stats_out, void *workspace, size_t workspace_bytes,
                          void *stream) {
  NvtxRange nvtx("gbdx_backsolve_bwd");
  if (!problem) return fail(GBDX_ERR_INVALID, "null problem");
  const gbdx_problem_desc &d = problem->d;
  if (d.adjoint != GBDX_ADJ_BACKSOLVE || (!problem->bs.launch && !problem->adj.bs_bwd))
    return fail(GBDX_ERR_UNSUPPORTED,
                "the problem was not created with BacksolveAdjoint");
  if (batch < 0) return fail(GBDX_ERR_INVALID, "negative batch");
  if (!grad_ys || !grad_y0 || !grad_params || !ys || !result_out || !stats_out)
    return fail(GBDX_ERR_INVALID, "null pointer argument");
  if (batch > 0 && !save_ts) return fail(GBDX_ERR_INVALID, "the forward's saved times are missing");
  gbdx::SolveParams P;
  WsLayout L;
  // y0 is not read by the backward; the saved states stand in for the check.
  int rc = prepare(problem, batch, t0, t1, dt0, time_stride, ys, args, args_stride, params,
                   save_ts, workspace, workspace_bytes, &P, &L);
  if (rc != GBDX_OK) return rc;
  P.result_out = result_out;
  P.stats_out = stats_out;
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
  rc = bounds_clear(P, s);
  if (rc != GBDX_OK) return rc;
  if (problem->adj.bs_bwd) {
    // analytic fields: grad_params receives dL/dargs as in gbdx_solve_bwd
    gbdx::AdjParams A;
    memset(&A, 0, sizeof A);
    A.grad_ys = grad_ys;
    A.ys = ys;
    A.grad_y0 = grad_y0;
    A.grad_args = args_stride != 0 ? grad_params : static_cast<char *>(workspace) + L.scratch;
    A.track_args = L.track ? 1 : 0;
    cudaError_t e = problem->adj.bs_bwd(P, A, s);
    if (e != cudaSuccess) return cuda_fail(e, "backsolve launch");
    if (args_stride == 0) {
      e = d.dtype == GBDX_F32
              ? gbdx::launch_reduce_arg_rows_f32(A.grad_args, batch, problem->adj.n_args,
                                                 grad_params, s)
              : gbdx::launch_reduce_arg_rows_f64(A.grad_args, batch, problem->adj.n_args,
                                                 grad_params, s);
      if (e != cudaSuccess) return cuda_fail(e, "gradient reduction");
    }
    return bounds_report(P, s, "gbdx_backsolve_bwd");
  }
  const int np = int(gbdx_param_count(problem));
  const int D = d.dim, H = d.mlp_widths[1];
  char *w = static_cast<char *>(workspace);
  gbdx::BsParams Q;
  memset(&Q, 0, sizeof Q);
  Q.ys = static_cast<const float *>(ys);
  Q.grad_ys = static_cast<const float *>(grad_ys);
  Q.grad_y0 = static_cast<float *>(grad_y0);
  Q.psum = reinterpret_cast<float *>(w + L.psum);
  Q.pcomp = reinterpret_cast<float *>(w + L.pcomp);
  Q.rec = reinterpret_cast<float *>(w + L.rec);
  Q.ath = reinterpret_cast<float *>(w + L.ath);
  Q.track = L.track ? 1 : 0;
  Q.n_norm = float(L.track ? 2 * D + np : 2 * D);
  cudaError_t e;
  if (problem->d.kernel == GBDX_KERNEL_PLAIN) {
    e = problem->bs.launch(P, Q, 0, s);
    if (e != cudaSuccess) return cuda_fail(e, "plain backsolve launch");
    e = gbdx::launch_reduce_columns(Q.ath, np, batch, static_cast<float *>(grad_params), s);
    if (e != cudaSuccess) return cuda_fail(e, "gradient reduction");
    return bounds_report(P, s, "gbdx_backsolve_bwd");
  }
  e = cudaMemsetAsync(w + L.psum, 0, L.ath - L.psum, s);
  if (e != cudaSuccess) return cuda_fail(e, "gradient partial reset");
  if (batch > 0) {
    if (problem->bs.gfrag) {
      const size_t part = up256(size_t(D) * H * 2);
      uint2 *f = reinterpret_cast<uint2 *>(w + L.frag);
      const float *W = static_cast<const float *>(params);
      const int ow0 = 0, ow2 = H * D + H + H * H + H;
      Q.w0f = f;
      Q.w0v = reinterpret_cast<uint2 *>(w + L.frag + part);
      Q.w2f = reinterpret_cast<uint2 *>(w + L.frag + 2 * part);
      Q.w2v = reinterpret_cast<uint2 *>(w + L.frag + 3 * part);
      // layer 0 forward: B[k][n] = W0[n][k] (K = D, N = H); VJP: B = W0 (K = H, N = D)
      e = gbdx::launch_frag_prep(W + ow0, D, D, H, 1, const_cast<uint2 *>(Q.w0f), s);
      if (e == cudaSuccess)
        e = gbdx::launch_frag_prep(W + ow0, D, H, D, 0, const_cast<uint2 *>(Q.w0v), s);
      // layer 2 forward: B[k][n] = W2[n][k] (K = H, N = D); VJP: B = W2 (K = D, N = H)
      if (e == cudaSuccess)
        e = gbdx::launch_frag_prep(W + ow2, H, H, D, 1, const_cast<uint2 *>(Q.w2f), s);
      if (e == cudaSuccess)
        e = gbdx::launch_frag_prep(W + ow2, H, D, H, 0, const_cast<uint2 *>(Q.w2v), s);
      if (e != cudaSuccess) return cuda_fail(e, "weight fragments");
    }
    e = cudaMemsetAsync(workspace, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return cuda_fail(e, "queue reset");
    e = problem->bs.launch(P, Q, L.n_cta, s);
    if (e != cudaSuccess) return cuda_fail(e, "backsolve launch");
  }
  // the tensor-core mode keeps the weight blocks in fragment order
  if (d.mlp_precision == GBDX_MLP_FP32)
    e = gbdx::launch_reduce_partials(Q.psum, Q.pcomp, batch > 0 ? L.n_cta : 0, np,
                                     static_cast<float *>(grad_params), s);
  else
    e = gbdx::launch_reduce_partials_frag(Q.psum, Q.pcomp, batch > 0 ? L.n_cta : 0, D, H, 0,
                                          static_cast<float *>(grad_params), s);
  if (e != cudaSuccess) return cuda_fail(e, "gradient reduction");
  return bounds_report(P, s, "gbdx_backsolve_bwd");
}

}  // extern "C"
