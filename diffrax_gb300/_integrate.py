"""diffeqsolve: lowers Diffrax-style objects to a gbdx problem and runs it.

Batched ("vmapped") semantics: ``y0`` is [B, dim]; ``t0``, ``t1`` and ``dt0``
are scalars or [B]; ``args`` is shared ([n_args]) or per trajectory
([B, n_args]).  Every array lives on the GPU during the solve; host tensors are
copied in (and the caller copies results out).  Reference entry point:
diffrax/_integrate.py:888-1543.
"""
from __future__ import annotations

import ctypes
import math
from typing import Any, Optional

import torch

from . import _lib
from ._core import (
    RESULT_MESSAGES, RESULTS, AbstractField, BacksolveAdjoint, ClipStepSizeController,
    ConstantStepSize, ControlTerm, Event, LinearCondition, SteadyStateCondition,
    Euler, MultiTerm, SpaceTimeLevyArea, ODETerm, OrnsteinUhlenbeck, PIDController,
    RecursiveCheckpointAdjoint, SaveAt, Solution, VirtualBrownianTree, adjoint_rms_seminorm,
    _tree_leaves, _tree_unflatten)

KERNELS = {"auto": 0, "plain": 1, "fused": 2, "tc": 3}
SCHEDULES = {"auto": 0, "index": 1, "longest_first": 2}


def _split_terms(terms):
    """Return (drift_field, diffusion, brownian) from ODETerm or
    MultiTerm(ODETerm, ControlTerm)."""
    if isinstance(terms, ODETerm):
        return terms.vector_field, None, None
    if isinstance(terms, MultiTerm):
        drift = diff = None
        for t in terms.terms:
            if isinstance(t, ODETerm) and drift is None:
                drift = t.vector_field
            elif isinstance(t, ControlTerm) and diff is None:
                diff = t
            else:
                raise NotImplementedError("MultiTerm must be (ODETerm, ControlTerm)")
        if drift is None or diff is None:
            raise NotImplementedError("MultiTerm must be (ODETerm, ControlTerm)")
        if not isinstance(diff.control, VirtualBrownianTree):
            raise NotImplementedError("ControlTerm must be driven by a VirtualBrownianTree")
        return drift, diff, diff.control
    if isinstance(terms, ControlTerm):
        raise NotImplementedError("a bare ControlTerm is not supported; use "
                                  "MultiTerm(ODETerm(...), ControlTerm(...))")
    raise TypeError(f"unsupported terms {terms!r}")


def _lower_event(event: Event, controller, dim: int) -> dict:
    """Descriptor fields of an Event (include/gbdx.h: GBDX_EV_*)."""
    kinds, dirs, coef = [], [], []
    inner = controller.controller if isinstance(controller, ClipStepSizeController) \
        else controller
    for c, d in zip(event._conds, event._dirs):
        dirs.append(0 if d is None else (1 if d else 2))
        if isinstance(c, LinearCondition):
            if len(c.y_coeffs) > dim:
                raise ValueError(f"the condition has {len(c.y_coeffs)} state coefficients "
                                 f"for a state of dimension {dim}")
            kinds.append(1 if c.boolean else 0)
            coef += c.y_coeffs + [0.0] * (4 - len(c.y_coeffs)) + [c.t_coeff, c.offset]
        else:
            rtol, atol = c.rtol, c.atol
            if rtol is None or atol is None:
                if not isinstance(inner, PIDController):
                    raise ValueError(
                        "The `rtol`, `atol`, and `norm` for `steady_state_event` default to "
                        "the values used with an adaptive step size controller (such as "
                        "`diffrax.PIDController`). Either use an adaptive step size "
                        "controller, or specify these tolerances manually.")
                rtol = inner.rtol if rtol is None else rtol
                atol = inner.atol if atol is None else atol
            kinds.append(2)
            coef += [float(rtol), float(atol), 0.0, 0.0, 0.0, 0.0]
    rf = event.root_finder
    return dict(n_event=len(kinds), event_root=int(rf is not None), ev_kind=kinds,
                ev_dir=dirs, ev_coef=coef, newton_rtol=rf.rtol if rf else 1e-5,
                newton_atol=rf.atol if rf else 1e-5)


def lower(terms, solver, stepsize_controller, saveat: SaveAt, *, dim: int, dtype,
          max_steps: int, n_ts: int, adjoint=None, kernel: str = "auto",
          block_threads: int = 0, ctas_per_sm: int = 0, schedule: str = "auto",
          event: Optional[Event] = None) -> dict:
    """Descriptor fields (gbdx_problem_desc) for one solve."""
    drift, diff, bm = _split_terms(terms)
    if not isinstance(drift, AbstractField):
        raise TypeError("the drift must be a registered vector field")
    f = dict(solver=solver.solver_id, field=drift.field_id, dim=int(dim),
             n_ts=int(n_ts), save_t0=int(saveat.t0),
             save_t1=int(saveat.t1 or getattr(saveat, "state_only", False)),
             max_steps=int(max_steps), n_args=drift.n_args,
             dtype=0 if dtype == torch.float32 else 1, kernel=KERNELS[kernel],
             block_threads=int(block_threads), ctas_per_sm=int(ctas_per_sm),
             rtol=0.0, atol=0.0, pcoeff=0.0, icoeff=1.0, dcoeff=0.0, safety=0.9,
             factormin=0.2, factormax=10.0, dtmin=None, dtmax=None, force_dtmin=1,
             error_order=0.0, mlp_depth=0, mlp_widths=(), diffusion=0, vbt_t0=0.0,
             vbt_t1=1.0, vbt_tol=1e-3, seed=0, norm=0, adjoint=0, checkpoints=0,
             schedule=SCHEDULES[schedule], mlp_precision=0,
             save_steps=int(saveat.steps), save_dense=int(saveat.dense), n_step_ts=0,
             n_jump_ts=0, n_event=0, event_root=0, ev_kind=(), ev_dir=(), levy_area=0,
             newton_rtol=1e-5, newton_atol=1e-5, ev_coef=())
    if event is not None:
        f.update(_lower_event(event, stepsize_controller, int(dim)))
    if hasattr(drift, "lower_fields"):
        f.update(drift.lower_fields(dim))
    if isinstance(stepsize_controller, ClipStepSizeController):
        clip = stepsize_controller
        f.update(n_step_ts=0 if clip.step_ts is None else int(clip.step_ts.size),
                 n_jump_ts=0 if clip.jump_ts is None else int(clip.jump_ts.size))
        stepsize_controller = clip.controller
    if isinstance(stepsize_controller, PIDController):
        c = stepsize_controller
        f.update(controller=1, rtol=float(c.rtol), atol=float(c.atol),
                 pcoeff=float(c.pcoeff), icoeff=float(c.icoeff), dcoeff=float(c.dcoeff),
                 safety=float(c.safety), factormin=float(c.factormin),
                 factormax=float(c.factormax),
                 dtmin=None if c.dtmin is None else float(c.dtmin),
                 dtmax=None if c.dtmax is None else float(c.dtmax),
                 force_dtmin=int(bool(c.force_dtmin)),
                 error_order=0.0 if c.error_order is None else float(c.error_order),
                 norm=1 if c.norm is adjoint_rms_seminorm else 0)
    elif isinstance(stepsize_controller, ConstantStepSize):
        f.update(controller=0)
    else:
        raise TypeError(f"unsupported step size controller {stepsize_controller!r}")
    if diff is not None:
        if isinstance(solver, Euler) and isinstance(stepsize_controller, PIDController):
            raise ValueError("An SDE should not be solved with adaptive step sizes with "
                             "Euler's method, as it may not converge to the correct "
                             "solution.")
        vf = diff.vector_field
        if isinstance(vf, OrnsteinUhlenbeck):
            f["diffusion"] = 1
        elif hasattr(vf, "diffusion_id"):
            f["diffusion"] = vf.diffusion_id
        else:
            raise NotImplementedError("unsupported diffusion")
        levy = getattr(bm, "levy_area", None) is SpaceTimeLevyArea
        f.update(vbt_t0=bm.t0, vbt_t1=bm.t1, vbt_tol=bm.tol, seed=bm.key,
                 levy_area=int(levy))
        if getattr(solver, "minimal_levy_area", None) is SpaceTimeLevyArea and not levy:
            # srk.py:374-379
            raise ValueError("The Brownian increment BrownianIncrement does not have the "
                             "minimal Levy Area SpaceTimeLevyArea.")
    elif getattr(solver, "minimal_levy_area", None) is not None:
        raise ValueError(f"{type(solver).__name__} solves SDEs: terms must be "
                         "MultiTerm(ODETerm, ControlTerm)")
    if isinstance(adjoint, RecursiveCheckpointAdjoint):
        cp = adjoint.checkpoints
        if cp is None:
            cp = max(1, math.ceil(math.log2(max(int(max_steps), 2))))
        f.update(adjoint=1, checkpoints=int(cp))
    elif isinstance(adjoint, BacksolveAdjoint):
        f.update(adjoint=2)
    return f


def _device():
    if not torch.cuda.is_available():
        raise RuntimeError("diffrax_gb300 needs a CUDA device: there is no CPU path")
    return torch.device("cuda", torch.cuda.current_device())


def _to_dev(x: torch.Tensor, dev, dtype=None) -> torch.Tensor:
    """x on the device.  A host tensor in page-locked memory is copied
    asynchronously on the current stream (the solve that reads it is queued
    behind the copy, so the host does not wait for it); other tensors as by
    Tensor.to."""
    nb = x.device.type == "cpu" and x.is_pinned()
    return x.to(device=dev, dtype=dtype or x.dtype, non_blocking=nb)


# Device copies of scalar times (value, device, length) -> FP64 array, so that
# a repeated solve with Python-number times neither copies from the host nor
# launches a fill.  The kernels only read them; entries made during a CUDA
# graph capture are not kept (their memory belongs to the graph).
_SCALAR_TIMES: dict = {}


def _scalar_time(x, n: int, dev) -> torch.Tensor:
    key = (float(x), dev.index, n)
    t = _SCALAR_TIMES.get(key)
    if t is None:
        t = torch.full((n,), float(x), dtype=torch.float64, device=dev)
        if not _capturing():
            if len(_SCALAR_TIMES) >= 32:
                _SCALAR_TIMES.clear()
            _SCALAR_TIMES[key] = t
    return t


# max_steps=None: an unbounded loop (_integrate.py:1283-1292, 1316-1319); the
# kernels take the largest step count they can count to
UNBOUNDED_STEPS = 2**31 - 1


def _max_steps(max_steps, saveat, recursive_grad):
    """The step bound handed to the kernels, with the reference's checks of
    max_steps=None (_integrate.py:1283-1292, 1316-1319; _adjoint.py:283-292)."""
    if max_steps is not None:
        return int(max_steps)
    if saveat.steps:
        raise ValueError("`max_steps=None` is incompatible with saving at `steps=n`")
    if saveat.dense:
        raise ValueError("`max_steps=None` is incompatible with `saveat.dense=True`")
    if recursive_grad:
        # the tape holds every accepted step's time, so it needs the bound
        raise NotImplementedError("gradients through RecursiveCheckpointAdjoint need a "
                                  "finite max_steps")
    return UNBOUNDED_STEPS


def _time_arrays(t0, t1, dt0, B, dev):
    """t0, t1, dt0 as FP64 device arrays: one entry each (stride 0) when all
    are scalars, else B entries each (stride 1)."""
    xs = [t0, t1] + ([dt0] if dt0 is not None else [])
    tens = [_to_dev(x, dev, torch.float64).reshape(-1) if isinstance(x, torch.Tensor) else None
            for x in xs]
    per_traj = any(t is not None and t.numel() != 1 for t in tens)
    n = B if per_traj else 1
    out = []
    for x, t in zip(xs, tens):
        if t is None:
            out.append(_scalar_time(x, n, dev))
        elif t.numel() == 1 and n > 1:
            out.append(t.expand(n).contiguous())
        elif t.numel() != n:
            raise ValueError("t0, t1 and dt0 must be scalars or have one entry per trajectory")
        else:
            out.append(t.contiguous())
    return out[0], out[1], (out[2] if dt0 is not None else None), int(per_traj)


def _capturing() -> bool:
    return torch.cuda.is_available() and torch.cuda.is_current_stream_capturing()


def _host_checks(t0, t1, dt0, ts, tstride):
    """The reference's dt0-sign and saveat.ts checks (_integrate.py:1036-1045,
    1222-1235).  Skipped while a CUDA graph is being captured."""
    if _capturing():
        return
    if dt0 is not None:
        if bool(((t1 - t0) * dt0 < 0).any()):
            raise ValueError("Must have (t1 - t0) * dt0 >= 0")
    if ts is not None and ts.numel() > 0:
        direction = torch.where(t0 < t1, 1.0, -1.0)
        tsd = ts.reshape(1, -1) * direction.reshape(-1, 1)
        if ts.numel() > 1 and bool((tsd[:, 1:] < tsd[:, :-1]).any()):
            raise RuntimeError("saveat.ts must be increasing or decreasing.")
        lo = (t0 * direction).reshape(-1, 1)
        hi = (t1 * direction).reshape(-1, 1)
        if bool(((tsd > hi) | (tsd < lo)).any()):
            raise RuntimeError("saveat.ts must lie between t0 and t1.")


class Lowered:
    """A lowered, validated solve ready for the C ABI (reused by autograd)."""

    def __init__(self, terms, solver, t0, t1, dt0, y0, args, saveat, stepsize_controller,
                 adjoint, max_steps, kernel, block_threads, ctas_per_sm, schedule="auto",
                 want_grad=False, event=None, throw=True):
        dev = _device()
        # diffrax/_adjoint.py:623-634: the backward solve of BacksolveAdjoint
        # takes the forward's `throw` unless its kwargs override it
        self.throw = bool(throw)
        if not isinstance(y0, torch.Tensor):
            y0 = torch.as_tensor(y0)
        if y0.dtype not in (torch.float32, torch.float64):
            y0 = y0.to(torch.float64)
        if y0.dim() != 2:
            raise ValueError("y0 must be [batch, dim] (vmapped semantics)")
        self.dtype = y0.dtype
        self.B, self.dim = int(y0.shape[0]), int(y0.shape[1])
        self.y0 = _to_dev(y0, dev).contiguous()
        max_steps = _max_steps(max_steps, saveat, want_grad and not isinstance(
            adjoint, BacksolveAdjoint))
        ts = saveat.ts
        if ts is not None:
            ts = torch.as_tensor(ts, dtype=torch.float64).to(dev).reshape(-1).contiguous()
        n_ts = 0 if ts is None else int(ts.numel())
        # the solve's times: SaveAt ts, then a ClipStepSizeController's sorted
        # step_ts and jump_ts (include/gbdx.h)
        clip_parts = []
        if isinstance(stepsize_controller, ClipStepSizeController):
            clip_parts = [torch.as_tensor(v, dtype=torch.float64).to(dev)
                          for v in (stepsize_controller.step_ts, stepsize_controller.jump_ts)
                          if v is not None]
        self.save_ts = (torch.cat(([ts] if ts is not None else []) + clip_parts).contiguous()
                        if clip_parts else ts)
        # The adjoint shapes the problem only when a gradient will be taken:
        # a plain forward solve records no tape.
        self.adjoint = adjoint if want_grad else None
        backsolve = isinstance(self.adjoint, BacksolveAdjoint)
        self.fields = lower(terms, solver, stepsize_controller, saveat, dim=self.dim,
                            dtype=self.dtype, max_steps=max_steps, n_ts=n_ts,
                            adjoint=None if backsolve else self.adjoint, kernel=kernel,
                            block_threads=block_threads, ctas_per_sm=ctas_per_sm,
                            schedule=schedule, event=event)
        drift = _split_terms(terms)[0]
        self.drift = drift
        self.problem = _lib.get_problem(self.fields)
        self.t0, self.t1, self.dt0, self.tstride = _time_arrays(t0, t1, dt0, self.B, dev)
        _host_checks(self.t0, self.t1, self.dt0, ts, self.tstride)
        self.bwd_problem = None
        if backsolve:
            # The backward solve reuses the forward's solver and controller
            # unless BacksolveAdjoint(**kwargs) overrides them
            # (diffrax/_adjoint.py:623-633).
            kw = self.adjoint.kwargs
            self.bwd_fields = lower(terms, kw.get("solver", solver),
                                    kw.get("stepsize_controller", stepsize_controller), saveat,
                                    dim=self.dim, dtype=self.dtype,
                                    max_steps=_max_steps(kw.get("max_steps", max_steps),
                                                         saveat, False), n_ts=n_ts,
                                    adjoint=self.adjoint, kernel=kernel, schedule=schedule)
            self.bwd_problem = _lib.get_problem(self.bwd_fields)
            self.bwd_throw = bool(kw.get("throw", throw))
            self.bwd_dt0 = self.dt0
            if kw.get("dt0") is not None:
                self.bwd_dt0 = _time_arrays(t0, t1, kw["dt0"], self.B, dev)[2]
                if self.bwd_dt0.numel() != self.t0.numel():
                    self.bwd_dt0 = self.bwd_dt0.expand(self.t0.numel()).contiguous()
            if self.bwd_fields["controller"] == 0 and self.bwd_dt0 is None:
                raise ValueError("Constant step size solvers cannot select step size "
                                 "automatically; please pass a value for `dt0`.")
        na = drift.n_args
        if na:
            if args is None:
                raise ValueError(f"{type(drift).__name__} needs args with {na} entries")
            a = _to_dev(torch.as_tensor(args), dev, self.dtype)
            if a.numel() == na:
                a = a.reshape(na).contiguous()
                self.args_stride = 0
            elif a.numel() == self.B * na:
                a = a.reshape(self.B, na).contiguous()
                self.args_stride = na
            else:
                raise ValueError(f"args must have shape [{na}] or [batch, {na}]")
            self.args = a
        else:
            self.args = None
            self.args_stride = 0
        _, diff_term, _ = _split_terms(terms)
        self.diffusion = None if diff_term is None else diff_term.vector_field
        parts = []
        if hasattr(drift, "flat_params"):
            parts.append(drift.flat_params(self.dtype, dev))
        if self.diffusion is not None and hasattr(self.diffusion, "flat_params"):
            parts.append(self.diffusion.flat_params(self.dtype, dev))
        self.params = torch.cat(parts).contiguous() if parts else None
        if self.params is not None and self.params.numel() != self.problem.param_count():
            raise ValueError(f"expected {self.problem.param_count()} field parameters, "
                             f"got {self.params.numel()}")
        self.n_save = self.problem.n_save
        self.device = dev

    def _outputs(self, io):
        """ys, ts, result, stats on the device, None for those `io` gives."""
        dev, B = self.device, self.B
        shapes = (("ys", (B, self.n_save, self.dim), self.dtype),
                  ("ts", (B, self.n_save), torch.float64), ("result", (B,), torch.int32),
                  ("stats", (B, 3), torch.int32))
        return [None if io and name in io else torch.empty(shape, dtype=dt, device=dev)
                for name, shape, dt in shapes]

    def run_forward(self, stream=None, y0=None, params=None, keep_workspace=False, io=None):
        """Forward solve through gbdx_solve_fwd.  `io` maps any of t0, t1, dt0,
        y0, args (inputs) and ys, ts, result, stats (outputs, then returned as
        None) to addresses used instead of this object's buffers: the
        zero-copy host I/O of GraphedSolve."""
        dev = self.device
        B = self.B
        y0 = self.y0 if y0 is None else y0
        params = self.params if params is None else params
        ys, ts_out, res, stats = self._outputs(io)
        ws_bytes = self.problem.workspace_size(B)
        ws = torch.empty((max(ws_bytes, 1),), dtype=torch.uint8, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev).cuda_stream
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        # io[name] when given (a device address of mapped page-locked host
        # memory), else the buffer's own address
        a = lambda name, t: io[name] if io and name in io else p(t)  # noqa: E731
        rc = self.problem.lib.gbdx_solve_fwd(
            self.problem.handle, B, a("t0", self.t0), a("t1", self.t1), a("dt0", self.dt0),
            self.tstride, a("y0", y0), a("args", self.args), self.args_stride, p(params),
            p(self.save_ts), a("ys", ys), a("ts", ts_out), a("result", res), a("stats", stats),
            p(ws), ws_bytes, stream)
        _lib.check(rc, "gbdx_solve_fwd")
        if keep_workspace:
            return ys, ts_out, res, stats, ws
        return ys, ts_out, res, stats

    def run_forward_ex(self, stream=None, state_in=None, want_state=False, io=None):
        """Forward solve through gbdx_solve_fwd_ex: the saved outputs plus the
        dense buffers (SaveAt(dense=True)) and the index of the event condition
        that ended each trajectory (-1 for none).  state_in ([B, GBDX_STATE_HEAD
        + dim] f64, include/gbdx.h) resumes a solve; want_state leaves the
        final record in self.state_record.  `io` as in run_forward, plus
        event_index."""
        dev = self.device
        B, D, n_save = self.B, self.dim, self.n_save
        ys, ts_out, res, stats = self._outputs(io)
        p = lambda t: None if t is None or t.numel() == 0 else t.data_ptr()  # noqa: E731
        a = lambda name, t: io[name] if io and name in io else p(t)  # noqa: E731
        ex = _lib.FwdExtras()
        interp = ev = None
        if self.fields["save_dense"]:
            L = int(self.fields["max_steps"]) + 1
            stages = {0: 1, 1: 2, 2: 7, 3: 7, 4: 14, 5: 2, 6: 2, 7: 1}[self.fields["solver"]]
            dense_ts = torch.empty((B, L), dtype=torch.float64, device=dev)
            dense_info = torch.empty((B, L - 1, (2 + stages) * D), dtype=self.dtype, device=dev)
            dense_n = torch.empty((B,), dtype=torch.int32, device=dev)
            ex.dense_ts, ex.dense_info, ex.dense_n = p(dense_ts), p(dense_info), p(dense_n)
            interp = DenseInterpolation(self, dense_ts, dense_info, dense_n)
        if self.fields["n_event"]:
            if io and "event_index" in io:
                ex.event_index = io["event_index"]
            else:
                ev = torch.empty((B,), dtype=torch.int32, device=dev)
                ex.event_index = p(ev)
        self.state_record = None
        if state_in is not None:
            state_in = state_in.to(device=dev, dtype=torch.float64).contiguous()
            ex.state_in = p(state_in)
        if want_state:
            self.state_record = torch.empty((B, STATE_HEAD + D), dtype=torch.float64,
                                            device=dev)
            ex.state_out = p(self.state_record)
        ws_bytes = self.problem.workspace_size(B)
        ws = torch.empty((max(ws_bytes, 1),), dtype=torch.uint8, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev).cuda_stream
        rc = self.problem.lib.gbdx_solve_fwd_ex(
            self.problem.handle, B, a("t0", self.t0), a("t1", self.t1), a("dt0", self.dt0),
            self.tstride, a("y0", self.y0), a("args", self.args), self.args_stride,
            p(self.params), p(self.save_ts), a("ys", ys), a("ts", ts_out), a("result", res),
            a("stats", stats), ctypes.byref(ex), p(ws), ws_bytes, stream)
        _lib.check(rc, "gbdx_solve_fwd_ex")
        return ys, ts_out, res, stats, interp, ev

    def run_backward(self, ws, grad_ys, y0, params, stream=None):
        """dL/dy0 and dL/dparams from the tape the forward left in `ws`."""
        dev = self.device
        grad_ys = grad_ys.to(device=dev, dtype=self.dtype).contiguous()
        grad_y0 = torch.empty((self.B, self.dim), dtype=self.dtype, device=dev)
        n_params = 0 if params is None else int(params.numel())
        grad_params = torch.empty((max(n_params, 1),), dtype=torch.float32, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev).cuda_stream
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        rc = self.problem.lib.gbdx_solve_bwd(
            self.problem.handle, self.B, p(self.t0), p(self.t1), p(self.dt0), self.tstride,
            p(y0), p(self.args), self.args_stride, p(params), p(self.save_ts), p(grad_ys),
            p(grad_y0), p(grad_params), p(ws), ws.numel(), stream)
        _lib.check(rc, "gbdx_solve_bwd")
        return grad_y0, grad_params[:n_params]


    def run_backward_args(self, ws, grad_ys, y0, args, stream=None):
        """Analytic fields: dL/dy0 and dL/dargs from the tape the forward left
        in `ws` (dL/dargs [B, n_args] for per-trajectory args, else [n_args])."""
        dev = self.device
        grad_ys = grad_ys.to(device=dev, dtype=self.dtype).contiguous()
        grad_y0 = torch.empty((self.B, self.dim), dtype=self.dtype, device=dev)
        na = self.drift.n_args
        grad_args = torch.empty((self.B, na) if self.args_stride else (na,),
                                dtype=self.dtype, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev).cuda_stream
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        rc = self.problem.lib.gbdx_solve_bwd(
            self.problem.handle, self.B, p(self.t0), p(self.t1), p(self.dt0), self.tstride,
            p(y0), p(args), self.args_stride, None, p(self.save_ts), p(grad_ys),
            p(grad_y0), p(grad_args), p(ws), ws.numel(), stream)
        _lib.check(rc, "gbdx_solve_bwd")
        return grad_y0, grad_args

    def run_backsolve_args(self, ts_out, ys, grad_ys, args, stream=None):
        """Analytic fields, BacksolveAdjoint: dL/dy0, dL/dargs and the
        backward's RESULTS codes and step counts."""
        dev = self.device
        prob = self.bwd_problem
        grad_ys = grad_ys.to(device=dev, dtype=self.dtype).contiguous()
        grad_y0 = torch.empty((self.B, self.dim), dtype=self.dtype, device=dev)
        na = self.drift.n_args
        grad_args = torch.empty((self.B, na) if self.args_stride else (na,),
                                dtype=self.dtype, device=dev)
        res = torch.empty((self.B,), dtype=torch.int32, device=dev)
        stats = torch.empty((self.B, 3), dtype=torch.int32, device=dev)
        ws_bytes = prob.workspace_size(self.B)
        ws = torch.empty((max(ws_bytes, 1),), dtype=torch.uint8, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev).cuda_stream
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        rc = prob.lib.gbdx_backsolve_bwd_ex(
            prob.handle, self.B, p(self.t0), p(self.t1), p(self.bwd_dt0), self.tstride,
            p(ts_out.contiguous()), p(ys.contiguous()), p(grad_ys), p(args), self.args_stride,
            None, p(grad_y0), p(grad_args), p(res), p(stats), p(ws), ws_bytes, stream)
        _lib.check(rc, "gbdx_backsolve_bwd_ex")
        return grad_y0, grad_args, res, stats

    def run_backsolve(self, ts_out, ys, grad_ys, params, stream=None):
        """BacksolveAdjoint backward from the forward's saved (ts, ys):
        dL/dy0, dL/dparams and the backward's RESULTS codes and step counts."""
        dev = self.device
        prob = self.bwd_problem
        grad_ys = grad_ys.to(device=dev, dtype=self.dtype).contiguous()
        grad_y0 = torch.empty((self.B, self.dim), dtype=self.dtype, device=dev)
        n_params = int(params.numel())
        grad_params = torch.empty((max(n_params, 1),), dtype=torch.float32, device=dev)
        res = torch.empty((self.B,), dtype=torch.int32, device=dev)
        stats = torch.empty((self.B, 3), dtype=torch.int32, device=dev)
        ws_bytes = prob.workspace_size(self.B)
        ws = torch.empty((max(ws_bytes, 1),), dtype=torch.uint8, device=dev)
        if stream is None:
            stream = torch.cuda.current_stream(dev).cuda_stream
        p = lambda t: None if t is None else t.data_ptr()  # noqa: E731
        rc = prob.lib.gbdx_backsolve_bwd(
            prob.handle, self.B, p(self.t0), p(self.t1), p(self.bwd_dt0), self.tstride,
            p(ts_out.contiguous()), p(ys.contiguous()), p(grad_ys), p(params), p(grad_y0),
            p(grad_params), p(res), p(stats), p(ws), ws_bytes, stream)
        _lib.check(rc, "gbdx_backsolve_bwd")
        return grad_y0, grad_params[:n_params], res, stats


class DenseInterpolation:
    """Batched diffrax.DenseInterpolation (diffrax/_global_interpolation.py:315-393)
    over a dense solve: ``ts`` [B, max_steps + 1] step times in the loop's
    direction-flipped time (+inf where unused), ``ts_size`` [B] entries used,
    ``infos`` [B, max_steps, (2 + stages) dim] per-step (y0, y1, k_0..k_{s-1}),
    ``direction`` [B].  Evaluation runs on the GPU (gbdx_dense_evaluate)."""

    def __init__(self, low: "Lowered", ts, infos, ts_size):
        self._low = low
        self.ts, self.infos, self.ts_size = ts, infos, ts_size
        self.direction = torch.where(low.t0 < low.t1, 1, -1).to(torch.int32)
        self.t0_if_trivial = low.t0 * self.direction
        self.y0_if_trivial = low.y0

    def _query(self, t):
        low = self._low
        q = torch.as_tensor(t, dtype=torch.float64).to(low.device)
        if q.dim() == 0:
            return q.reshape(1).contiguous(), 1, 0, True
        if q.dim() == 1:
            return q.contiguous(), int(q.numel()), 0, False
        if q.dim() == 2 and q.shape[0] == low.B:
            return q.contiguous(), int(q.shape[1]), int(q.shape[1]), False
        raise ValueError("query times must be a scalar, [Q] or [batch, Q]")

    def _run(self, t, left, order):
        low = self._low
        q, Q, qstride, scalar = self._query(t)
        out = torch.empty((low.B, Q, low.dim), dtype=low.dtype, device=low.device)
        stream = torch.cuda.current_stream(low.device).cuda_stream
        rc = low.problem.lib.gbdx_dense_evaluate(
            low.problem.handle, low.B, low.t0.data_ptr(), low.t1.data_ptr(), low.tstride,
            low.y0.data_ptr(), self.ts.data_ptr(), self.infos.data_ptr(),
            self.ts_size.data_ptr(), Q, q.data_ptr(), qstride, int(bool(left)), order,
            out.data_ptr(), stream)
        _lib.check(rc, "gbdx_dense_evaluate")
        return out[:, 0] if scalar else out

    def evaluate(self, t0, t1=None, left: bool = True):
        if t1 is not None:
            return self.evaluate(t1, left=left) - self.evaluate(t0, left=left)
        return self._run(t0, left, 0)

    def derivative(self, t, left: bool = True):
        return self._run(t, left, 1)

    @property
    def t0(self):
        first = torch.where(self.ts_size == 1, self.t0_if_trivial, self.ts[:, 0])
        return first * self.direction

    @property
    def t1(self):
        last = self.ts.gather(1, (self.ts_size.long() - 1).clamp(min=0)[:, None])[:, 0]
        return torch.where(self.ts_size == 1, self.t0_if_trivial, last) * self.direction


# gbdx_fwd_extras' resume record: GBDX_STATE_HEAD doubles, then f0 (include/gbdx.h)
STATE_HEAD = 7
_FSAL_SOLVERS = (2, 3, 4)  # Dopri5, Tsit5, Dopri8


def _state_record(low: "Lowered", solver_state, controller_state, made_jump):
    """The [B, STATE_HEAD + dim] resume record from diffeqsolve's
    solver_state / controller_state / made_jump (_integrate.py:1252-1271,
    1309), in the layouts Solution documents."""
    f = low.fields
    if f["n_step_ts"] or f["n_jump_ts"] or (f["field"] == 3 and f["kernel"] in (1, 3)):
        raise NotImplementedError("resuming is supported without a ClipStepSizeController, "
                                  "on the trajectory kernels and the fused MLP kernel")
    B, D, dev = low.B, low.dim, low.device
    rec = torch.zeros((B, STATE_HEAD + D), dtype=torch.float64, device=dev)
    rec[:, 5] = 1.0

    def col(v):
        return torch.as_tensor(v).to(device=dev, dtype=torch.float64).reshape(-1).expand(B)

    if controller_state is not None:
        cs = tuple(controller_state)
        want = 3 if f["controller"] == 1 else 4
        if len(cs) != want:
            raise ValueError(f"controller_state must hold {want} entries for this controller")
        for k, v in enumerate(cs):
            rec[:, k] = col(v)
        rec[:, 4] = 1.0
    if solver_state is not None:
        if f["solver"] not in _FSAL_SOLVERS:
            raise ValueError("this solver has no solver state (None)")
        first_step, f0 = solver_state
        rec[:, 5] = col(first_step)
        rec[:, STATE_HEAD:] = torch.as_tensor(f0).to(device=dev, dtype=torch.float64
                                                     ).reshape(-1, D).expand(B, D)
    if made_jump is not None:
        rec[:, 6] = col(made_jump)
    return rec


def _split_state(low: "Lowered", rec: torch.Tensor, saveat: SaveAt, sol: "Solution"):
    """Solution.solver_state / controller_state / made_jump from the final
    record (_integrate.py:1489-1500)."""
    f = low.fields
    if saveat.controller_state:
        if f["controller"] == 1:
            sol.controller_state = (rec[:, 0], rec[:, 1], rec[:, 2] != 0)
        else:
            sol.controller_state = (rec[:, 0].to(torch.int32), rec[:, 1].to(torch.int32),
                                    rec[:, 2], rec[:, 3])
    if saveat.solver_state and f["solver"] in _FSAL_SOLVERS:
        sol.solver_state = (rec[:, 5] != 0, rec[:, STATE_HEAD:].to(low.dtype))
    if saveat.made_jump:
        sol.made_jump = rec[:, 6] != 0


def _raise_on_failure(result: torch.Tensor):
    if _capturing():
        return
    # successful and event_occurred are both fine (is_okay, _solution.py:52-54)
    bad = (result != 0) & (result != int(RESULTS.event_occurred))
    if bool(bad.any()):
        code = int(result[bad][0].item())
        n = int(bad.sum().item())
        raise RuntimeError(f"{RESULT_MESSAGES.get(RESULTS(code), 'failed')} "
                           f"({n} of {result.numel()} trajectories failed)")


def diffeqsolve(terms, solver, t0, t1, dt0, y0, args=None, *,
                saveat: SaveAt = SaveAt(t1=True),
                stepsize_controller=ConstantStepSize(),
                adjoint=RecursiveCheckpointAdjoint(), event=None,
                max_steps: Optional[int] = 4096, throw: bool = True,
                progress_meter: Any = None, solver_state=None, controller_state=None,
                made_jump=None, kernel: str = "auto", block_threads: int = 0,
                ctas_per_sm: int = 0, schedule: str = "auto",
                autotune: bool = False) -> Solution:
    """Batched diffrax.diffeqsolve on the GPU (diffrax/_integrate.py:888-1543).

    Extra keyword arguments select the GB300 execution policy: ``kernel`` is
    "fused" (persistent work-stealing integrator, the default), "plain" (one
    trajectory per thread) or "tc" (MLP-field forward on tcgen05 tensor cores); ``block_threads`` / ``ctas_per_sm`` override the
    autotuned launch shape of the fused kernel; ``schedule`` ("auto",
    "index", "longest_first") sets the order in which the fused kernel takes
    trajectories (results do not depend on it); ``autotune=True`` times a few
    launch shapes on this problem and batch the first time it is seen and
    keeps the fastest (diffrax_gb300._tune).

    Inputs may live on the host: those in page-locked memory are copied to the
    device asynchronously, so they must not be modified until the solution's
    tensors have been read.
    """
    if getattr(saveat, "subs", None) is not None:
        # one solve per SubSaveAt (the solves take the same steps); the first
        # also carries the dense output and the states
        leaves = _tree_leaves(saveat.subs)
        sols = []
        for k, sub in enumerate(leaves):
            first = k == 0
            sa = SaveAt(t0=sub.t0, t1=sub.t1, ts=sub.ts, steps=sub.steps, fn=sub.fn,
                        dense=saveat.dense and first,
                        solver_state=saveat.solver_state and first,
                        controller_state=saveat.controller_state and first,
                        made_jump=saveat.made_jump and first)
            sols.append(diffeqsolve(
                terms, solver, t0, t1, dt0, y0, args, saveat=sa,
                stepsize_controller=stepsize_controller, adjoint=adjoint, event=event,
                max_steps=max_steps, throw=throw, progress_meter=progress_meter,
                solver_state=solver_state, controller_state=controller_state,
                made_jump=made_jump, kernel=kernel, block_threads=block_threads,
                ctas_per_sm=ctas_per_sm, schedule=schedule, autotune=autotune))
        sol = sols[0]
        sol.ys = _tree_unflatten(saveat.subs, [x.ys for x in sols])
        sol.ts = _tree_unflatten(saveat.subs, [x.ts for x in sols])
        return sol
    resume = solver_state is not None or controller_state is not None or made_jump is not None
    keep_state = saveat.solver_state or saveat.controller_state or saveat.made_jump
    from ._autograd import needs_grad, solve_with_grad
    want_grad = needs_grad(terms, y0, args)
    if want_grad and (saveat.dense or saveat.steps or event is not None or resume
                      or keep_state):
        raise NotImplementedError("gradients through SaveAt(steps=...), SaveAt(dense=True), "
                                  "events or solver/controller states are not supported")
    if (autotune and not want_grad and block_threads == 0 and ctas_per_sm == 0
            and kernel in ("auto", "fused")):
        from ._tune import autotune_launch

        def factory(kern, bt, cps):
            return Lowered(terms, solver, t0, t1, dt0, y0, args, saveat, stepsize_controller,
                           adjoint, max_steps, kern, bt, cps, schedule, event=event)
        base = factory(kernel, 0, 0)
        kernel, block_threads, ctas_per_sm = autotune_launch(factory, base.B, base.fields)
    low = Lowered(terms, solver, t0, t1, dt0, y0, args, saveat, stepsize_controller,
                  adjoint, max_steps, kernel, block_threads, ctas_per_sm, schedule,
                  want_grad=want_grad, event=event, throw=throw)
    interp = ev = None
    if saveat.dense or event is not None or resume or keep_state:
        rec = None
        if resume:
            rec = _state_record(low, solver_state, controller_state, made_jump)
        elif keep_state:
            _state_record(low, None, None, None)  # the same support check
        ys, ts_out, res, stats, interp, ev = low.run_forward_ex(state_in=rec,
                                                                want_state=keep_state)
    elif want_grad:
        ys, ts_out, res, stats = solve_with_grad(low, y0, args)
    else:
        ys, ts_out, res, stats = low.run_forward()
    if low.n_save == 0 or saveat.state_only:
        # SaveAt(dense=True) or the states alone save no ys (_integrate.py:1527-1539)
        ys = ts_out = None
    elif getattr(saveat, "fn", None) is not None:
        ys = saveat.fn(ts_out, ys, args)
    sol = Solution(t0=t0, t1=t1, ts=ts_out, ys=ys,
                   stats=dict(num_steps=stats[:, 0], num_accepted_steps=stats[:, 1],
                              num_rejected_steps=stats[:, 2], max_steps=max_steps),
                   result=res, interpolation=interp)
    if event is not None:
        masks = [ev == i for i in range(len(event._conds))]
        sol.event_mask = masks[0] if event._single else masks
    if keep_state:
        _split_state(low, low.state_record, saveat, sol)
    # the lowered solve; after a backward pass under BacksolveAdjoint it holds
    # the backward's RESULTS codes and step counts (bwd_result, bwd_stats)
    sol.lowered = low
    if throw:
        _raise_on_failure(res)
    return sol
