"""Diffrax-compatible objects: fields, terms, solvers, controllers, SaveAt,
adjoints, RESULTS and Solution.

Names, defaults and argument meaning follow Diffrax v0.7.2; each class cites
the reference definition it mirrors.  These objects carry no computation --
``diffeqsolve`` lowers them to a ``gbdx_problem_desc`` and calls libgbdx.so.
"""
from __future__ import annotations

import dataclasses
import enum
from typing import Any, Optional, Sequence

import numpy as np

# ---------------------------------------------------------------------------
# Registered vector fields.  A field is a vector_field(t, y, args) that the
# library knows how to evaluate on the GPU.
# ---------------------------------------------------------------------------


class AbstractField:
    field_id: int = -1
    n_args: int = 0

    def dim_for(self, dim: int) -> int:
        return dim


class LotkaVolterra(AbstractField):
    """x' = a x - b x y,  y' = -c y + d x y.  args = (a, b, c, d), shared or per
    trajectory ([4] or [B, 4])."""
    field_id = 0
    n_args = 4


class VanDerPol(AbstractField):
    """x' = y,  y' = mu (1 - x^2) y - x.  args = mu ([1], [B] or [B, 1])."""
    field_id = 1
    n_args = 1


class OrnsteinUhlenbeck(AbstractField):
    """Drift theta (mu - y) and, inside a ControlTerm, constant diagonal
    diffusion sigma.  args = (theta, mu, sigma)."""
    field_id = 2
    n_args = 3


def _flat(tensors, dtype, device):
    import torch
    return torch.cat([t.detach().reshape(-1) if not t.requires_grad else t.reshape(-1)
                      for t in tensors]).to(device=device, dtype=torch.float32).contiguous()


class MLPField(AbstractField):
    """An eqx.nn.MLP vector field f(t, y) = W2 tanh(W1 tanh(W0 y + b0) + b1) + b2
    (tanh on the hidden layers, identity output; equinox/nn/_mlp.py semantics)
    given its weights as tensors.  weights[l] is [out, in] as in a Linear layer.

    precision "bf16" runs the products on the tensor cores with FP32
    accumulation: the weights are held as BF16 values and every activation
    operand is split into three BF16 pieces (24 significant bits, three
    products per tile), so the field equals an FP32 evaluation of the
    BF16-rounded weights and stays smooth under adaptive stepping.  "fp32"
    runs the products in FP32 on the CUDA cores with the FP32 weights (parity
    mode)."""
    field_id = 3
    n_args = 0

    def __init__(self, weights, biases, precision: str = "bf16"):
        if len(weights) != len(biases):
            raise ValueError("one bias per weight")
        if precision not in ("bf16", "fp32"):
            raise ValueError("precision must be 'bf16' or 'fp32'")
        self.weights = list(weights)
        self.biases = list(biases)
        self.precision = precision

    @property
    def widths(self):
        return [int(self.weights[0].shape[1])] + [int(w.shape[0]) for w in self.weights]

    def lower_fields(self, dim):
        w = self.widths
        if w[0] != dim or w[-1] != dim:
            raise ValueError(f"MLP maps {w[0]} -> {w[-1]} but the state has dimension {dim}")
        return dict(mlp_depth=len(self.weights), mlp_widths=tuple(w),
                    mlp_precision=0 if self.precision == "bf16" else 1)

    def tensors(self):
        out = []
        for W, b in zip(self.weights, self.biases):
            out += [W, b]
        return out

    def flat_params(self, dtype, device):
        return _flat(self.tensors(), dtype, device)

    @property
    def requires_grad(self):
        return any(getattr(t, "requires_grad", False) for t in self.tensors())


class TanhDiagonalDiffusion:
    """Diagonal diffusion g(y) = scale * tanh(W y + b) of a ControlTerm, with W
    [dim, dim]: dY_i = f_i dt + g_i(Y) dW_i."""
    diffusion_id = 2

    def __init__(self, weight, bias, scale: float = 0.1):
        if float(scale) != 0.1:
            raise NotImplementedError("the tanh diffusion is compiled with scale 0.1")
        self.weight, self.bias, self.scale = weight, bias, float(scale)

    def tensors(self):
        return [self.weight, self.bias]

    def flat_params(self, dtype, device):
        return _flat(self.tensors(), dtype, device)

    @property
    def requires_grad(self):
        return any(getattr(t, "requires_grad", False) for t in self.tensors())


# ---------------------------------------------------------------------------
# Terms (diffrax/_term.py).
# ---------------------------------------------------------------------------


class AbstractTerm:
    pass


class ODETerm(AbstractTerm):
    """f(t, y, args) dt (diffrax/_term.py:174-226)."""

    def __init__(self, vector_field: AbstractField):
        if not isinstance(vector_field, AbstractField):
            raise TypeError("ODETerm needs a registered vector field "
                            "(LotkaVolterra, VanDerPol, OrnsteinUhlenbeck, MLPField)")
        self.vector_field = vector_field


class ControlTerm(AbstractTerm):
    """g(t, y, args) dW with a diagonal g (diffrax/_term.py:271-555)."""

    def __init__(self, vector_field: Any, control: Any):
        self.vector_field = vector_field
        self.control = control


class MultiTerm(AbstractTerm):
    """Sum of terms (diffrax/_term.py:666-731)."""

    def __init__(self, *terms: AbstractTerm):
        self.terms = tuple(terms)


class AbstractBrownianIncrement:
    """The quantities a Brownian path returns over an interval
    (diffrax/_custom_types.py)."""


class BrownianIncrement(AbstractBrownianIncrement):
    """W only."""


class SpaceTimeLevyArea(AbstractBrownianIncrement):
    """W and the space-time Levy area H = (1/h) int (W_{s,r} - (r-s)/h W_{s,t}) dr."""


class VirtualBrownianTree:
    """Brownian motion on [t0, t1] discretised to `tol`, evaluated by binary
    bridge descent (diffrax/_brownian/tree.py:177-354): with
    ``levy_area=BrownianIncrement`` the midpoint rule of W alone
    (tree.py:752-768), with ``levy_area=SpaceTimeLevyArea`` the joint rule of
    W and the space-time Levy area (tree.py:727-750, 562-603), which ShARK
    needs and Euler / Heun also accept (they use its W).

    `key` is an integer seed of this library's counter-based generator
    (Philox4x32-10); trajectory b of a batch uses its own independent path.
    """

    def __init__(self, t0: float, t1: float, tol: float, shape: Sequence[int] | int,
                 key: int = 0, levy_area: type = BrownianIncrement):
        if not t0 < t1:
            raise ValueError("t0 must be strictly less than t1")
        if levy_area not in (BrownianIncrement, SpaceTimeLevyArea):
            raise ValueError(f"levy_area must be BrownianIncrement or SpaceTimeLevyArea, "
                             f"got {levy_area!r}")
        self.t0, self.t1, self.tol = float(t0), float(t1), float(tol)
        self.shape = (shape,) if isinstance(shape, int) else tuple(shape)
        self.key = int(key)
        self.levy_area = levy_area


# ---------------------------------------------------------------------------
# Solvers (diffrax/_solver/*.py).
# ---------------------------------------------------------------------------


class AbstractSolver:
    solver_id: int = -1
    _order: int = 0
    _strong_order: Optional[float] = None

    def order(self, terms=None) -> int:
        return self._order

    def strong_order(self, terms=None) -> Optional[float]:
        return self._strong_order

    def __eq__(self, other):
        return type(self) is type(other)

    def __hash__(self):
        return hash(type(self))

    def __repr__(self):
        return f"{type(self).__name__}()"


class Euler(AbstractSolver):
    """diffrax/_solver/euler.py:17-73."""
    solver_id, _order, _strong_order = 0, 1, 0.5


class Heun(AbstractSolver):
    """diffrax/_solver/heun.py:20-45."""
    solver_id, _order, _strong_order = 1, 2, 0.5


class Dopri5(AbstractSolver):
    """diffrax/_solver/dopri5.py:53-100."""
    solver_id, _order = 2, 5


class Tsit5(AbstractSolver):
    """diffrax/_solver/tsit5.py:159-190."""
    solver_id, _order = 3, 5


class Dopri8(AbstractSolver):
    """diffrax/_solver/dopri8.py:306-353 (analytic fields)."""
    solver_id, _order = 4, 8


class ShARK(AbstractSolver):
    """Shifted Additive-noise Runge-Kutta (diffrax/_solver/shark.py:38-80):
    two drift evaluations per step, strong order 1.5 for additive noise;
    needs a VirtualBrownianTree with levy_area=SpaceTimeLevyArea."""
    solver_id, _order, _strong_order = 5, 2, 1.5
    minimal_levy_area = SpaceTimeLevyArea


class SRA1(AbstractSolver):
    """Roessler's SRA1 for additive noise (diffrax/_solver/sra1.py:37-68):
    two drift evaluations per step, strong order 1.5; needs a
    VirtualBrownianTree with levy_area=SpaceTimeLevyArea."""
    solver_id, _order, _strong_order = 6, 2, 1.5
    minimal_levy_area = SpaceTimeLevyArea


class SEA(AbstractSolver):
    """Shifted Euler for additive noise (diffrax/_solver/sea.py:37-69): one
    drift evaluation per step, strong order 1, no error estimate (constant
    steps); needs a VirtualBrownianTree with levy_area=SpaceTimeLevyArea."""
    solver_id, _order, _strong_order = 7, 1, 1.0
    minimal_levy_area = SpaceTimeLevyArea


# ---------------------------------------------------------------------------
# Step size controllers.
# ---------------------------------------------------------------------------


class AbstractStepSizeController:
    pass


@dataclasses.dataclass(frozen=True)
class ConstantStepSize(AbstractStepSizeController):
    """diffrax/_step_size_controller/constant.py:20-104."""


def rms_norm(x):  # marker for PIDController(norm=...), optx.rms_norm
    raise NotImplementedError("rms_norm is evaluated inside the kernels")


def adjoint_rms_seminorm(x):  # marker, diffrax/_misc.py:85-116
    raise NotImplementedError("adjoint_rms_seminorm is evaluated inside the kernels")


class _MetaPID(type):
    """PIDController(..., step_ts=s, jump_ts=j) is
    ClipStepSizeController(PIDController(...), s, j) (pid.py:88-97)."""

    def __call__(cls, *args, **kwargs):
        step_ts = kwargs.pop("step_ts", None)
        jump_ts = kwargs.pop("jump_ts", None)
        if step_ts is not None or jump_ts is not None:
            return ClipStepSizeController(super().__call__(*args, **kwargs), step_ts=step_ts,
                                          jump_ts=jump_ts)
        return super().__call__(*args, **kwargs)


@dataclasses.dataclass(frozen=True)
class PIDController(AbstractStepSizeController, metaclass=_MetaPID):
    """diffrax/_step_size_controller/pid.py:109-580 (same fields and defaults;
    ``step_ts`` / ``jump_ts`` build the ClipStepSizeController)."""
    rtol: float
    atol: float
    pcoeff: float = 0.0
    icoeff: float = 1.0
    dcoeff: float = 0.0
    dtmin: Optional[float] = None
    dtmax: Optional[float] = None
    force_dtmin: bool = True
    factormin: float = 0.2
    factormax: float = 10.0
    safety: float = 0.9
    error_order: Optional[float] = None
    norm: Any = rms_norm


class ClipStepSizeController(AbstractStepSizeController):
    """diffrax/_step_size_controller/clip.py:120-427: steps exactly to
    ``step_ts`` and to just before / just after ``jump_ts`` (where FSAL solvers
    evaluate the vector field afresh).  Wraps a PIDController;
    ``store_rejected_steps`` (revisiting rejected steps of SDE solves) is not
    available."""

    def __init__(self, controller, step_ts=None, jump_ts=None, store_rejected_steps=None):
        if not isinstance(controller, PIDController):
            if isinstance(controller, ClipStepSizeController):
                raise NotImplementedError("nested ClipStepSizeController wrappers are not "
                                          "supported; pass all step_ts/jump_ts to one")
            raise ValueError("Can only apply `ClipStepSizeController` to adaptive step size "
                             f"controllers, but got {controller}.")
        if store_rejected_steps is not None:
            if store_rejected_steps <= 0:
                raise ValueError("`store_rejected_steps must either be `None` or a "
                                 "non-negative integer.")
            raise NotImplementedError("store_rejected_steps is not supported")
        self.controller = controller
        sort = lambda x: None if x is None else np.sort(  # noqa: E731
            np.asarray(x, dtype=np.float64).reshape(-1))
        self.step_ts = sort(step_ts)
        self.jump_ts = sort(jump_ts)
        self.store_rejected_steps = None

    @property
    def rtol(self):
        return self.controller.rtol

    @property
    def atol(self):
        return self.controller.atol

    @property
    def norm(self):
        return self.controller.norm


# ---------------------------------------------------------------------------
# Events (diffrax/_event.py).  The kernels evaluate registered conditions; a
# condition sees the loop's time (t * sign(t1 - t0), as the reference's
# cond_fn does) and the state.
# ---------------------------------------------------------------------------


class LinearCondition:
    """A registered event condition: ``sum_n y_coeffs[n] y[n] + t_coeff t +
    offset`` (at most 4 state coefficients).  Real-valued: the event fires when
    it changes sign (``Event.direction`` picks up- or down-crossings).  With
    ``boolean=True`` it is the condition ``value > 0`` and fires when true.
    Examples: ``LinearCondition([1, 0])`` is the reference's ``cond_fn = y[0]``;
    ``LinearCondition([], t_coeff=1, offset=-10, boolean=True)`` is
    ``t > 10``."""

    def __init__(self, y_coeffs=(), t_coeff: float = 0.0, offset: float = 0.0,
                 boolean: bool = False):
        w = [float(x) for x in np.asarray(y_coeffs, dtype=np.float64).reshape(-1)]
        if len(w) > 4:
            raise ValueError("a LinearCondition takes at most 4 state coefficients")
        self.y_coeffs, self.t_coeff, self.offset = w, float(t_coeff), float(offset)
        self.boolean = bool(boolean)


class SteadyStateCondition:
    """steady_state_event (diffrax/_event.py:120-175): fires once
    ``rms(f(t, y)) < atol + rtol * rms(y)``; unset tolerances default to the
    adaptive step size controller's."""

    def __init__(self, rtol=None, atol=None, norm=None):
        if norm is not None and norm is not rms_norm:
            raise NotImplementedError("steady_state_event takes the rms_norm only")
        self.rtol, self.atol = rtol, atol


def steady_state_event(rtol=None, atol=None, norm=None):
    """diffrax/_event.py:120-175."""
    return SteadyStateCondition(rtol, atol, norm)


class Newton:
    """The root finder of an event (optimistix.Newton(rtol, atol, norm)): Newton's
    method with Cauchy termination on the last step's interpolant."""

    def __init__(self, rtol: float, atol: float, norm=None):
        self.rtol, self.atol = float(rtol), float(atol)


class Event:
    """diffrax/_event.py:13-51.  ``cond_fn`` is one registered condition or a
    list of them (at most 4); ``direction`` is None / True / False, or a list of
    them (True: up-crossings only, False: down-crossings only)."""

    def __init__(self, cond_fn, root_finder=None, direction=None):
        single = not isinstance(cond_fn, (list, tuple))
        conds = [cond_fn] if single else list(cond_fn)
        if direction in (None, False, True):
            dirs = [direction] * len(conds)
        else:
            dirs = list(direction)
            if single or len(dirs) != len(conds):
                raise ValueError("Missmatch in the structure of `cond_fn` and `direction`.")
        if any(x not in (None, False, True) for x in dirs):
            raise ValueError("`direction` must be a `None`, `bool`, or a PyTree of "
                             "`None | bool`s with the same structure as `cond_fn`.")
        for c in conds:
            if not isinstance(c, (LinearCondition, SteadyStateCondition)):
                raise NotImplementedError("event conditions must be registered conditions "
                                          "(LinearCondition, steady_state_event)")
        if not 1 <= len(conds) <= 4:
            raise ValueError("an Event takes 1 to 4 conditions")
        if root_finder is not None and not isinstance(root_finder, Newton):
            raise NotImplementedError("the event root finder must be Newton(rtol, atol)")
        self.cond_fn, self.root_finder, self.direction = cond_fn, root_finder, direction
        self._conds, self._dirs, self._single = conds, dirs, single


# ---------------------------------------------------------------------------
# SaveAt (diffrax/_saveat.py:14-105).
# ---------------------------------------------------------------------------


# ---------------------------------------------------------------------------
# Progress meters (diffrax/_progress_meter.py): accepted for the reference's
# signature; a solve is one launch with no host loop to report from.
# ---------------------------------------------------------------------------


class AbstractProgressMeter:
    pass


class NoProgressMeter(AbstractProgressMeter):
    pass


class TextProgressMeter(AbstractProgressMeter):
    def __init__(self, minimum_increase: float = 0.02):
        self.minimum_increase = minimum_increase


class TqdmProgressMeter(AbstractProgressMeter):
    def __init__(self, refresh_steps: int = 20):
        self.refresh_steps = refresh_steps


class SubSaveAt:
    """diffrax/_saveat.py:14-57: one set of saves (t0, ts, every n-th step,
    t1) with its own map fn(t, y, args) (called on the batched saves)."""

    def __init__(self, *, t0: bool = False, t1: bool = False, ts=None, steps=False, fn=None):
        if isinstance(steps, bool):
            steps = 1 if steps else 0
        steps = int(steps)
        if steps < 0:
            raise ValueError("SaveAt(steps=n) needs n >= 0")
        if not (t0 or t1 or ts is not None or steps):
            raise ValueError("Empty saveat -- nothing will be saved.")
        self.t0, self.t1, self.ts, self.steps, self.fn = bool(t0), bool(t1), ts, steps, fn


def _tree_leaves(tree):
    """The SubSaveAt leaves of a list / tuple / dict tree, in order."""
    if isinstance(tree, SubSaveAt):
        return [tree]
    if isinstance(tree, dict):
        return [x for k in sorted(tree) for x in _tree_leaves(tree[k])]
    if isinstance(tree, (list, tuple)):
        return [x for v in tree for x in _tree_leaves(v)]
    raise TypeError("SaveAt(subs=...) takes SubSaveAt leaves in lists, tuples and dicts")


def _tree_unflatten(tree, leaves):
    """`tree` with its SubSaveAt leaves replaced, in order, by `leaves`."""
    it = iter(leaves)

    def go(t):
        if isinstance(t, SubSaveAt):
            return next(it)
        if isinstance(t, dict):
            out = {k: None for k in t}
            for k in sorted(t):
                out[k] = go(t[k])
            return out
        return type(t)(go(v) for v in t)
    return go(tree)


class SaveAt:
    """diffrax/_saveat.py:69-105.  ``steps`` is a bool or an int n (save every
    n-th accepted step); ``fn(t, y, args)`` maps the saved values (called on
    the batched saves); ``subs`` is a tree (lists, tuples, dicts) of
    SubSaveAt, whose solution ``ys`` / ``ts`` have the same tree (one solve
    per SubSaveAt: the solves take the same steps); ``dense=True`` records
    the solution's dense output (``Solution.evaluate`` / ``.derivative``);
    ``solver_state``, ``controller_state`` and ``made_jump`` keep the final
    states, which a later ``diffeqsolve`` resumes from."""

    def __init__(self, *, t0: bool = False, t1: bool = False, ts=None, steps=False,
                 fn=None, subs=None, dense: bool = False, solver_state: bool = False,
                 controller_state: bool = False, made_jump: bool = False):
        if subs is not None:
            if t0 or t1 or (ts is not None) or steps:
                raise ValueError("Cannot pass both `subs` and any of `t0`, `t1`, `ts`, "
                                 "`steps` to `SaveAt`.")
            _tree_leaves(subs)  # type check
        self.subs = subs
        # fn(t, y, args) is applied to every saved value (SubSaveAt.fn,
        # _saveat.py:20-43); it is called once on the whole batch of saves
        # (t [B, n_save], y [B, n_save, dim]) and must broadcast over those
        # leading dimensions, as a vmapped function would
        self.fn = fn
        self.solver_state, self.controller_state = bool(solver_state), bool(controller_state)
        self.made_jump = bool(made_jump)
        # SubSaveAt.__init__: steps=True means every step (_saveat.py:40-43)
        if isinstance(steps, bool):
            steps = 1 if steps else 0
        steps = int(steps)
        if steps < 0:
            raise ValueError("SaveAt(steps=n) needs n >= 0")
        # the states alone save no ys (subs = None, _saveat.py:91-93)
        self.state_only = subs is None and not (t0 or t1 or ts is not None or steps or dense)
        if self.state_only and not (solver_state or controller_state or made_jump):
            raise ValueError("Empty saveat -- nothing will be saved.")
        self.t0, self.t1, self.ts = bool(t0), bool(t1), ts
        self.steps, self.dense = steps, bool(dense)


# ---------------------------------------------------------------------------
# Adjoints (diffrax/_adjoint.py).
# ---------------------------------------------------------------------------


class AbstractAdjoint:
    pass


@dataclasses.dataclass(frozen=True)
class RecursiveCheckpointAdjoint(AbstractAdjoint):
    """diffrax/_adjoint.py:179-312.  `checkpoints` bounds the per-trajectory
    checkpoint slots; None means ceil(log2(max_steps)) slots as the reference."""
    checkpoints: Optional[int] = None


class BacksolveAdjoint(AbstractAdjoint):
    """diffrax/_adjoint.py:737-871.  kwargs override the backward solve."""

    _valid = {"dt0", "solver", "stepsize_controller", "adjoint", "max_steps", "throw"}

    def __init__(self, **kwargs):
        diff = set(kwargs) - self._valid
        if diff:
            raise ValueError("The following keyword argments are not valid for "
                             f"`BacksolveAdjoint`: {diff}")
        self.kwargs = kwargs


# ---------------------------------------------------------------------------
# RESULTS and Solution (diffrax/_solution.py).
# ---------------------------------------------------------------------------


class RESULTS(enum.IntEnum):
    successful = 0
    max_steps_reached = 1
    dt_min_reached = 2
    event_occurred = 3
    max_steps_rejected = 4
    internal_error = 5
    nonlinear_max_steps_reached = 6


RESULT_MESSAGES = {
    RESULTS.successful: "",
    RESULTS.max_steps_reached: "The maximum number of solver steps was reached. Try "
                               "increasing `max_steps`.",
    RESULTS.dt_min_reached: "The minimum step size was reached in the differential "
                            "equation solver.",
    RESULTS.event_occurred: "Terminating differential equation solve because an event "
                            "occurred.",
    RESULTS.max_steps_rejected: "Maximum number of rejected steps was reached.",
    RESULTS.internal_error: "An internal error occurred.",
    RESULTS.nonlinear_max_steps_reached: "The maximum number of steps was reached in the "
                                         "nonlinear solver.",
}


@dataclasses.dataclass
class Solution:
    """Batched diffrax.Solution: every per-trajectory field has a leading batch
    dimension (diffrax/_solution.py:82-201)."""
    t0: Any
    t1: Any
    ts: Any        # [B, n_save] float64
    ys: Any        # [B, n_save, dim]
    stats: dict    # num_steps / num_accepted_steps / num_rejected_steps: [B] int32
    result: Any    # [B] int32 RESULTS codes
    interpolation: Any = None  # DenseInterpolation under SaveAt(dense=True)
    event_mask: Any = None     # Event: [B] bool per condition (cond_fn's structure)
    # SaveAt(solver_state=, controller_state=, made_jump=): PID (prev_inv
    # [B], prev_prev_inv [B], at_dtmin [B] bool) or ConstantStepSize
    # (steps_completed [B], num_steps [B], t0 [B], t1_or_dt0 [B]); FSAL
    # solvers (first_step [B] bool, f0 [B, dim]), others None; made_jump [B]
    solver_state: Any = None
    controller_state: Any = None
    made_jump: Any = None

    def evaluate(self, t0, t1=None, left: bool = True):
        """y(t0) of every trajectory from the dense output, or y(t1) - y(t0)
        (diffrax/_solution.py:128-152).  t0 is a scalar ([B, dim] out), [Q]
        times shared by the batch or [B, Q] per trajectory ([B, Q, dim] out)."""
        if self.interpolation is None:
            raise ValueError("Dense solution has not been saved; pass SaveAt(dense=True).")
        return self.interpolation.evaluate(t0, t1, left)

    def derivative(self, t, left: bool = True):
        """dy/dt of the numerical solution (diffrax/_solution.py:154-201);
        shapes as evaluate."""
        if self.interpolation is None:
            raise ValueError("Dense solution has not been saved; pass SaveAt(dense=True).")
        return self.interpolation.derivative(t, left)
