"""torch.autograd bridge: the forward and adjoint kernels behind one
autograd.Function per adjoint kind (diffrax/_adjoint.py)."""
from __future__ import annotations

import torch

from ._core import BacksolveAdjoint, RecursiveCheckpointAdjoint


def _drift_and_diffusion(terms):
    from ._integrate import _split_terms
    drift, diff, _ = _split_terms(terms)
    return drift, (None if diff is None else diff.vector_field)


def needs_grad(terms, y0, args) -> bool:
    if not torch.is_grad_enabled():
        return False
    if isinstance(y0, torch.Tensor) and y0.requires_grad:
        return True
    if isinstance(args, torch.Tensor) and args.requires_grad:
        return True
    drift, diffusion = _drift_and_diffusion(terms)
    return bool(getattr(drift, "requires_grad", False) or
                getattr(diffusion, "requires_grad", False))


class _RecursiveCheckpointSolve(torch.autograd.Function):
    """RecursiveCheckpointAdjoint (diffrax/_adjoint.py:179-312): the forward
    kernel records the accepted-step grid and state checkpoints in the
    workspace; the backward kernel returns dL/dy0 and dL/dparams."""

    @staticmethod
    def forward(ctx, low, y0, params):
        ys, ts, res, stats, ws = low.run_forward(y0=y0.detach(), params=params.detach(),
                                                 keep_workspace=True)
        ctx.low = low
        ctx.save_for_backward(y0, params)
        ctx.ws = ws
        ctx.mark_non_differentiable(ts, res, stats)
        return ys, ts, res, stats

    @staticmethod
    def backward(ctx, grad_ys, _gts, _gres, _gstats):
        y0, params = ctx.saved_tensors
        low = ctx.low
        if grad_ys is None:
            grad_ys = torch.zeros((low.B, low.n_save, low.dim), dtype=low.dtype,
                                  device=low.device)
        grad_y0, grad_params = low.run_backward(ctx.ws, grad_ys, y0.detach(), params.detach())
        ctx.ws = None
        return (None, grad_y0 if ctx.needs_input_grad[1] else None,
                grad_params.to(params.dtype) if ctx.needs_input_grad[2] else None)


class _BacksolveSolve(torch.autograd.Function):
    """BacksolveAdjoint (diffrax/_adjoint.py:538-734): the forward keeps only
    the saved (ts, ys); the backward kernel solves the augmented adjoint system
    backwards between the saved times and returns dL/dy0 and dL/dparams."""

    @staticmethod
    def forward(ctx, low, y0, params):
        ys, ts, res, stats = low.run_forward(y0=y0.detach(), params=params.detach())
        ctx.low = low
        ctx.save_for_backward(params, ys, ts)
        ctx.mark_non_differentiable(ts, res, stats)
        return ys, ts, res, stats

    @staticmethod
    def backward(ctx, grad_ys, _gts, _gres, _gstats):
        params, ys, ts = ctx.saved_tensors
        low = ctx.low
        if grad_ys is None:
            grad_ys = torch.zeros_like(ys)
        grad_y0, grad_params, res, stats = low.run_backsolve(ts, ys.detach(), grad_ys,
                                                             params.detach())
        low.bwd_result, low.bwd_stats = res, stats
        if low.bwd_throw:
            # a reverse solve that failed (max_steps, dtmin) gives no gradient:
            # raise as the reference's backward diffeqsolve does with throw=True
            from ._integrate import _raise_on_failure
            _raise_on_failure(res)
        return (None, grad_y0 if ctx.needs_input_grad[1] else None,
                grad_params.to(params.dtype) if ctx.needs_input_grad[2] else None)


def _grad_like(g, x):
    """A gradient returned for input x: its shape, dtype and device."""
    if g is None or not isinstance(x, torch.Tensor):
        return None
    return g.reshape(x.shape).to(device=x.device, dtype=x.dtype)


class _AnalyticSolve(torch.autograd.Function):
    """Gradients of an analytic-field solve (Lotka-Volterra, Van der Pol,
    Ornstein-Uhlenbeck) with respect to y0 and args, under either adjoint:
    RecursiveCheckpointAdjoint (diffrax/_adjoint.py:179-312; the forward
    records every accepted step, the backward kernel applies the VJP of each
    step in reverse) or BacksolveAdjoint (diffrax/_adjoint.py:538-734; the
    backward kernel solves the augmented (y, a, a_args) system between the
    saved times).  `args_in` is the caller's args tensor, so that autograd
    hands dL/dargs back in its shape."""

    @staticmethod
    def forward(ctx, low, y0, args_in):
        backsolve = isinstance(low.adjoint, BacksolveAdjoint)
        ctx.low, ctx.backsolve = low, backsolve
        ctx.args_in = args_in
        if backsolve:
            ys, ts, res, stats = low.run_forward(y0=y0.detach())
            ctx.save_for_backward(ys, ts)
            ctx.ws = None
        else:
            ys, ts, res, stats, ws = low.run_forward(y0=y0.detach(), keep_workspace=True)
            ctx.save_for_backward(y0)
            ctx.ws = ws
        ctx.mark_non_differentiable(ts, res, stats)
        return ys, ts, res, stats

    @staticmethod
    def backward(ctx, grad_ys, _gts, _gres, _gstats):
        low = ctx.low
        if grad_ys is None:
            grad_ys = torch.zeros((low.B, low.n_save, low.dim), dtype=low.dtype,
                                  device=low.device)
        if ctx.backsolve:
            ys, ts = ctx.saved_tensors
            g_y0, g_args, res, stats = low.run_backsolve_args(ts, ys.detach(), grad_ys,
                                                              low.args.detach())
            low.bwd_result, low.bwd_stats = res, stats
            if low.bwd_throw:
                from ._integrate import _raise_on_failure
                _raise_on_failure(res)
        else:
            (y0,) = ctx.saved_tensors
            g_y0, g_args = low.run_backward_args(ctx.ws, grad_ys, y0.detach(),
                                                 low.args.detach())
            ctx.ws = None
        return (None, g_y0 if ctx.needs_input_grad[1] else None,
                _grad_like(g_args, ctx.args_in) if ctx.needs_input_grad[2] else None)


def solve_with_grad(low, y0, args):
    if low.params is None:
        # analytic fields: gradients with respect to y0 and args
        y0_dev = y0 if isinstance(y0, torch.Tensor) else torch.as_tensor(y0)
        y0_dev = y0_dev.to(device=low.device, dtype=low.dtype)
        if not y0_dev.is_contiguous():
            y0_dev = y0_dev.contiguous()
        args_in = args if isinstance(args, torch.Tensor) else None
        if not isinstance(low.adjoint, (RecursiveCheckpointAdjoint, BacksolveAdjoint)):
            raise NotImplementedError(f"adjoint {low.adjoint!r} is not supported")
        if args_in is None:
            # a placeholder input: no gradient flows to non-tensor args
            args_in = torch.zeros((), device=low.device)
        return _AnalyticSolve.apply(low, y0_dev, args_in)
    if isinstance(args, torch.Tensor) and args.requires_grad:
        raise NotImplementedError("MLP fields take no args to differentiate")
    if isinstance(low.adjoint, RecursiveCheckpointAdjoint):
        y0_dev = y0 if isinstance(y0, torch.Tensor) else torch.as_tensor(y0)
        y0_dev = y0_dev.to(device=low.device, dtype=low.dtype)
        if not y0_dev.is_contiguous():
            y0_dev = y0_dev.contiguous()
        if not y0_dev.requires_grad:
            y0_dev = y0_dev.detach()
        return _RecursiveCheckpointSolve.apply(low, y0_dev, low.params)
    if isinstance(low.adjoint, BacksolveAdjoint):
        y0_dev = y0 if isinstance(y0, torch.Tensor) else torch.as_tensor(y0)
        y0_dev = y0_dev.to(device=low.device, dtype=low.dtype)
        if not y0_dev.is_contiguous():
            y0_dev = y0_dev.contiguous()
        if not y0_dev.requires_grad:
            y0_dev = y0_dev.detach()
        return _BacksolveSolve.apply(low, y0_dev, low.params)
    raise NotImplementedError(f"adjoint {low.adjoint!r} is not supported")
