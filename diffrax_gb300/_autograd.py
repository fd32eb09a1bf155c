"""torch.autograd bridge: the forward and adjoint kernels behind one
autograd.Function per adjoint kind."""
from __future__ import annotations

import torch


def needs_grad(low, y0, args) -> bool:
    if not torch.is_grad_enabled():
        return False
    if isinstance(y0, torch.Tensor) and y0.requires_grad:
        return True
    if isinstance(args, torch.Tensor) and args.requires_grad:
        return True
    return bool(getattr(low.drift, "requires_grad", False))


def solve_with_grad(low, y0, args):
    raise NotImplementedError("gradients for this field are not available")
