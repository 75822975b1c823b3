"""Differentiable operators: each forward runs one hand-written kernel and its
backward runs the hand-written adjoint kernel.

* ``Projector``: y = A x, backward A^T g           (projection <-> projection_t)
* ``ProjectorT``: x = A^T y, backward A g
* ``Backprojector``: x = B y, backward B^T g       (backprojection <-> backprojection_t)
* ``BackprojectorT``: y = B^T x, backward B g
* ``data_fidelity(x, y, options)``: 0.5*||A x - y||^2, whose forward computes the
  residual and A^T(A x - y) in one fused library call

For equal-angle fan geometry the reference's backprojection_t carries an extra
dImg/cbar factor (src/fan_ea_kernel.cu:590-607) and is therefore not the exact
transpose of its backprojection; the Backprojector pair reproduces the
reference operators as they are, so its gradient is the reference's
backprojection_t (which is what a CTLIB user wrapping the pair gets).

All four work with ``torch.utils.checkpoint`` (they save no activations: the
backward of a linear operator needs only its plan), so unrolled iterative
reconstructions can be checkpointed per iteration.
"""

from __future__ import annotations

import torch

from . import _native as N
from . import tune
from .ops import _check_input, get_plan


def _run(op: int, x: torch.Tensor, plan) -> torch.Tensor:
    x = _check_input(x.contiguous(), "input")
    B = x.shape[0]
    if op in (N.OP_PROJECTION, N.OP_BACKPROJECTION_T):
        shape = (B, 1, plan.views, plan.dets)
    else:
        shape = (B, 1, plan.height, plan.width)
    out = torch.empty(shape, dtype=x.dtype, device=x.device)
    if B == 0:
        return out
    tune.apply_cached(plan, op, B)
    with torch.cuda.device(x.device):
        return plan.run(op, x, out)


class _LinearOp(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, options, fwd: int, bwd: int):
        plan = get_plan(options, x.dtype, x.device)
        ctx.plan = plan
        ctx.bwd = bwd
        return _run(fwd, x.detach(), plan)

    @staticmethod
    def backward(ctx, g):
        if g is None:
            return None, None, None, None
        return _run(ctx.bwd, g.contiguous(), ctx.plan), None, None, None


def projection(x, options):
    return _LinearOp.apply(x, options, N.OP_PROJECTION, N.OP_PROJECTION_T)


def projection_t(y, options):
    return _LinearOp.apply(y, options, N.OP_PROJECTION_T, N.OP_PROJECTION)


def backprojection(y, options):
    return _LinearOp.apply(y, options, N.OP_BACKPROJECTION, N.OP_BACKPROJECTION_T)


def backprojection_t(x, options):
    return _LinearOp.apply(x, options, N.OP_BACKPROJECTION_T, N.OP_BACKPROJECTION)


class _Module(torch.nn.Module):
    _fn = None

    def __init__(self, options):
        super().__init__()
        if isinstance(options, torch.Tensor):
            options = options.detach().cpu().to(torch.float64)
        else:
            options = torch.tensor(list(options), dtype=torch.float64)
        self.register_buffer("options", options, persistent=False)

    def forward(self, x):
        return type(self)._fn(x, self.options)


class Projector(_Module):
    _fn = staticmethod(projection)


class ProjectorT(_Module):
    _fn = staticmethod(projection_t)


class Backprojector(_Module):
    _fn = staticmethod(backprojection)


class BackprojectorT(_Module):
    _fn = staticmethod(backprojection_t)


class _DataFidelity(torch.autograd.Function):
    """0.5*||A x - y||^2 summed over the batch. The forward pass computes the
    residual and the gradient A^T(A x - y) in one library call
    (ctgb_data_gradient); backward only scales them."""

    @staticmethod
    def forward(ctx, x, y, options):
        from .ops import data_gradient
        grad, res = data_gradient(x.detach(), y.detach(), options, return_residual=True)
        ctx.save_for_backward(grad, res)
        return 0.5 * (res.double() * res.double()).sum().to(x.dtype)

    @staticmethod
    def backward(ctx, g):
        grad, res = ctx.saved_tensors
        gx = g * grad if ctx.needs_input_grad[0] else None
        gy = -g * res if ctx.needs_input_grad[1] else None
        return gx, gy, None


def data_fidelity(x, y, options):
    """0.5*||A x - y||^2 for an image batch x and measured sinograms y, with
    d/dx = A^T(A x - y) and d/dy = -(A x - y) from one fused call."""
    return _DataFidelity.apply(x, y, options)
