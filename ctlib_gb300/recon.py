"""Unrolled iterative reconstruction on the differentiable operators.

The reference leaves iterative reconstruction to its callers, who compose
``projection`` and ``projection_t`` (src/ctlib.cpp:56-84, README.md:37-48).
This module is such a caller, written once:

* ``poisson_log_sinogram``: noisy measured data y = -log(N / I0) with photon
  counts N ~ Poisson(I0 exp(-A x)) clamped to >= 1, drawn with numpy from a
  fixed seed;
* ``gd_step_size``: 1 / (largest eigenvalue of A^T A), from power iteration,
  so that gradient descent on 0.5 ||A x - y||^2 is stable;
* ``unrolled_gd``: K iterations x <- x - step * A^T(A x - y), each iteration
  wrapped in ``torch.utils.checkpoint`` so that backpropagation through the
  recursion recomputes an iteration instead of keeping its activations.

The linear operators themselves keep no activations (their backward needs only
the plan), so for plain gradient descent checkpointing stores nothing less; it
is there for recursions that add learned or nonlinear steps per iteration.
"""

from __future__ import annotations

import numpy as np
import torch
from torch.utils.checkpoint import checkpoint

from . import autograd as _ag


def poisson_log_sinogram(line_integrals: np.ndarray, i0: float = 1e5, seed: int = 11) -> np.ndarray:
    """Noisy log sinogram of noiseless line integrals A x: counts
    N ~ Poisson(i0 * exp(-A x)), clamped to >= 1 (a detector reading of zero
    would make the log infinite), and y = -log(N / i0), in the input's dtype."""
    ax = np.asarray(line_integrals, dtype=np.float64)
    counts = np.random.default_rng(seed).poisson(i0 * np.exp(-ax))
    counts = np.maximum(counts, 1)
    return (-np.log(counts / i0)).astype(np.asarray(line_integrals).dtype)


def gd_step_size(options, height: int, width: int, device, iters: int = 30, seed: int = 0,
                 dtype=torch.float32) -> float:
    """1 / lambda_max(A^T A) by power iteration from a seeded Gaussian start."""
    g = torch.Generator().manual_seed(seed)
    x = torch.randn(1, 1, height, width, generator=g, dtype=torch.float64).to(device=device, dtype=dtype)
    lam = 0.0
    for _ in range(iters):
        x = x / x.double().norm().to(dtype)
        y = _ag.projection_t(_ag.projection(x, options), options)
        lam = float((x.double() * y.double()).sum())
        x = y
    return 1.0 / lam


def _gd_iteration(x, y, options, step):
    return x - step * _ag.projection_t(_ag.projection(x, options) - y, options)


def unrolled_gd(y: torch.Tensor, options, iters: int, step: float, x0: torch.Tensor | None = None,
                use_checkpoint: bool = True) -> torch.Tensor:
    """x_K of K gradient-descent iterations on 0.5 ||A x - y||^2 from x0
    (zeros by default), differentiable with respect to y (and x0) through the
    hand-written adjoint kernels; each iteration is checkpointed unless
    ``use_checkpoint`` is False."""
    B = y.shape[0]
    if x0 is None:
        plan_shape = _image_shape(options)
        x = torch.zeros((B, 1) + plan_shape, dtype=y.dtype, device=y.device)
    else:
        x = x0
    for _ in range(iters):
        if use_checkpoint:
            x = checkpoint(_gd_iteration, x, y, options, step, use_reentrant=False)
        else:
            x = _gd_iteration(x, y, options, step)
    return x


def _image_shape(options) -> tuple:
    vals = options.detach().cpu().tolist() if isinstance(options, torch.Tensor) else list(options)
    return (int(vals[3]), int(vals[2]))
