"""Gradients of a field-ramp run through libgpe's adjoint kernel, as a
``torch.autograd.Function``.

The forward and the reverse run happen in libgpe (``gpe_adjoint_forward`` /
``gpe_adjoint_backward``: CUDA step and adjoint kernels, sqrt(N) checkpoints with
recomputation).  torch only carries the chain rule from the per-step fields to
whatever parametrises them, here piecewise-linear knots of Bz(t) and of the
quadrupole gradient Bq(t).  The reference has no differentiable path; its ramps
are fixed tables (Spin1GpeBCC/AliceRingRamps.h:74-141, KnotRamps.h:64-135).
"""
from __future__ import annotations

from typing import Callable

import numpy as np
import torch

from .stepper import Stepper

# Indices of the five numbers the recorded run returns.
OVERLAP_RE, OVERLAP_IM, MAG_X, MAG_Y, MAG_Z = range(5)
# Columns of the per-step field rows.
BQ, BB_X, BB_Y, BB_Z = range(4)


def knot_matrix(n_knots: int, n_steps: int) -> np.ndarray:
    """(n_steps, n_knots) matrix of piecewise-linear interpolation: step j sits at
    s = j (n_knots - 1) / (n_steps - 1) on the knot axis and takes
    (1 - f) k_i + f k_{i+1}, i = floor(s), f = s - i."""
    if n_knots < 2 or n_steps < 1:
        raise ValueError("need at least two knots and one step")
    W = np.zeros((n_steps, n_knots))
    for j in range(n_steps):
        s = j * (n_knots - 1) / max(n_steps - 1, 1)
        i = min(int(np.floor(s)), n_knots - 2)
        f = s - i
        W[j, i] += 1.0 - f
        W[j, i + 1] += f
    return W


class FinalStateObservables(torch.autograd.Function):
    """fields (n, 4) float64 -> (5,) float64: Re <T|psi_N>, Im <T|psi_N>, M_x, M_y, M_z.

    ``reset`` puts the initial state into the stepper's PSI_ODD slot (an upload or
    a seeded device initialisation); the run starts from there every call."""

    @staticmethod
    def forward(ctx, fields: torch.Tensor, stepper: Stepper, reset: Callable[[], None], target: np.ndarray,
                stride: int = 0):
        reset()
        out = stepper.adjoint_forward(fields.detach().cpu().numpy(), target, stride)
        ctx.stepper = stepper
        ctx.dtype = fields.dtype
        ctx.device = fields.device
        return torch.from_numpy(out)

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        g = ctx.stepper.adjoint_backward(grad_out.detach().cpu().numpy())
        return torch.from_numpy(g).to(dtype=ctx.dtype, device=ctx.device), None, None, None, None


class RampControl:
    """Loss 1 - |<target|psi(T)>|^2 of a run whose Bz(t) and Bq(t) are
    piecewise-linear in n_knots knots each (Bb_x = Bb_y = 0)."""

    def __init__(self, stepper: Stepper, n_steps: int, n_knots: int, reset: Callable[[], None], target: np.ndarray,
                 stride: int = 0):
        self.stepper = stepper
        self.n_steps = n_steps
        self.reset = reset
        self.target = np.ascontiguousarray(target, dtype=np.float64)
        self.stride = stride
        self.W = torch.from_numpy(knot_matrix(n_knots, n_steps))

    def fields(self, bq_knots: torch.Tensor, bz_knots: torch.Tensor) -> torch.Tensor:
        zero = torch.zeros(self.n_steps, dtype=torch.float64)
        return torch.stack([self.W @ bq_knots, zero, zero, self.W @ bz_knots], dim=1)

    def observables(self, bq_knots: torch.Tensor, bz_knots: torch.Tensor) -> torch.Tensor:
        return FinalStateObservables.apply(self.fields(bq_knots, bz_knots), self.stepper, self.reset, self.target,
                                           self.stride)

    def loss(self, bq_knots: torch.Tensor, bz_knots: torch.Tensor) -> torch.Tensor:
        o = self.observables(bq_knots, bz_knots)
        return 1.0 - (o[OVERLAP_RE] ** 2 + o[OVERLAP_IM] ** 2)
