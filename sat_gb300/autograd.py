"""torch.autograd over the SAT kernels: a differentiable SAT and a box-filter
layer.  The reference has no backward pass; these extend its forward SAT
(integralImage/integralImage.h:105-124 defines S(y,x) = sum_{i<=y, j<=x} I(i,j)).

Backward of the SAT.  S is linear in I with dS(y,x)/dI(i,j) = [i <= y][j <= x],
so dL/dI(i,j) = sum_{y >= i, x >= j} dL/dS(y,x): the suffix (reverse) SAT of
the incoming gradient, one launch of the same kernel with direction=reverse.

Box filter.  box_filter_means(x, radii) returns the clipped box means of every
radius, read by four corners from the SAT of x (one SAT launch plus one box
launch forward).  Backward: the adjoint gather into the gradient tensor,
then the reverse SAT of that tensor in place (the plain mode in one call of
the library, the compensated mode with the compensated reverse SAT).
"""
from __future__ import annotations

from typing import Sequence

import torch

from . import api


def _as_f32_cuda(t: torch.Tensor) -> torch.Tensor:
    if not t.is_cuda:
        raise api.SatError(api._lib.ERR_INVALID_ARG, "tensors must be CUDA tensors (there is no CPU path)")
    if t.dtype != torch.float32:
        raise api.SatError(api._lib.ERR_UNSUPPORTED_TYPES, "the autograd SAT takes f32 tensors")
    return t.contiguous()


class SATFunction(torch.autograd.Function):
    """S = SAT(x) over the last two dimensions of an f32 (..., H, W) tensor;
    backward is the reverse SAT of dL/dS."""

    @staticmethod
    def forward(ctx, x: torch.Tensor, mode: str = "plain"):
        x = _as_f32_cuda(x)
        ctx.mode = mode
        return api.sat(x, torch.float32, mode=mode)

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        g = _as_f32_cuda(g)
        return api.sat(g, torch.float32, mode=ctx.mode, reverse=True), None


def sat(x: torch.Tensor, mode: str = "plain") -> torch.Tensor:
    """Differentiable SAT of an f32 (..., H, W) tensor."""
    return SATFunction.apply(x, mode)


class BoxMeansFunction(torch.autograd.Function):
    """(..., H, W) -> (..., R, H, W): clipped box means of radius radii[k],
    computed from the SAT of x.  Backward: the four-corner adjoint (a gather)
    gives dL/dSAT, whose reverse SAT is dL/dx."""

    @staticmethod
    def forward(ctx, x: torch.Tensor, radii: tuple, mode: str = "plain"):
        x = _as_f32_cuda(x)
        ctx.radii = radii
        ctx.mode = mode
        s = api.sat(x, torch.float32, mode=mode)
        return api.box_means_from_sat(s, radii)

    @staticmethod
    def backward(ctx, g: torch.Tensor):
        g = _as_f32_cuda(g)
        if ctx.mode == "plain":
            # adjoint gather and in-place reverse SAT in one library call
            return api.box_means_grad_x(g, ctx.radii), None, None
        gs = api.box_means_adjoint(g, ctx.radii)
        # the reverse SAT may overwrite its input in place: gs is ours alone
        return api.sat(gs, torch.float32, mode=ctx.mode, reverse=True, out=gs), None, None


def box_filter_means(x: torch.Tensor, radii: Sequence[int], mode: str = "plain") -> torch.Tensor:
    """Box means of x (f32, (..., H, W)) for 1..4 radii, stacked as (..., R, H, W)."""
    radii = tuple(int(r) for r in radii)
    return BoxMeansFunction.apply(x, radii, mode)


class BoxFilter(torch.nn.Module):
    """A box-filter layer: (..., H, W) -> (..., R, H, W) box means."""

    def __init__(self, radii: Sequence[int] = (3, 7, 15), mode: str = "plain"):
        super().__init__()
        self.radii = tuple(int(r) for r in radii)
        self.mode = mode

    def forward(self, x: torch.Tensor) -> torch.Tensor:
        return box_filter_means(x, self.radii, self.mode)

    def extra_repr(self) -> str:
        return f"radii={self.radii}, mode={self.mode!r}"
