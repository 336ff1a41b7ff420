"""``forward`` / ``backward`` and the autograd functions, mirroring curadon's
forward.py:7-28, backward.py:7-29 and diffable.py:14-38.

``forward(volume, sinogram, geom)`` overwrites ``sinogram`` (3D: rays that
miss the volume keep their value) and returns it; ``backward(sinogram,
volume, geom)`` adds the backprojection into ``volume`` and returns it.

``TorchForward.apply(volume, geom)`` / ``TorchBackprojection.apply(sino,
geom)`` are the reference's autograd functions made to work: they allocate
their outputs (the reference's versions call the 3-argument API with two
arguments and fail).  The backward of the forward projection is the
backprojector, and vice versa, as in the reference.
"""
from __future__ import annotations

from typing import Union

import torch
from torch.autograd import Function

from . import backend as _C
from .geometry import ConeGeometry, FanGeometry

__all__ = ["forward", "backward", "adjoint", "TorchForward", "TorchBackprojection"]


def forward(volume, sinogram, geom: Union[FanGeometry, ConeGeometry], exact: bool = False):
    """Forward projection into ``sinogram``.  ``exact=True`` uses the
    geometry's FP32-filtering plan, whose transpose ``adjoint`` is exactly."""
    if isinstance(geom, FanGeometry):
        _C.forward_2d(volume, sinogram, geom.exact_plan if exact else geom.plan)
        return sinogram
    if isinstance(geom, ConeGeometry):
        (geom.exact_plan if exact else geom.plan).forward(volume, sinogram)
        return sinogram
    raise ValueError("Unknown geometry type")


def backward(sinogram, volume, geom: Union[FanGeometry, ConeGeometry]):
    if isinstance(geom, FanGeometry):
        _C.backward_2d(volume, sinogram, geom.plan)
        return volume
    if isinstance(geom, ConeGeometry):
        geom.plan.backward(volume, sinogram)
        return volume
    raise ValueError("Unknown geometry type")


def adjoint(sinogram, volume, geom: Union[FanGeometry, ConeGeometry]):
    """Adds the matched adjoint A^T sinogram -- the exact transpose of
    ``forward(..., exact=True)`` -- to ``volume`` and returns it.  An addition
    beside the reference's API."""
    if isinstance(geom, FanGeometry):
        _C.adjoint_2d(volume, sinogram, geom.exact_plan)
        return volume
    if isinstance(geom, ConeGeometry):
        geom.exact_plan.adjoint(volume, sinogram)
        return volume
    raise ValueError("Unknown geometry type")


def _vol_shape(geom):
    return tuple(int(v) for v in geom.vol_shape)


class TorchForward(Function):
    """Differentiable forward projection.

    ``TorchForward.apply(volume, geom)``: the gradient is the reference's
    voxel-driven backprojector (as in diffable.py:21-24).
    ``TorchForward.apply(volume, geom, True)``: the forward filters in FP32
    and the gradient is its matched adjoint, so it is the exact gradient."""

    @staticmethod
    def forward(ctx, volume, geom, matched=False):
        sino = torch.zeros(geom.sinogram_shape(), device=volume.device, dtype=torch.float32)
        forward(volume.detach().contiguous(), sino, geom, exact=bool(matched))
        ctx.geom = geom
        ctx.matched = bool(matched)
        return sino

    @staticmethod
    def backward(ctx, grad_sino):
        grad = torch.zeros(_vol_shape(ctx.geom), device=grad_sino.device, dtype=torch.float32)
        op = adjoint if ctx.matched else backward
        op(grad_sino.detach().contiguous(), grad, ctx.geom)
        return grad, None, None


class TorchBackprojection(Function):
    """Differentiable backprojection; gradient = forward projection."""

    @staticmethod
    def forward(ctx, sino, geom):
        vol = torch.zeros(_vol_shape(geom), device=sino.device, dtype=torch.float32)
        backward(sino.detach().contiguous(), vol, geom)
        ctx.geom = geom
        return vol

    @staticmethod
    def backward(ctx, grad_vol):
        grad = torch.zeros(ctx.geom.sinogram_shape(), device=grad_vol.device,
                           dtype=torch.float32)
        forward(grad_vol.detach().contiguous(), grad, ctx.geom)
        return grad, None
