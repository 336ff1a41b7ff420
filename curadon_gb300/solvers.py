"""Fixed-iteration reconstructions on the GPU operators: SIRT and CGLS.

Both run entirely on the device with preallocated iterates, so one iteration
can be captured in a CUDA graph and replayed (``graph=True``): the scalars of
CGLS stay device tensors and no iteration synchronises with the host.

* ``sirt``: x <- x + lam C A^T R (y - A x), R = 1 / A 1, C = 1 / A^T 1, with
  A the forward projection and A^T the drop-in backprojector (the pair the
  reference's API offers); iterates are clipped at 0 if asked.
* ``cgls``: conjugate gradients on the normal equations with the matched
  adjoint, A^T the exact transpose of A (``forward(..., exact=True)`` and
  ``adjoint``), for 2D and 3D.
"""
from __future__ import annotations

from typing import Optional, Union

import torch

from .geometry import ConeGeometry, FanGeometry
from .ops import adjoint, backward, forward

__all__ = ["sirt", "cgls", "SirtSolver", "CglsSolver"]

Geom = Union[FanGeometry, ConeGeometry]


def _vol_shape(geom: Geom):
    return tuple(int(v) for v in geom.vol_shape)


def _capture(fn, device) -> "torch.cuda.CUDAGraph":
    """Captures ``fn()`` as a CUDA graph on a side stream that follows the
    current stream, without synchronising the device (so that a server's
    other streams keep running while a new solver is captured); capturing
    does not execute ``fn``'s work."""
    cur = torch.cuda.current_stream(device)
    side = torch.cuda.Stream(device)
    side.wait_stream(cur)
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(side):
        g.capture_begin(capture_error_mode="thread_local")
        try:
            fn()
        finally:
            g.capture_end()
    cur.wait_stream(side)
    return g


def _safe_inv(t: torch.Tensor) -> torch.Tensor:
    return torch.where(t > 1e-6, 1.0 / t.clamp_min(1e-6), torch.zeros_like(t))


class SirtSolver:
    """SIRT with all buffers allocated once; ``run(y, iters)`` returns x."""

    def __init__(self, geom: Geom, device, lam: float = 1.0, nonneg: bool = True,
                 graph: bool = False):
        self.geom, self.lam, self.nonneg = geom, float(lam), bool(nonneg)
        shape = _vol_shape(geom)
        dev = torch.device(device)
        self.x = torch.zeros(shape, device=dev)
        self.y = torch.zeros(geom.sinogram_shape(), device=dev)
        self.r = torch.zeros_like(self.y)
        self.bp = torch.zeros_like(self.x)
        ones_v = torch.ones(shape, device=dev)
        ones_s = torch.ones_like(self.y)
        rs = torch.zeros_like(self.y)
        cs = torch.zeros_like(self.x)
        forward(ones_v, rs, geom)
        backward(ones_s, cs, geom)
        self.R = _safe_inv(rs)
        self.C = _safe_inv(cs) * self.lam
        self.use_graph = bool(graph)
        self._graph = None

    def _iteration(self):
        forward(self.x, self.r, self.geom)
        torch.sub(self.y, self.r, out=self.r)
        self.r.mul_(self.R)
        self.bp.zero_()
        backward(self.r, self.bp, self.geom)
        self.x.addcmul_(self.C, self.bp)
        if self.nonneg:
            self.x.clamp_(min=0.0)

    def _capture(self):
        self._iteration()  # warm-up outside the capture (scratch, texture arrays)
        self._graph = _capture(self._iteration, self.x.device)

    def run(self, y: torch.Tensor, iters: int, x0: Optional[torch.Tensor] = None) -> torch.Tensor:
        if self.use_graph and self._graph is None:
            self._capture()
        self.y.copy_(y)
        if x0 is None:
            self.x.zero_()
        else:
            self.x.copy_(x0)
        for _ in range(int(iters)):
            if self._graph is not None:
                self._graph.replay()
            else:
                self._iteration()
        return self.x


class CglsSolver:
    """CGLS with the matched adjoint; ``run(y, iters)`` returns x."""

    def __init__(self, geom: Geom, device, graph: bool = False):
        self.geom = geom
        shape = _vol_shape(geom)
        dev = torch.device(device)
        self.x = torch.zeros(shape, device=dev)
        self.p = torch.zeros_like(self.x)
        self.s = torch.zeros_like(self.x)
        self.r = torch.zeros(geom.sinogram_shape(), device=dev)
        self.q = torch.zeros_like(self.r)
        self.gamma = torch.zeros((), device=dev)
        self.use_graph = bool(graph)
        self._graph = None

    def _start(self, y, x0):
        if x0 is None:
            self.x.zero_()
            self.r.copy_(y)
        else:
            self.x.copy_(x0)
            forward(self.x, self.q, self.geom, exact=True)
            torch.sub(y, self.q, out=self.r)
        self.s.zero_()
        adjoint(self.r, self.s, self.geom)
        self.p.copy_(self.s)
        self.gamma.copy_(torch.sum(self.s * self.s))

    def _iteration(self):
        forward(self.p, self.q, self.geom, exact=True)
        qq = torch.sum(self.q * self.q)
        alpha = torch.where(qq > 0, self.gamma / qq.clamp_min(1e-30), torch.zeros_like(qq))
        self.x.add_(alpha * self.p)
        self.r.sub_(alpha * self.q)
        self.s.zero_()
        adjoint(self.r, self.s, self.geom)
        gamma_new = torch.sum(self.s * self.s)
        beta = torch.where(self.gamma > 0, gamma_new / self.gamma.clamp_min(1e-30),
                           torch.zeros_like(gamma_new))
        self.p.mul_(beta).add_(self.s)
        self.gamma.copy_(gamma_new)

    def _capture(self):
        self._graph = _capture(self._iteration, self.x.device)

    def run(self, y: torch.Tensor, iters: int, x0: Optional[torch.Tensor] = None) -> torch.Tensor:
        self._start(y, x0)
        if self.use_graph and self._graph is None and iters > 0:
            # the first iteration runs outside the capture (scratch exists after
            # it); capturing does not execute, so the state is unchanged
            self._iteration()
            iters -= 1
            self._capture()
        for _ in range(int(iters)):
            if self._graph is not None:
                self._graph.replay()
            else:
                self._iteration()
        return self.x


def sirt(geom: Geom, sinogram: torch.Tensor, iters: int = 20, lam: float = 1.0,
         nonneg: bool = True, graph: bool = False) -> torch.Tensor:
    """SIRT reconstruction (returns a new volume)."""
    return SirtSolver(geom, sinogram.device, lam, nonneg, graph).run(sinogram, iters).clone()


def cgls(geom: Geom, sinogram: torch.Tensor, iters: int = 30, graph: bool = False) -> torch.Tensor:
    """CGLS reconstruction with the matched adjoint (returns a new volume)."""
    return CglsSolver(geom, sinogram.device, graph).run(sinogram, iters).clone()
