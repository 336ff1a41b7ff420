"""Many 2D and 3D problems per launch (``cg_batch2d_*``, ``cg_batch3d_*``).

``Batch2d(geoms, volumes, sinograms)`` binds any number of fan-beam problems
-- any sizes, circular or vector geometries -- to their float32 CUDA
tensors.  ``forward()`` then projects every volume into its sinogram and
``backward()`` adds every backprojection into its volume, each over a
(problem, tile) work list in one or two launches instead of two per problem.
The buffers stay bound, so both calls can be captured in a CUDA graph
(``torch.cuda.graph``) and an iteration loop replayed without launch
overhead.  The forward is the texture-unit ray march (``forward="texture"``,
default: one array copy per problem, then one launch), the FP32 register
march (``forward="registers"``) or each problem's own plan default
(``forward="plans"``: the chunked shared-memory forward for problems from
704^2 pixels, in one re-layout and one bundle launch over all of them, the
texture march for the others); ``forward="auto"`` times them on the bound
problems once and keeps the fastest (the sinograms' contents are restored
afterwards).  The backprojection is the staged one; results equal the
single-problem operators with those algorithms bit for bit; ``adjoint()``
adds the matched adjoint (the exact transpose of the register forward).
``BatchProjector`` wraps a batch as a differentiable PyTorch function over
flat buffers.  ``Batch3d`` does the same for cone-beam problems (any volume
and detector sizes, views and geometries): the quad forward with each
plan's texture warps and the axial or general backprojection, bit-equal to
the single-problem operators, and the matched adjoint of the quad forward.
No counterpart in the reference, which runs
one problem per call.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np
import torch

from ._lib import check, load
from .backend import _check_tensor, _stream
from .geometry import ConeGeometry, FanGeometry

__all__ = ["Batch2d", "Batch3d", "BatchProjector"]


def _bind_plans(geoms, volumes, sinograms, kind, ndim, exact=False):
    """The plans of a batch's problems after checking its tensors (with
    ``exact``, the geometries' FP32-filtering plans); a geometry used twice
    gets a private plan for its second use (each problem needs its own plan
    scratch)."""
    if not (len(geoms) == len(volumes) == len(sinograms)) or not geoms:
        raise ValueError("geoms, volumes and sinograms must be non-empty and of one length")
    dev = volumes[0].device
    plans, seen = [], set()
    for g, v, s in zip(geoms, volumes, sinograms):
        if not isinstance(g, kind):
            raise TypeError(f"batches hold {kind.__name__} problems")
        _check_tensor(v, "volume", ndim)
        _check_tensor(s, "sinogram", ndim)
        if v.device != dev or s.device != dev:
            raise AttributeError("all tensors of a batch must be on one device")
        if tuple(v.shape) != tuple(int(x) for x in g.vol_shape):
            raise ValueError(f"volume shape {tuple(v.shape)} != geometry {tuple(g.vol_shape)}")
        if tuple(s.shape) != tuple(g.sinogram_shape()):
            raise ValueError(f"sinogram shape {tuple(s.shape)} != {tuple(g.sinogram_shape())}")
        if id(g) not in seen:
            p = g.exact_plan if exact else g.plan
        else:
            p = g._make_plan()
            if exact:
                p.set_algorithm(forward="quad" if ndim == 3 else "registers")
        seen.add(id(g))
        plans.append(p)
    return plans, dev


def _pointers(objs):
    return (C.c_void_p * len(objs))(*objs)


class Batch2d:
    FORWARD = ("registers", "texture", "plans")

    def __init__(self, geoms: Sequence[FanGeometry], volumes: Sequence[torch.Tensor],
                 sinograms: Sequence[torch.Tensor], forward: str = "texture"):
        if forward not in self.FORWARD + ("auto",):
            raise ValueError(f"batched forward must be one of {self.FORWARD + ('auto',)}")
        plans, dev = _bind_plans(geoms, volumes, sinograms, FanGeometry, 2)
        self._L = load()
        n = len(plans)
        h = C.c_void_p()
        check(self._L.cg_batch2d_create(
            C.byref(h), _pointers([p.handle.value for p in plans]),
            _pointers([v.data_ptr() for v in volumes]),
            _pointers([s.data_ptr() for s in sinograms]), n))
        self._h = h
        self._keep = (list(geoms), list(volumes), list(sinograms), plans)
        self.device = dev
        self.count = n
        self.tuned_ms: dict[str, float] = {}
        if forward == "auto":
            self._tune_forward()
        else:
            check(self._L.cg_batch2d_set_forward(h, self.FORWARD.index(forward)))

    def _tune_forward(self, reps: int = 3) -> None:
        """Times every batched forward on the bound problems (CUDA events on
        the current stream, median of ``reps`` after one warm-up) and keeps
        the fastest; the bound sinograms are restored."""
        sinos = self._keep[2]
        saved = [s.clone() for s in sinos]
        best = None
        for i, name in enumerate(self.FORWARD):
            check(self._L.cg_batch2d_set_forward(self._h, i))
            self.forward()
            ts = []
            for _ in range(reps):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record()
                self.forward()
                b.record()
                b.synchronize()
                ts.append(a.elapsed_time(b))
            t = sorted(ts)[len(ts) // 2]
            self.tuned_ms[name] = t
            if best is None or t < best[0]:
                best = (t, i)
        check(self._L.cg_batch2d_set_forward(self._h, best[1]))
        for s, c in zip(sinos, saved):
            s.copy_(c)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.cg_batch2d_destroy(h)
            self._h = None

    @property
    def forward_algorithm(self) -> str:
        a = C.c_int()
        check(self._L.cg_batch2d_get_forward(self._h, C.byref(a)))
        return self.FORWARD[a.value]

    def forward(self):
        """sinogram_i = A_i volume_i for every problem (on the current stream)."""
        check(self._L.cg_batch2d_forward(self._h, _stream(self._keep[1][0])))

    def backward(self):
        """volume_i += A_i^T sinogram_i for every problem."""
        check(self._L.cg_batch2d_backward(self._h, _stream(self._keep[1][0])))

    def set_active(self, active: int):
        """Later calls run problems [0, active) only (a resident batch serving
        however many requests are waiting)."""
        check(self._L.cg_batch2d_set_active(self._h, int(active)))

    def adjoint(self):
        """volume_i += the matched adjoint of sinogram_i for every problem (the
        exact transpose of the ``forward="registers"`` march; the first call
        allocates the accumulators, so make it before a graph capture)."""
        check(self._L.cg_batch2d_adjoint(self._h, _stream(self._keep[1][0])))


class Batch3d:
    """Cone-beam problems bound to their float32 CUDA volumes and projections
    (``cg_batch3d_*``).  ``forward()`` projects every volume (the quad ray
    march with each plan's texture warps; as the single-problem forward, it
    writes only the rays that hit the volume's box) and ``backward()`` adds
    every backprojection into its volume (axial runs where the geometry
    allows them, the general kernel otherwise), each over a (problem, tile)
    work list in a few launches; results equal ``plan.forward`` /
    ``plan.backward`` bit for bit (plans set to the "registers" or "texture"
    forward run the "quad" forward here).  With ``exact=True`` the batch
    binds the geometries' FP32-filtering plans (``exact_plan``: the quad
    forward without texture warps), whose transpose ``adjoint()`` adds.
    Binding allocates each plan's quad copies.  Capturable in a CUDA graph."""

    def __init__(self, geoms: Sequence[ConeGeometry], volumes: Sequence[torch.Tensor],
                 sinograms: Sequence[torch.Tensor], exact: bool = False):
        plans, dev = _bind_plans(geoms, volumes, sinograms, ConeGeometry, 3, exact=exact)
        self._L = load()
        h = C.c_void_p()
        check(self._L.cg_batch3d_create(
            C.byref(h), _pointers([p.handle.value for p in plans]),
            _pointers([v.data_ptr() for v in volumes]),
            _pointers([s.data_ptr() for s in sinograms]), len(plans)))
        self._h = h
        self._keep = (list(geoms), list(volumes), list(sinograms), plans)
        self.device = dev
        self.count = len(plans)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.cg_batch3d_destroy(h)
            self._h = None

    def forward(self):
        """projections_i = A_i volume_i for every problem (on the current stream)."""
        check(self._L.cg_batch3d_forward(self._h, _stream(self._keep[1][0])))

    def backward(self):
        """volume_i += A_i^T projections_i for every problem."""
        check(self._L.cg_batch3d_backward(self._h, _stream(self._keep[1][0])))

    def set_active(self, active: int):
        """Later calls run problems [0, active) only."""
        check(self._L.cg_batch3d_set_active(self._h, int(active)))

    def adjoint(self):
        """volume_i += the matched adjoint of projections_i for every problem
        (the exact transpose of the quad forward without texture warps; the
        first call allocates the accumulators, so make it before a graph
        capture)."""
        check(self._L.cg_batch3d_adjoint(self._h, _stream(self._keep[1][0])))


class _BatchProject(torch.autograd.Function):
    """s = A x over a whole batch, x and s flat (every problem's volume, then
    every problem's sinogram, concatenated); the backward is the batched
    drop-in backprojector or, for a matched projector, the batched adjoint."""

    @staticmethod
    def forward(ctx, x, proj):
        proj.X.copy_(x)
        if proj.cone:
            proj.S.zero_()  # the 3D forward writes only the rays that hit the box
        proj._fwd.forward()
        ctx.proj = proj
        return proj.S.clone()

    @staticmethod
    def backward(ctx, grad):
        p = ctx.proj
        p.R.copy_(grad)
        p.G.zero_()
        if p.matched:
            p._bwd.adjoint()
        else:
            p._bwd.backward()
        return p.G.clone(), None


class BatchProjector:
    """The projection operator of a whole batch as a differentiable PyTorch
    function.  ``BatchProjector(geoms, device)`` binds the problems to flat
    buffers once; ``proj(x)`` takes every volume concatenated (float32, as
    ``proj.split_volumes`` splits it) and returns every sinogram
    concatenated, through ``torch.autograd``: its gradient is the batched
    backprojection (the reference's gradient of the forward is its
    backprojector, python/standalone/src/curadon/diffable.py:14-38) or, with
    ``matched=True``, the batched matched adjoint, the exact transpose of the
    register forward that ``matched`` selects.  Both directions are a few
    launches for the whole batch, capturable in a CUDA graph.  A list of
    ``ConeGeometry`` problems makes a 3D batch (``Batch3d``; with
    ``matched=True`` the quad forward without texture warps and its batched
    matched adjoint)."""

    def __init__(self, geoms: Sequence[FanGeometry | ConeGeometry], device=None,
                 forward: str = "plans", matched: bool = False):
        dev = torch.device("cuda", 0) if device is None else torch.device(device)
        self.geoms = list(geoms)
        self.matched = bool(matched)
        self.cone = bool(self.geoms) and isinstance(self.geoms[0], ConeGeometry)
        self.vol_shapes = [tuple(int(v) for v in g.vol_shape) for g in self.geoms]
        self.sino_shapes = [tuple(g.sinogram_shape()) for g in self.geoms]
        nv = [int(np.prod(s)) for s in self.vol_shapes]
        ns = [int(np.prod(s)) for s in self.sino_shapes]
        self.vol_offsets = np.cumsum([0] + nv)
        self.sino_offsets = np.cumsum([0] + ns)
        self.X = torch.zeros(int(self.vol_offsets[-1]), device=dev)
        self.G = torch.zeros_like(self.X)
        self.S = torch.zeros(int(self.sino_offsets[-1]), device=dev)
        self.R = torch.zeros_like(self.S)
        if self.cone:
            self._fwd = Batch3d(self.geoms, self.split_volumes(self.X),
                                self.split_sinograms(self.S), exact=self.matched)
            self._bwd = Batch3d(self.geoms, self.split_volumes(self.G),
                                self.split_sinograms(self.R), exact=self.matched)
        else:
            self._fwd = Batch2d(self.geoms, self.split_volumes(self.X),
                                self.split_sinograms(self.S),
                                forward="registers" if self.matched else forward)
            self._bwd = Batch2d(self.geoms, self.split_volumes(self.G),
                                self.split_sinograms(self.R))
        self.device = dev

    def split_volumes(self, flat: torch.Tensor):
        o = self.vol_offsets
        return [flat[o[i]:o[i + 1]].view(s) for i, s in enumerate(self.vol_shapes)]

    def split_sinograms(self, flat: torch.Tensor):
        o = self.sino_offsets
        return [flat[o[i]:o[i + 1]].view(s) for i, s in enumerate(self.sino_shapes)]

    def __call__(self, x: torch.Tensor) -> torch.Tensor:
        if x.shape != self.X.shape or x.dtype != torch.float32 or x.device != self.device:
            raise ValueError(f"x must be a float32 tensor of {tuple(self.X.shape)} elements on "
                             f"{self.device}")
        return _BatchProject.apply(x, self)

    def adjoint(self, s: torch.Tensor) -> torch.Tensor:
        """A^T s (no autograd) with this projector's backward operator."""
        self.R.copy_(s)
        self.G.zero_()
        if self.matched:
            self._bwd.adjoint()
        else:
            self._bwd.backward()
        return self.G.clone()
