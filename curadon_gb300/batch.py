"""Many 2D problems per launch (``cg_batch2d_*``).

``Batch2d(geoms, volumes, sinograms)`` binds any number of fan-beam problems
-- any sizes, circular or vector geometries -- to their float32 CUDA
tensors.  ``forward()`` then projects every volume into its sinogram and
``backward()`` adds every backprojection into its volume, each over a
(problem, tile) work list in one or two launches instead of two per problem.
The buffers stay bound, so both calls can be captured in a CUDA graph
(``torch.cuda.graph``) and an iteration loop replayed without launch
overhead.  The forward is the texture-unit ray march (``forward="texture"``,
default: one array copy per problem, then one launch) or the FP32 register
march (``forward="registers"``); the backprojection is the staged one; their
results equal the single-problem operators with those algorithms bit for
bit.  No counterpart in the reference, which runs one problem per call.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import torch

from ._lib import check, load
from .backend import _check_tensor, _stream
from .geometry import FanGeometry

__all__ = ["Batch2d"]


class Batch2d:
    FORWARD = ("registers", "texture")

    def __init__(self, geoms: Sequence[FanGeometry], volumes: Sequence[torch.Tensor],
                 sinograms: Sequence[torch.Tensor], forward: str = "texture"):
        if forward not in self.FORWARD:
            raise ValueError(f"batched forward must be one of {self.FORWARD}")
        if not (len(geoms) == len(volumes) == len(sinograms)) or not geoms:
            raise ValueError("geoms, volumes and sinograms must be non-empty and of one length")
        dev = volumes[0].device
        plans, seen = [], set()
        for g, v, s in zip(geoms, volumes, sinograms):
            if not isinstance(g, FanGeometry):
                raise TypeError("batches hold FanGeometry problems")
            _check_tensor(v, "volume", 2)
            _check_tensor(s, "sinogram", 2)
            if v.device != dev or s.device != dev:
                raise AttributeError("all tensors of a batch must be on one device")
            if tuple(v.shape) != tuple(int(x) for x in g.vol_shape):
                raise ValueError(f"volume shape {tuple(v.shape)} != geometry {tuple(g.vol_shape)}")
            if tuple(s.shape) != g.sinogram_shape():
                raise ValueError(f"sinogram shape {tuple(s.shape)} != {g.sinogram_shape()}")
            # each problem needs its own plan scratch: a geometry used twice
            # gets a private plan for its second use
            p = g.plan if id(g) not in seen else g._make_plan()
            seen.add(id(g))
            plans.append(p)
        self._L = load()
        n = len(plans)
        hp = (C.c_void_p * n)(*[p.handle.value for p in plans])
        vp = (C.c_void_p * n)(*[v.data_ptr() for v in volumes])
        sp = (C.c_void_p * n)(*[s.data_ptr() for s in sinograms])
        h = C.c_void_p()
        check(self._L.cg_batch2d_create(C.byref(h), hp, vp, sp, n))
        self._h = h
        check(self._L.cg_batch2d_set_forward(h, self.FORWARD.index(forward)))
        self._keep = (list(geoms), list(volumes), list(sinograms), plans)
        self.device = dev
        self.count = n

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
