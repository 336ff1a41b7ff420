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
march (``forward="registers"``); ``forward="auto"`` times both on the bound
problems once and keeps the faster (the sinograms' contents are restored
afterwards).  The backprojection is the staged one; results equal the
single-problem operators with those algorithms bit for bit.  No
counterpart in the reference, which runs one problem per call.
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
        if forward not in self.FORWARD + ("auto",):
            raise ValueError(f"batched forward must be one of {self.FORWARD + ('auto',)}")
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
