"""Reconstruction serving with continuous admission.

``Server`` runs FBP, fixed-iteration SIRT and CGLS requests of mixed 2D / 3D
sizes.  A request is admitted as soon as an execution slot (a CUDA stream
with its own resident plans and iterates) and device memory are free; work
of admitted requests overlaps on the GPU while later requests arrive.
Geometry plans, filters and solver iterates stay resident per slot, keyed by
the geometry, so a repeated geometry costs no set-up.  Admission is capped
by a device-memory budget and by the memory the device reports free.  Every
request's result is the same whether it runs alone or among others: each
slot has private scratch and the kernels are deterministic (CGLS's matched
adjoint accumulates with atomics, so its results agree to rounding, within
relative L2 1e-3).

Latencies (submission to result on the host) and throughput are kept for
``stats()`` (p50 / p99 latency, solves per second).
"""
from __future__ import annotations

import collections
import hashlib
import threading
import time
from concurrent.futures import Future
from dataclasses import dataclass, field
from typing import Dict, List, Optional, Union

import numpy as np
import torch

from .fbp import fbp
from .geometry import ConeGeometry, FanGeometry, FanVecGeometry
from .solvers import CglsSolver, SirtSolver

__all__ = ["Request", "Server", "solve_alone"]

Geom = Union[FanGeometry, ConeGeometry]


@dataclass
class Request:
    kind: str                      # "fbp", "sirt" or "cgls"
    geom: Geom
    sinogram: torch.Tensor         # host (pinned for overlap) or device
    iters: int = 20
    filter_name: str = "ram-lak"
    t_submit: float = field(default=0.0, compare=False)


def _geom_key(g: Geom) -> str:
    h = hashlib.sha1()
    h.update(type(g).__name__.encode())
    for name in ("vol_shape", "vol_spacing", "vol_offset", "det_shape", "det_spacing",
                 "det_offset", "det_rotation", "angles", "DSO", "DSD", "COR", "vecs"):
        v = getattr(g, name, None)
        if v is not None:
            h.update(name.encode())
            h.update(np.ascontiguousarray(np.asarray(v, np.float64)).tobytes())
    return h.hexdigest()


def _clone_geom(g: Geom, device: int) -> Geom:
    """A private geometry object (own plan and scratch) for one slot."""
    if isinstance(g, FanVecGeometry):
        return FanVecGeometry(g.vol_shape, g.det_shape, g.vecs, vol_spacing=g.vol_spacing,
                              vol_offset=g.vol_offset, device=device)
    if isinstance(g, FanGeometry):
        return FanGeometry(DSD=g.DSD, DSO=g.DSO, angles=g.angles, vol_shape=g.vol_shape,
                           det_shape=g.det_shape, det_spacing=g.det_spacing,
                           det_offset=g.det_offset, det_rotation=g.det_rotation,
                           vol_spacing=g.vol_spacing, vol_offset=g.vol_offset, device=device)
    return ConeGeometry(DSD=g.DSD, DSO=g.DSO, angles=g.angles, vol_shape=g.vol_shape,
                        det_shape=g.det_shape, det_spacing=g.det_spacing,
                        det_offset=g.det_offset, det_rotation=g.det_rotation,
                        vol_spacing=g.vol_spacing, vol_offset=g.vol_offset, COR=g.COR,
                        device=device)


def _numel(shape) -> int:
    return int(np.prod([int(v) for v in shape]))


def request_bytes(req: Request) -> int:
    """Device bytes a request holds while in flight (inputs, outputs, plan
    scratch and iterates), an upper estimate."""
    g = req.geom
    nv, ns = _numel(g.vol_shape), _numel(g.sinogram_shape())
    plan = 2 * 8 * _numel([int(v) + 4 for v in g.vol_shape]) + 16 * ns + 4 * nv
    work = {"fbp": 2 * ns + nv, "sirt": 3 * nv + 3 * ns, "cgls": 3 * nv + 2 * ns}[req.kind]
    return 4 * (ns + nv + work) + plan


class _Slot:
    def __init__(self, device: torch.device, max_resident: int):
        self.stream = torch.cuda.Stream(device)
        self.device = device
        self.resident: "collections.OrderedDict[tuple, object]" = collections.OrderedDict()
        self.max_resident = max_resident

    def resource(self, kind: str, geom: Geom):
        key = (kind, _geom_key(geom))
        r = self.resident.get(key)
        if r is None:
            g = _clone_geom(geom, self.device.index or 0)
            if kind == "sirt":
                r = (g, SirtSolver(g, self.device, graph=True))
            elif kind == "cgls":
                r = (g, CglsSolver(g, self.device, graph=True))
            else:
                r = (g, None)
            self.resident[key] = r
            while len(self.resident) > self.max_resident:
                self.resident.popitem(last=False)
        else:
            self.resident.move_to_end(key)
        return r


def _execute(slot: _Slot, req: Request) -> torch.Tensor:
    """Enqueues the request on the slot's stream; returns the device result."""
    g, solver = slot.resource(req.kind, req.geom)
    y = req.sinogram.to(slot.device, non_blocking=True)
    if req.kind == "fbp":
        return fbp(y, g, req.filter_name)
    return solver.run(y, req.iters)


def solve_alone(req: Request, device=0) -> torch.Tensor:
    """The request's result computed on its own (the reference point of the
    'same alone and in the mix' check)."""
    dev = torch.device("cuda", device)
    slot = _Slot(dev, 1)
    with torch.cuda.stream(slot.stream):
        out = _execute(slot, req).clone()
    slot.stream.synchronize()
    return out


class Server:
    def __init__(self, device: int = 0, slots: int = 8, hbm_budget: float = 150e9,
                 max_resident: int = 16):
        self.device = torch.device("cuda", device)
        torch.cuda.init()
        self.slots = [_Slot(self.device, max_resident) for _ in range(slots)]
        self.free = list(range(slots))
        self.budget = float(hbm_budget)
        self.inflight_bytes = 0
        self._pending: "collections.deque[tuple]" = collections.deque()
        self._inflight: List[tuple] = []
        self._cv = threading.Condition()
        self._stop = False
        self.latencies: List[float] = []
        self.completed = 0
        self.t_first: Optional[float] = None
        self.t_last: Optional[float] = None
        self._thread = threading.Thread(target=self._loop, daemon=True)
        self._thread.start()

    # --------------------------------------------------------- client side
    def submit(self, req: Request) -> Future:
        fut: Future = Future()
        req.t_submit = time.perf_counter()
        with self._cv:
            if self._stop:
                raise RuntimeError("server is closed")
            self._pending.append((req, fut))
            self._cv.notify()
        return fut

    def close(self, wait: bool = True):
        with self._cv:
            self._stop = True
            self._cv.notify()
        if wait:
            self._thread.join()

    def stats(self) -> Dict[str, float]:
        lat = np.asarray(self.latencies) if self.latencies else np.zeros(1)
        span = (self.t_last - self.t_first) if self.completed > 1 else float("nan")
        return {"completed": self.completed, "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "solves_per_s": (self.completed / span) if span and span > 0 else float("nan")}

    # ---------------------------------------------------------- GPU thread
    def _next(self):
        """The next request that fits a free slot and the memory budget, or
        None; the queue is served in arrival order."""
        with self._cv:
            if not self._pending or not self.free:
                return None
            req, fut = self._pending[0]
            need = request_bytes(req)
            if self._inflight and self.inflight_bytes + need > self.budget:
                return None
            if self._inflight and torch.cuda.mem_get_info(self.device)[0] < need:
                return None
            self._pending.popleft()
            return req, fut, need

    def _admit(self) -> bool:
        progressed = False
        while True:
            nxt = self._next()
            if nxt is None:
                break
            req, fut, need = nxt
            k = self.free.pop()
            slot = self.slots[k]
            try:
                with torch.cuda.stream(slot.stream):
                    out = _execute(slot, req)
                    host = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
                    host.copy_(out, non_blocking=True)
                    ev = torch.cuda.Event()
                    ev.record(slot.stream)
            except Exception as e:  # a bad request fails alone
                self.free.append(k)
                fut.set_exception(e)
                continue
            self.inflight_bytes += need
            self._inflight.append((req, fut, k, ev, host, need))
            progressed = True
        return progressed

    def _poll(self) -> bool:
        progressed = False
        still = []
        for item in self._inflight:
            req, fut, k, ev, host, need = item
            if ev.query():
                now = time.perf_counter()
                self.free.append(k)
                self.inflight_bytes -= need
                self.latencies.append(now - req.t_submit)
                self.completed += 1
                if self.t_first is None:
                    self.t_first = req.t_submit
                self.t_last = now
                fut.set_result(host)
                progressed = True
            else:
                still.append(item)
        self._inflight = still
        return progressed

    def _loop(self):
        torch.cuda.set_device(self.device)
        while True:
            with self._cv:
                if self._stop and not self._pending and not self._inflight:
                    return
                if not self._pending and not self._inflight:
                    self._cv.wait(timeout=0.05)
                    continue
            admitted = self._admit()
            polled = self._poll()
            if not admitted and not polled:
                time.sleep(50e-6)
