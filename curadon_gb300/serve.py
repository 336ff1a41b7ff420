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

2D FBP and SIRT requests below 704^2 pixels are coalesced: requests of one
geometry and kind that wait together run as one batch on a resident
``Batch2d`` of that geometry class (built only when two requests of the
class wait together, reused while it stays resident; up to ``batch_slots`` problems, one
filter launch and one batched backprojection for FBP; for SIRT each
iteration is one batched forward, one batched backprojection and three
elementwise launches over all of them, captured once per batch size as a
CUDA graph and replayed).  Batched results equal the single-request path bit
for bit (the same kernels per problem).

3D requests, each of which fills the GPU for a long time, may hold at most
``heavy_slots`` slots (default half), so that 2D requests queued behind them
keep being admitted, and 2D requests run on high-priority streams, so that
their blocks start ahead of the 3D requests' as SMs free up.  Latencies
(submission to result on the host) and throughput are kept for ``stats()``
(p50 / p99 latency, also per kind; solves per second).
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
    def __init__(self, device: torch.device, max_resident: int, retire=None):
        self.stream = torch.cuda.Stream(device)
        # 2D requests run on a high-priority stream: when a 3D request's long
        # kernels occupy the GPU, the block scheduler starts the 2D blocks as
        # SMs free up instead of queueing them behind the 3D work
        lo, hi = torch.cuda.Stream.priority_range()
        self.stream_hi = torch.cuda.Stream(device, priority=min(lo, hi))
        self.device = device
        self.resident: "collections.OrderedDict[tuple, object]" = collections.OrderedDict()
        self.max_resident = max_resident
        # receives the resources the LRU evicts (None: dropped at once)
        self.retire = retire

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
                old = self.resident.popitem(last=False)[1]
                if self.retire is not None:
                    self.retire(old)
        else:
            self.resident.move_to_end(key)
        return r


# 2D requests below this many pixels are coalesced into class batches (the
# texture-unit forward's range, where single launches leave SMs idle)
BATCH_PIXELS = 704 * 704


def _batchable(req: Request) -> bool:
    g = req.geom
    return (req.kind in ("fbp", "sirt") and isinstance(g, FanGeometry)
            and int(g.vol_shape[0]) * int(g.vol_shape[1]) < BATCH_PIXELS)


def _heavy(req: Request) -> bool:
    """3D requests: each fills the GPU on its own for a long time."""
    return isinstance(req.geom, ConeGeometry)


def _class_key(req: Request) -> tuple:
    return (req.kind, req.iters if req.kind == "sirt" else 0, req.filter_name,
            _geom_key(req.geom))


class _ClassBatch:
    """``capacity`` resident problems of one 2D geometry and one kind: a
    private plan per problem, stacked device buffers and bound batches.
    ``run(ys, stream)`` solves len(ys) <= capacity requests at once."""

    def __init__(self, req: Request, device: torch.device, capacity: int, lam: float = 1.0):
        from .batch import Batch2d
        from .fbp import _device_kernel

        self.kind, self.iters, self.filter_name = req.kind, int(req.iters), req.filter_name
        self.device, self.capacity = device, int(capacity)
        self.busy = False
        K = self.capacity
        g0 = req.geom
        self.geoms = [_clone_geom(g0, device.index or 0) for _ in range(K)]
        H, W = (int(v) for v in g0.vol_shape)
        V, D = g0.sinogram_shape()
        self.nangles = V
        self.Y = torch.zeros((K, V, D), device=device)
        self.S = torch.zeros_like(self.Y)
        self.X = torch.zeros((K, H, W), device=device)
        if self.kind == "fbp":
            self.h = _device_kernel(D, self.filter_name, 1.0, device)
            self.bb = Batch2d(self.geoms, list(self.X), list(self.S))
        else:
            self.BP = torch.zeros_like(self.X)
            self.bf = Batch2d(self.geoms, list(self.X), list(self.S), forward="texture")
            self.bb = Batch2d(self.geoms, list(self.BP), list(self.S))
            # SIRT row / column normalisations, the same for every problem
            solver = SirtSolver(self.geoms[0], device, lam=lam)
            self.R, self.C = solver.R, solver.C
            self.graphs: Dict[int, torch.cuda.CUDAGraph] = {}
        # stacked buffers plus each problem's plan scratch, as admission counts it
        self.bytes = self.capacity * request_bytes(req)

    def _sirt_iteration(self, m: int):
        X, S, BP = self.X[:m], self.S[:m], self.BP[:m]
        self.bf.forward()
        torch.sub(self.Y[:m], S, out=S)
        S.mul_(self.R)
        BP.zero_()
        self.bb.backward()
        X.addcmul_(self.C, BP)
        X.clamp_(min=0.0)

    def run(self, ys: List[torch.Tensor], stream) -> torch.Tensor:
        """Enqueues the solves of ``ys`` (host or device sinograms) on the
        current stream; returns the stacked device results (a view)."""
        from .fbp import filter_sinogram

        m = len(ys)
        for i, y in enumerate(ys):
            self.Y[i].copy_(y, non_blocking=True)
        if self.kind == "fbp":
            filter_sinogram(self.Y[:m], self.filter_name, 1.0, np.pi / (2 * self.nangles),
                            out=self.S[:m])
            self.X[:m].zero_()
            self.bb.set_active(m)
            self.bb.backward()
            return self.X[:m]
        self.bf.set_active(m)
        self.bb.set_active(m)
        self.X[:m].zero_()
        g = self.graphs.get(m)
        if g is None:
            # one iteration captured on this stream without a device-wide
            # synchronisation (other requests keep running meanwhile)
            g = torch.cuda.CUDAGraph()
            g.capture_begin(capture_error_mode="thread_local")
            try:
                self._sirt_iteration(m)
            finally:
                g.capture_end()
            self.graphs[m] = g
        for _ in range(self.iters):
            g.replay()
        return self.X[:m]


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
                 max_resident: int = 16, batching: bool = True, batch_slots: int = 16,
                 max_class_batches: int = 32, heavy_slots: Optional[int] = None):
        self.device = torch.device("cuda", device)
        torch.cuda.init()
        # 3D requests (each fills the GPU for a long time) may hold at most
        # heavy_slots of the slots at once, so the 2D requests behind them in
        # the queue keep flowing; default: half the slots
        self.heavy_slots = max(1, slots // 2) if heavy_slots is None else max(1, int(heavy_slots))
        self.heavy_inflight = 0
        self.batching = bool(batching)
        self.batch_slots = int(batch_slots)
        self.max_class_batches = int(max_class_batches)
        self._classes: "collections.OrderedDict[tuple, _ClassBatch]" = collections.OrderedDict()
        self.batches_run = 0
        # resources evicted from the slots' and the class batches' caches:
        # releasing a plan's device memory (cudaFree) synchronises the whole
        # device, which would stall this thread until every request in flight
        # finished, so they are released while nothing is in flight, or all
        # at once when retire_limit of them wait
        self._graveyard: List[object] = []
        self.retire_limit = 256
        self.slots = [_Slot(self.device, max_resident, self._graveyard.append)
                      for _ in range(slots)]
        self.free = list(range(slots))
        self.budget = float(hbm_budget)
        self.inflight_bytes = 0
        self._pending: "collections.deque[tuple]" = collections.deque()
        # waiting requests per class key (batchable requests only)
        self._waiting: "collections.Counter[tuple]" = collections.Counter()
        self._inflight: List[tuple] = []
        self._cv = threading.Condition()
        self._stop = False
        self.latencies: List[float] = []
        self.latencies_by_kind: Dict[str, List[float]] = {}
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
            # what admission needs to know about the request, worked out once
            # (the geometry key hashes the per-view arrays)
            meta = (_heavy(req), _class_key(req) if _batchable(req) else None,
                    request_bytes(req))
            self._pending.append((req, fut, meta))
            if meta[1] is not None:
                self._waiting[meta[1]] += 1
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
        by_kind = {k: {"p50_ms": float(np.percentile(v, 50) * 1e3),
                       "p99_ms": float(np.percentile(v, 99) * 1e3), "count": len(v)}
                   for k, v in self.latencies_by_kind.items() if v}
        return {"completed": self.completed, "p50_ms": float(np.percentile(lat, 50) * 1e3),
                "p99_ms": float(np.percentile(lat, 99) * 1e3),
                "solves_per_s": (self.completed / span) if span and span > 0 else float("nan"),
                "by_kind": by_kind}

    # ---------------------------------------------------------- GPU thread
    def _next(self):
        """The next work that fits a free slot and the memory budget, or None:
        the oldest waiting request, with -- when it is a batchable 2D request
        whose class batch is idle -- every later waiting request of its class,
        up to the batch's size and the budget.  Returns (items, need, class
        key or None) with items a list of (request, future)."""
        with self._cv:
            if not self._pending or not self.free:
                return None
            for idx, (req, fut, (heavy, ckey, need)) in enumerate(self._pending):
                if heavy and self.heavy_inflight >= self.heavy_slots:
                    continue  # its lane is full; lighter requests behind it may go
                key = ckey if self.batching else None
                cb = self._classes.get(key) if key is not None else None
                if cb is not None and cb.busy:
                    continue  # its class batch is in flight; later requests may go
                if self._inflight and self.inflight_bytes + need > self.budget:
                    return None
                if self._inflight and torch.cuda.mem_get_info(self.device)[0] < need:
                    return None
                if key is not None and cb is None:
                    # a new class batch holds `batch_slots` problems' buffers and
                    # plans for as long as it stays resident, and building it
                    # (a plan per problem) stalls this thread: it is built only
                    # when another request of the class waits too, and only
                    # with room for it in the budget; else the request runs on
                    # its own
                    extra = self.batch_slots * need
                    if (self._waiting[key] < 2 or
                            self.resident_bytes() + self.inflight_bytes + extra > self.budget):
                        key = None
                items = [(req, fut)]
                taken = [idx]
                if key is not None:
                    for j in range(idx + 1, len(self._pending)):
                        if len(items) >= self.batch_slots:
                            break
                        r2, f2, (_, k2, n2) = self._pending[j]
                        if k2 == key:
                            if self.inflight_bytes + need + n2 > self.budget:
                                break
                            items.append((r2, f2))
                            taken.append(j)
                            need += n2
                for j in reversed(taken):
                    ck = self._pending[j][2][1]
                    if ck is not None:
                        self._waiting[ck] -= 1
                        if self._waiting[ck] <= 0:
                            del self._waiting[ck]
                    del self._pending[j]
                return items, need, key
            return None

    def resident_bytes(self) -> int:
        """Device bytes held by the resident class batches (an estimate)."""
        return sum(cb.bytes for cb in self._classes.values())

    def _class_batch(self, key, req: Request) -> _ClassBatch:
        cb = self._classes.get(key)
        if cb is None:
            cb = _ClassBatch(req, self.device, self.batch_slots)
            self._classes[key] = cb
            while len(self._classes) > self.max_class_batches:
                old_key = next(k for k, v in self._classes.items() if not v.busy)
                self._graveyard.append(self._classes.pop(old_key))
        else:
            self._classes.move_to_end(key)
        return cb

    def _admit(self) -> bool:
        progressed = False
        while True:
            nxt = self._next()
            if nxt is None:
                break
            items, need, key = nxt
            k = self.free.pop()
            slot = self.slots[k]
            stream = slot.stream if _heavy(items[0][0]) else slot.stream_hi
            cb = None
            try:
                with torch.cuda.stream(stream):
                    if key is None:
                        outs = [_execute(slot, items[0][0])]
                    else:
                        cb = self._class_batch(key, items[0][0])
                        cb.busy = True
                        stacked = cb.run([r.sinogram for r, _ in items], stream)
                        outs = list(stacked)
                        self.batches_run += 1
                    hosts = []
                    for out in outs:
                        host = torch.empty(out.shape, dtype=out.dtype, pin_memory=True)
                        host.copy_(out, non_blocking=True)
                        hosts.append(host)
                    ev = torch.cuda.Event()
                    ev.record(stream)
            except Exception as e:  # a bad request fails alone (with its batch)
                self.free.append(k)
                if cb is not None:
                    cb.busy = False
                for _, fut in items:
                    fut.set_exception(e)
                continue
            self.inflight_bytes += need
            heavy = _heavy(items[0][0])
            self.heavy_inflight += heavy
            self._inflight.append((items, k, ev, hosts, need, cb, heavy))
            progressed = True
        return progressed

    def _poll(self) -> bool:
        progressed = False
        still = []
        for item in self._inflight:
            items, k, ev, hosts, need, cb, heavy = item
            if ev.query():
                now = time.perf_counter()
                self.free.append(k)
                self.inflight_bytes -= need
                self.heavy_inflight -= heavy
                if cb is not None:
                    cb.busy = False
                for (req, fut), host in zip(items, hosts):
                    self.latencies.append(now - req.t_submit)
                    self.latencies_by_kind.setdefault(req.kind, []).append(now - req.t_submit)
                    self.completed += 1
                    if self.t_first is None or req.t_submit < self.t_first:
                        self.t_first = req.t_submit
                    fut.set_result(host)
                self.t_last = now
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
                    self._graveyard.clear()
                    return
                if not self._pending and not self._inflight:
                    self._graveyard.clear()
                    self._cv.wait(timeout=0.05)
                    continue
            admitted = self._admit()
            polled = self._poll()
            if self._graveyard and (not self._inflight
                                    or len(self._graveyard) >= self.retire_limit):
                self._graveyard.clear()
            if not admitted and not polled:
                time.sleep(50e-6)
