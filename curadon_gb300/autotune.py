"""Per-geometry-class autotuning of the 2D operators' algorithm and kernel shape.

The reference has one kernel per direction (forward_2d.hpp:21-79,
backward_2d.hpp:21-100); this library compiles several algorithms and, for
the shared-memory ones, several kernel shapes (``plan_2d.set_shapes``). A new
plan starts at a rule measured on the n-sweep (``cg_plan2d_create``); the
tuner instead times the candidates on the plan's own geometry and keeps the
fastest. Every candidate is a parity-tested variant computing the
reference's samples and weights, so tuning changes speed, not results beyond
FP32 rounding (the texture-unit candidates filter with the reference's
8-bit weights).

Results are cached per geometry class: the plan kind (circular / vector),
volume shape, detector cells, view count and device. ``tune`` applies the
cached choice to another plan of the same class without timing again.
"""
from __future__ import annotations

import statistics

import torch

from . import backend
from ._lib import CuradonError

# (algorithm name, kernel shape or None); shapes are compiled chunk shapes of
# the chunked forward and variants of the staged backprojector
FORWARD_CANDIDATES = (("texture", None), ("chunked", 484), ("chunked", 474),
                      ("chunked", 443))
BACKWARD_CANDIDATES = (("shared", 68), ("shared", 48), ("shared", 27), ("texture", None))

_cache: dict[tuple, dict] = {}


def geometry_class(plan) -> tuple:
    """Key of the plan's geometry class."""
    vec = isinstance(plan, backend.plan_2d_vec)
    return ("fan-vec" if vec else "fan", tuple(int(v) for v in plan.vol_shape),
            int(plan.det_count), int(plan.nangles), int(plan.device_id))


def clear_cache() -> None:
    _cache.clear()


def _time(fn, reps: int, warmup: int) -> float:
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    ts = []
    for _ in range(reps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts)


def _apply(plan, choice: dict) -> None:
    (fname, fshape), (bname, bshape) = choice["forward"], choice["backward"]
    plan.set_algorithm(forward=fname, backward=bname)
    plan.set_shapes(forward=fshape, backward=bshape)


def tune(geom, reps: int = 5, warmup: int = 2, use_cache: bool = True) -> dict:
    """Times the forward and backprojection candidates on ``geom``'s plan
    (a FanGeometry or FanVecGeometry, or a plan_2d) with synthetic data of
    its shapes, applies the fastest of each to the plan and returns
    ``{"forward": (name, shape), "backward": (name, shape), "ms": {...}}``
    (``ms`` maps every timed candidate to its median time in milliseconds).
    Candidates the plan refuses (e.g. the texture backprojection of a vector
    geometry) are skipped."""
    plan = geom if isinstance(geom, backend.plan_2d) else geom.plan
    key = geometry_class(plan)
    if use_cache and key in _cache:
        _apply(plan, _cache[key])
        return _cache[key]

    from .phantom import ellipses_2d

    H, W = (int(v) for v in plan.vol_shape)
    dev = torch.device("cuda", int(plan.device_id))
    n = max(H, W)
    x = torch.zeros(H, W, device=dev)
    ph = ellipses_2d(n, 0, device=dev)
    x.copy_(ph[:H, :W])
    sino = torch.zeros(int(plan.nangles), int(plan.det_count), device=dev)
    vol = torch.zeros_like(x)
    prev_alg, prev_shapes = plan.algorithm, plan.shapes
    ms: dict[str, float] = {}
    try:
        best_f, best_b = None, None
        for name, shape in FORWARD_CANDIDATES:
            try:
                plan.set_algorithm(forward=name)
                if shape is not None:
                    plan.set_shapes(forward=shape)
            except (CuradonError, ValueError):
                continue
            t = _time(lambda: backend.forward_2d(x, sino, plan), reps, warmup)
            ms[f"forward {name}{'' if shape is None else f' {shape}'}"] = t
            if best_f is None or t < best_f[0]:
                best_f = (t, name, shape)
        plan.set_algorithm(forward=best_f[1])
        if best_f[2] is not None:
            plan.set_shapes(forward=best_f[2])
        backend.forward_2d(x, sino, plan)
        for name, shape in BACKWARD_CANDIDATES:
            try:
                plan.set_algorithm(backward=name)
                if shape is not None:
                    plan.set_shapes(backward=shape)
            except (CuradonError, ValueError):
                continue
            t = _time(lambda: backend.backward_2d(vol, sino, plan), reps, warmup)
            ms[f"backward {name}{'' if shape is None else f' {shape}'}"] = t
            if best_b is None or t < best_b[0]:
                best_b = (t, name, shape)
    except BaseException:
        plan.set_algorithm(forward=prev_alg[0], backward=prev_alg[1])
        plan.set_shapes(forward=prev_shapes[0], backward=prev_shapes[1])
        raise
    choice = {"forward": (best_f[1], best_f[2] if best_f[2] is not None else prev_shapes[0]),
              "backward": (best_b[1], best_b[2] if best_b[2] is not None else prev_shapes[1]),
              "ms": ms}
    _apply(plan, choice)
    _cache[key] = choice
    return choice
