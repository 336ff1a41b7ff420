"""Seeded synthetic phantoms and geometries for the benchmark workloads.

No public dataset is involved: the reference benchmarks on a Shepp-Logan
phantom (benchmark/bench_curadon_2d.py); these seeded ellipse / ellipsoid
phantoms stand in for it with the shapes and value ranges of the workloads:

* ``ellipses_2d(n, seed)``: 10 ellipses, centres U[-24,24]^2, semi-axes
  U[3,20], rotation U[0,pi), additive value U[0,1], clipped to [0,2]; all
  lengths scaled by n/64 (pixel units, image centred on the origin).
* ``ellipsoids_3d(n, seed)``: 20 ellipsoids, centres within 0.7 of the
  half-extent, semi-axes U[0.05,0.4] of the extent, random rotations,
  values U[0,1] (additive), clipped to [0,2].

Parameters are drawn with numpy's ``default_rng(seed)``; the images are
evaluated with torch on the requested device.
"""
from __future__ import annotations

import math

import numpy as np
import torch

__all__ = ["ellipses_2d", "ellipsoids_3d", "fan_config", "cone_config", "seed_for"]


def seed_for(config: int, problem: int = 0) -> int:
    return 1000 * config + problem


def ellipses_2d(n: int, seed: int, device="cpu", count: int = 10) -> torch.Tensor:
    rng = np.random.default_rng(seed)
    s = n / 64.0
    cx, cy = rng.uniform(-24, 24, count) * s, rng.uniform(-24, 24, count) * s
    ax, ay = rng.uniform(3, 20, count) * s, rng.uniform(3, 20, count) * s
    rot = rng.uniform(0, math.pi, count)
    val = rng.uniform(0, 1, count)
    c = torch.arange(n, device=device, dtype=torch.float64) - n / 2 + 0.5
    Y, X = torch.meshgrid(c, c, indexing="ij")
    img = torch.zeros((n, n), device=device, dtype=torch.float64)
    for k in range(count):
        co, si = math.cos(rot[k]), math.sin(rot[k])
        xr = (X - cx[k]) * co + (Y - cy[k]) * si
        yr = -(X - cx[k]) * si + (Y - cy[k]) * co
        img += val[k] * ((xr / ax[k]) ** 2 + (yr / ay[k]) ** 2 <= 1.0)
    return img.clamp_(0, 2).to(torch.float32)


def _rotation(rng) -> np.ndarray:
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def ellipsoids_3d(n, seed: int, device="cpu", count: int = 20) -> torch.Tensor:
    """(Z, Y, X) phantom; ``n`` is an int (cube) or a (Z, Y, X) tuple."""
    shape = (n, n, n) if isinstance(n, int) else tuple(int(v) for v in n)
    rng = np.random.default_rng(seed)
    ext = np.array(shape[::-1], dtype=np.float64)  # (X, Y, Z) extents
    half = ext / 2
    params = []
    for _ in range(count):
        c = rng.uniform(-0.7, 0.7, 3) * half
        a = rng.uniform(0.05, 0.4, 3) * ext
        R = _rotation(rng)
        v = rng.uniform(0, 1)
        params.append((c, a, R, v))
    Z, Y, X = shape
    out = torch.zeros(shape, device=device, dtype=torch.float32)
    xs = torch.arange(X, device=device, dtype=torch.float32) - X / 2 + 0.5
    ys = torch.arange(Y, device=device, dtype=torch.float32) - Y / 2 + 0.5
    zs_all = torch.arange(Z, device=device, dtype=torch.float32) - Z / 2 + 0.5
    slab = max(1, (1 << 24) // max(1, X * Y))
    for z0 in range(0, Z, slab):
        zs = zs_all[z0:z0 + slab]
        G = torch.stack(torch.meshgrid(zs, ys, xs, indexing="ij"), dim=-1)  # (z,y,x,[z,y,x])
        P = G[..., [2, 1, 0]]  # (x, y, z)
        acc = torch.zeros(G.shape[:3], device=device, dtype=torch.float32)
        for c, a, R, v in params:
            d = P - torch.tensor(c, device=device, dtype=torch.float32)
            q = d @ torch.tensor(R, device=device, dtype=torch.float32)
            r = ((q / torch.tensor(a, device=device, dtype=torch.float32)) ** 2).sum(-1)
            acc += float(v) * (r <= 1.0)
        out[z0:z0 + slab] = acc.clamp_(0, 2)
    return out


def fan_config(n: int, nangles: int | None = None, det: int | None = None,
               det_spacing: float = 1.5, DSO: float | None = None, DSD: float | None = None):
    """Keyword arguments of ``FanGeometry`` for an n x n fan-beam problem.

    Defaults are the n-sweep workload: det = ceil(sqrt(2) n) cells of 1.5,
    n views over [0, 2 pi), source-isocentre 2n, isocentre-detector n, per-view
    DSO/DSD arrays.  The 64 x 64 case with 360 views, DSO 256, DSD 384 and
    91 cells is ``fan_config(64, 360, 91, 1.5, 256, 384)``."""
    nangles = n if nangles is None else nangles
    det = int(math.ceil(math.sqrt(2) * n)) if det is None else det
    DSO = 2.0 * n if DSO is None else DSO
    DSD = DSO + n if DSD is None else DSD
    angles = np.linspace(0, 2 * np.pi, nangles, endpoint=False).astype(np.float32)
    return dict(DSD=np.full(nangles, DSD, np.float32), DSO=np.full(nangles, DSO, np.float32),
                angles=angles, vol_shape=(n, n), det_shape=det, det_spacing=det_spacing)


def cone_config(n: int, nangles: int, det: int, det_spacing: float = 1.5):
    """Keyword arguments of ``ConeGeometry`` for the circular cone-beam
    workload: n^3 volume, ``nangles`` over [0, 2 pi) as phi, det x det cells
    of ``det_spacing``, source-isocentre 2n, isocentre-detector n."""
    angles = np.linspace(0, 2 * np.pi, nangles, endpoint=False).astype(np.float32)
    return dict(DSD=3.0 * n, DSO=2.0 * n, angles=angles, vol_shape=(n, n, n),
                det_shape=(det, det), det_spacing=(det_spacing, det_spacing))
