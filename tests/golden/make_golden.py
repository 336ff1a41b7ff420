"""Generates the golden vectors in tests/golden/ from the reference's own CUDA
operators (run on a GPU machine after ``python oracle/build_ref.py``).

Each ``<case>.npz`` holds the inputs (seeded phantoms, geometry arrays) and
the reference's outputs for them:

  fan_cfg0   64x64, 360 views, det 91 x 1.5, DSO 256, DSD 384 (the CPU-runnable
             fan-beam workload): forward sinogram, backprojection into zeros,
             and the plan's per-view tables
  fan_var    96 x 48 volume, anisotropic spacing, volume and detector offsets,
             per-view jittered DSO/DSD, 97 irregular views (the image is a
             multiple of the reference backprojector's 32 x 8 thread block:
             in partial blocks it reads an uninitialised shared table)
  cone_small 36 x 40 x 32 volume, 24 views, 48 x 40 detector
  cone_rot   as cone_small with volume/detector offsets, detector
             roll/pitch/yaw, COR and full (phi, theta, psi) angles

The 3D forward leaves rays that miss the volume unwritten, so its output
buffer starts filled with -7; the 3D backprojection accumulates, so its
volume starts at 1.

Usage: python tests/golden/make_golden.py [outdir]
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import torch

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from curadon_gb300.phantom import ellipses_2d, ellipsoids_3d, fan_config  # noqa: E402


def fan_cases():
    g0 = fan_config(64, 360, 91, 1.5, 256.0, 384.0)
    g0["vol_spacing"], g0["vol_offset"], g0["det_offset"] = (1.0, 1.0), (0.0, 0.0), 0.0
    yield "fan_cfg0", g0, ellipses_2d(64, 0).numpy()

    rng = np.random.default_rng(7)
    n = 97
    angles = np.sort(rng.uniform(0, 2 * np.pi, n)).astype(np.float32)
    g1 = dict(angles=angles, DSO=(150 + rng.normal(0, 0.5, n)).astype(np.float32),
              DSD=(260 + rng.normal(0, 0.5, n)).astype(np.float32), vol_shape=(48, 96),
              vol_spacing=(0.8, 1.2), vol_offset=(3.0, -2.0), det_shape=120, det_spacing=1.3,
              det_offset=1.7)
    ph = ellipses_2d(96, 1).numpy()[24:72, :]
    yield "fan_var", g1, np.ascontiguousarray(ph)


def cone_cases():
    n = 24
    phi = np.linspace(0, 2 * np.pi, n, endpoint=False).astype(np.float32)
    g0 = dict(vol_shape=(32, 40, 36), vol_spacing=(1.0, 1.0, 1.0), vol_offset=(0.0, 0.0, 0.0),
              det_shape=(40, 48), det_spacing=(1.2, 1.5), det_offset=(0.0, 0.0),
              det_rotation=(0.0, 0.0, 0.0), angles=np.vstack([phi, 0 * phi, 0 * phi]),
              DSO=80.0, DSD=130.0, COR=0.0)
    yield "cone_small", g0, ellipsoids_3d((32, 40, 36), 2).numpy()

    rng = np.random.default_rng(11)
    ang = np.vstack([phi + rng.uniform(-0.05, 0.05, n), rng.uniform(-0.1, 0.1, n),
                     rng.uniform(-0.1, 0.1, n)]).astype(np.float32)
    g1 = dict(g0, vol_spacing=(1.1, 0.9, 1.0), vol_offset=(1.5, -2.0, 0.5),
              det_offset=(2.5, -1.5), det_rotation=(0.05, -0.03, 0.08), angles=ang, COR=1.5)
    yield "cone_rot", g1, ellipsoids_3d((32, 40, 36), 3).numpy()


def pack(g):
    out = {}
    for k, v in g.items():
        out["g_" + k] = np.asarray(v)
    return out


def main(outdir: Path):
    outdir.mkdir(parents=True, exist_ok=True)
    ref = oracle.RefOps()
    dev = torch.device("cuda:0")
    for name, g, vol in fan_cases():
        h, n = ref.plan2d(g)
        v = torch.from_numpy(vol).to(dev).contiguous()
        s = torch.zeros((n, int(g["det_shape"])), device=dev)
        ref.forward2d(h, v.data_ptr(), s.data_ptr())
        ref.sync()
        b = torch.zeros_like(v)
        ref.backward2d(h, b.data_ptr(), s.data_ptr())
        ref.sync()
        src, u0, du = ref.plan2d_tables(h, n)
        ref.destroy2d(h)
        np.savez_compressed(outdir / f"{name}.npz", volume=vol, sino_ref=s.cpu().numpy(),
                            bwd_ref=b.cpu().numpy(), sources=src, u_origins=u0, delta_us=du,
                            **pack(g))
        print(name, "ok", float(s.abs().max()), float(b.abs().max()))
    for name, g, vol in cone_cases():
        v = torch.from_numpy(vol).to(dev).contiguous()
        n = np.asarray(g["angles"]).shape[-1]
        V, U = g["det_shape"]
        s = torch.full((n, V, U), -7.0, device=dev)
        ref.forward3d(g, v.data_ptr(), s.data_ptr())
        ref.sync()
        # backproject the reference's own sinogram (misses set to 0) into ones
        s_in = torch.where(s == -7.0, torch.zeros_like(s), s).contiguous()
        b = torch.ones_like(v)
        ref.backward3d(g, b.data_ptr(), s_in.data_ptr())
        ref.sync()
        np.savez_compressed(outdir / f"{name}.npz", volume=vol, sino_ref=s.cpu().numpy(),
                            bwd_in=s_in.cpu().numpy(), bwd_ref=b.cpu().numpy(), **pack(g))
        print(name, "ok", float(s.abs().max()), float(b.abs().max()))


if __name__ == "__main__":
    main(Path(sys.argv[1]) if len(sys.argv) > 1 else Path(__file__).resolve().parent)
