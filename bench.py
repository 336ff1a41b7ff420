#!/usr/bin/env python
"""Benchmark of the projection operators (one JSON line on rank 0).

A step is one forward projection plus one backprojection of the workload
(default: the 2D fan-beam n=2048 problem of the n-sweep: 2048 x 2048 image,
2048 views over [0, 2 pi), 2897 cells of 1.5, source-isocentre 4096,
isocentre-detector 2048, seeded 10-ellipse phantom).  ``value`` = operator
calls per second over all ranks (2 per step), inputs resident in HBM;
``e2e`` = the same through the public API with the volume copied in from
pinned host memory and both results copied back every step.

L2 is flushed (a 512 MiB write) between timed steps, outside the per-step
CUDA events.  Multi-GPU runs are independent replicas (the operators do not
exchange data), so scaling is weak.

--impl reference     the reference has no CPU path; its operators restated
                     by the FP64 oracle on the host cores (all threads), each
                     step a bounded sample of views scaled to full operators
--impl reference-gpu the reference's own CUDA operators (oracle/_ref shim),
                     timed like its benchmark: wall clock with a device sync
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

import numpy as np  # noqa: E402

# Main kernel of each operator by the plan's algorithm name.
KERNELS = {
    ("fan", "forward", "texture"): "k_fwd2d_tex", ("fan", "forward", "chunked"): "k_fwd2d_cslab",
    ("fan", "forward", "registers"): "k_fwd2d", ("fan", "backward", "shared"): "k_bwd2d_smem",
    ("fan", "backward", "registers"): "k_bwd2d", ("fan", "backward", "texture"): "k_bwd2d_tex",
    ("fan", "backward", "shared, quarter-turn"): "k_bwd2d_sym",
    ("cone", "forward", "texture"): "k_fwd3d_tex3", ("cone", "forward", "registers"): "k_fwd3d",
    ("cone", "forward", "quad"): "k_fwd3d_quad", ("cone", "forward", "mixed"): "k_fwd3d_quad",
    ("cone", "backward", "registers"): "k_bwd3d", ("cone", "backward", "axial"): "k_bwd3d_ax",
}


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=50)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference", "reference-gpu"])
    p.add_argument("--workload", default="fan2048",
                   help="fan<n> (n-sweep: n x n, n views), cone256 / cone512, serve "
                        "(served reconstruction stream vs the plain loop), batch (64 "
                        "jittered problems, batched gradient descent vs the plain loop), "
                        "batch3d (the same on 24 cone-beam problems) or "
                        "sweep (the 2D n-sweep against the reference's CUDA operators)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--sweep-sizes", default="64,128,256,512,1024,2048",
                   help="image sizes of --workload sweep")
    p.add_argument("--cone-views", type=int, default=0,
                   help="views of the cone workloads (default: 360 at 256^3, 720 at 512^3)")
    p.add_argument("--serve-requests", type=int, default=400,
                   help="requests of --workload serve")
    p.add_argument("--serve-seconds", type=float, default=0.0,
                   help="with --workload serve: also a sustained pass of this many seconds of "
                        "arrivals at 0.7x the measured capacity (0: skip)")
    p.add_argument("--serve-rate", type=float, default=200.0,
                   help="Poisson arrival rate of --workload serve (per second)")
    p.add_argument("--no-reference-gpu", action="store_true",
                   help="skip the reference's own CUDA operators beside ours (default run)")
    p.add_argument("--batch-forward", default="plans", choices=["plans", "texture", "registers"],
                   help="forward algorithm of the batch workload")
    p.add_argument("--batch3d-sizes", default="48,64,96,128",
                   help="volume edges n (n^3 voxels) drawn for --workload batch3d")
    p.add_argument("--batch3d-count", type=int, default=24,
                   help="problems of --workload batch3d")
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="CPU work budget of the cpu_baseline sample")
    return p.parse_args()


# ------------------------------------------------------------ workloads

# view count of the cone workloads when --cone-views overrides it (smaller
# profiling captures of the same volume); 0 = the workload's own
CONE_VIEWS = 0


def workload(name: str):
    from curadon_gb300.phantom import cone_config, fan_config, seed_for

    if name.startswith("fan"):
        n = int(name[3:])
        g = fan_config(n)
        return dict(kind="fan", name=name, n=n, geom=g, seed=seed_for(1, 0),
                    desc=f"2D fan-beam n={n} forward+backprojection",
                    config={"workload": f"2D fan-beam n={n}: {n}x{n} image, {n} views over "
                                        f"[0,2pi), {g['det_shape']} cells x 1.5, DSO {2 * n}, "
                                        f"DSD {3 * n}; forward + backprojection",
                            "n": n, "views": n, "det": g["det_shape"]})
    if name in ("cone256", "cone512"):
        n = int(name[4:])
        nangles, det = (360, 384) if n == 256 else (720, 768)
        if CONE_VIEWS:
            nangles = CONE_VIEWS
        g = cone_config(n, nangles, det)
        return dict(kind="cone", name=name, n=n, geom=g, seed=seed_for(2, n),
                    desc=f"3D cone-beam {n}^3 forward+backprojection",
                    config={"workload": f"3D circular cone-beam {n}^3 volume, {nangles} views, "
                                        f"{det}x{det} cells x 1.5, DSO {2 * n}, DSD {3 * n}; "
                                        "forward + backprojection",
                            "n": n, "views": nangles, "det": det})
    raise SystemExit(f"unknown workload {name}")


def fan_sample_count(g) -> int:
    """Interpolated samples of one 2D forward (sum over rays of rint(max|rd|)),
    evaluated in float64 (unit spacing, zero offsets, as the workloads use)."""
    H, W = g["vol_shape"]
    det = g["det_shape"]
    ds = float(g.get("det_spacing", 1.0))
    a = np.asarray(g["angles"], np.float64)
    dso = np.asarray(g["DSO"], np.float64)
    dod = np.asarray(g["DSD"], np.float64) - dso
    c, s_ = np.cos(a), np.sin(a)
    swx, swy = dso * s_, dso * c
    p0x, p1x = -det * ds / 2 + 0.5 * ds, -det * ds / 2 + 1.5 * ds
    c0x, c0y = p0x * c - dod * s_ - swx, -p0x * s_ - dod * c - swy
    c1x, c1y = p1x * c - dod * s_ - swx, -p1x * s_ - dod * c - swy
    src = np.stack([swx + W / 2, swy + H / 2], 1)
    u0 = np.stack([c0x, c0y], 1)
    du = np.stack([c1x - c0x, c1y - c0y], 1)
    u = np.arange(det, dtype=np.float64)
    total = 0
    for i in range(src.shape[0]):
        dx = u0[i, 0] + u * du[i, 0]
        dy = u0[i, 1] + u * du[i, 1]
        with np.errstate(divide="ignore", invalid="ignore"):
            tmin = np.full(det, np.finfo(np.float32).tiny)
            tmax = np.full(det, np.finfo(np.float32).max, dtype=np.float64)
            for s, d, hi in ((src[i, 0], dx, W), (src[i, 1], dy, H)):
                t1, t2 = (-1 - s) / d, (hi - s) / d
                tmin = np.fmin(np.fmax(t1, tmin), np.fmax(t2, tmin))
                tmax = np.fmax(np.fmin(t1, tmax), np.fmin(t2, tmax))
        hit = tmin <= tmax - 1e-6
        m = np.maximum(np.abs(dx), np.abs(dy)) * (tmax - tmin)
        total += int(np.rint(m[hit]).sum())
    return total


def cone_sample_count(g, views: int = 8) -> int:
    """Interpolated samples of one 3D forward (sum over rays that hit of
    nsteps + 1, nsteps = ceil((tmax - tmin) ceil(|dir|))), evaluated in
    float64 on ``views`` views spread over the circular orbit and scaled to
    all views (every view of a circular orbit casts the same rays, rotated)."""
    Z, Y, X = (int(v) for v in g["vol_shape"])
    V, U = (int(v) for v in g["det_shape"])
    sv, su = (float(v) for v in g["det_spacing"])
    dso, dsd = float(g["DSO"]), float(g["DSD"])
    ang = np.asarray(g["angles"], np.float64)
    pick = ang[np.linspace(0, len(ang) - 1, min(views, len(ang))).astype(int)]
    u = -su * U / 2 + su * 0.5 + su * np.arange(U)
    v = -sv * V / 2 + sv * 0.5 + sv * np.arange(V)
    uu, vv = np.meshgrid(u, v)
    ext = np.array([X, Y, Z], np.float64)
    total = 0
    for phi in pick:
        c, s_ = np.cos(phi), np.sin(phi)
        # rotation about y (rotation.hpp:7-28 with theta = psi = 0)
        rot = lambda x, y, z: (x * c + z * s_, y, -x * s_ + z * c)  # noqa: E731
        src = np.array(rot(0.0, 0.0, -dso)) + ext / 2 - 0.5
        det = np.stack(rot(uu, vv, np.full_like(uu, dsd - dso)), 0) + (ext / 2 - 0.5)[:, None, None]
        d = det - src[:, None, None]
        ns = np.ceil(np.sqrt((d * d).sum(0)))
        tmin = np.full(uu.shape, np.finfo(np.float32).tiny)
        tmax = np.full(uu.shape, np.finfo(np.float32).max, np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            for k in range(3):
                t1, t2 = (-1.0 - src[k]) / d[k], (ext[k] + 1 - src[k]) / d[k]
                tmin = np.fmin(np.fmax(t1, tmin), np.fmax(t2, tmin))
                tmax = np.fmax(np.fmin(t1, tmax), np.fmin(t2, tmax))
        hit = tmin <= tmax
        total += int((np.ceil((tmax[hit] - tmin[hit]) * ns[hit]) + 1).sum())
    return int(round(total * len(ang) / len(pick)))


# ------------------------------------------------------------ clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            import tempfile

            self.path = tempfile.mktemp(suffix=".csv")
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-i", str(self.index), "-lms", "50"], stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows)}


# ------------------------------------------------------------ ranks

def reduce_max(values, world: int, device="cpu"):
    """Element-wise max of per-rank timings over all ranks (the replicas run
    independently; only their timings are exchanged)."""
    import torch

    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    if world > 1:
        import torch.distributed as dist

        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(v) for v in t.cpu()]


# ------------------------------------------------------------ ours

def kernels_per_step(wl, geom) -> int:
    """Kernels of this library launched by one forward + one backprojection
    with the plan's algorithms (texture-unit paths copy the input into a
    CUDA array with a memcpy, which is not a kernel)."""
    fwd, bwd = geom.plan.algorithm
    nv = len(wl["geom"]["angles"])
    if wl["kind"] == "fan":
        # forward: texture 1 (plus an array copy); others: re-layout + kernel
        f = 1 if fwd == "texture" else 2
        # backprojection: texture one per 2048 views; others: re-layout + kernel
        b = -(-nv // 2048) if bwd == "texture" else 2
        return f + b
    # forward: texture 1; registers: two re-layouts + kernel; quad, mixed: two
    # re-layouts + kernel (plus the texture array copy)
    f = 1 if fwd == "texture" else 3
    # backprojection: re-layout + one kernel (axial: one per 768 views)
    b = 1 + (-(-nv // 768) if bwd == "axial" else 1)
    return f + b


def make_problem(wl, dev, local_rank=0):
    """(geometry, volume, sinogram, backprojection buffer) of a workload on
    ``dev``, the volume a seeded phantom."""
    import torch

    import curadon_gb300 as cg
    from curadon_gb300.phantom import ellipses_2d, ellipsoids_3d

    g = wl["geom"]
    if wl["kind"] == "fan":
        geom = cg.FanGeometry(**g, device=local_rank)
        vol = ellipses_2d(wl["n"], wl["seed"], device=dev).contiguous()
    else:
        geom = cg.ConeGeometry(**g, device=local_rank)
        vol = ellipsoids_3d(wl["n"], wl["seed"], device=dev).contiguous()
    sino = torch.zeros(geom.sinogram_shape(), device=dev)
    return geom, vol, sino, torch.zeros_like(vol)


def time_steps(fwd, bwd, steps: int, warmup: int, flush, stream):
    """Per-step forward and backprojection times (ms, CUDA events on
    ``stream``, L2 flushed before each step outside the events)."""
    import torch

    for _ in range(warmup):
        fwd(), bwd()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(steps)]
    for k in range(steps):
        flush.zero_()
        e0, e1, e2 = ev[k]
        e0.record(stream)
        fwd()
        e1.record(stream)
        bwd()
        e2.record(stream)
    torch.cuda.synchronize()
    return ([ev[k][0].elapsed_time(ev[k][1]) for k in range(steps)],
            [ev[k][1].elapsed_time(ev[k][2]) for k in range(steps)])


def reference_ops():
    """The reference's own CUDA operators (the oracle/_ref shim over its
    header-only library, compiled for sm_103a), or (None, reason)."""
    try:
        import oracle
        from oracle import build_ref

        if build_ref.build() is None or not oracle.ref_available():
            return None, "reference headers not staged, shim not built"
        return oracle.RefOps(), ""
    except Exception as e:  # reported in the JSON line, never fatal
        return None, f"reference shim unavailable: {e}"


def time_reference_gpu(ref, wl, vol, steps: int, warmup: int, flush, stream):
    """Times the reference's operators on ``vol`` exactly as this library's
    are timed: CUDA events on ``stream`` around each call, L2 flushed before
    each step.  The reference's calls are synchronous and run on its own
    streams, so an event pair spans the whole call, its host-side set-up
    (texture arrays, geometry upload, synchronisations) included, as its
    users see it.  Returns per-step forward / backprojection ms and the
    sinogram it computed."""
    import torch

    g = wl["geom"]
    dev = vol.device
    if wl["kind"] == "fan":
        h, n = ref.plan2d(g)
        sino = torch.zeros((n, g["det_shape"]), device=dev)
        vbp = torch.zeros_like(vol)

        def fwd():
            ref.forward2d(h, vol.data_ptr(), sino.data_ptr())

        def bwd():
            vbp.zero_()
            ref.backward2d(h, vbp.data_ptr(), sino.data_ptr())
    else:
        h = None
        sino = torch.zeros((len(g["angles"]), *g["det_shape"]), device=dev)
        vbp = torch.zeros_like(vol)

        def fwd():
            ref.forward3d(g, vol.data_ptr(), sino.data_ptr())

        def bwd():
            vbp.zero_()
            ref.backward3d(g, vbp.data_ptr(), sino.data_ptr())
    try:
        tf, tb = time_steps(fwd, bwd, steps, warmup, flush, stream)
    finally:
        if h is not None:
            ref.destroy2d(h)
    return tf, tb, sino


def plan_algorithms(geom) -> dict:
    """The plan's algorithm names; a 2D staged backprojection that runs over
    the views' quarter-turn symmetry is named so."""
    algos = dict(zip(("forward", "backward"), geom.plan.algorithm))
    if algos["backward"] == "shared" and getattr(geom.plan, "quarter_turn", 0):
        algos["backward"] = "shared, quarter-turn"
    return algos


def roofline_of(wl, ms_fwd, ms_bwd, algos, peaks):
    """Roofline of the dominant operator: compulsory bytes per call over its
    event-timed duration against the measured HBM copy peak, with the
    interpolation rate and gather bandwidth beside it."""
    g = wl["geom"]
    if wl["kind"] == "fan":
        nvox = wl["n"] * wl["n"]
        nrays = len(g["angles"]) * g["det_shape"]
        s_fwd = fan_sample_count(g)
        gather = {"forward": 16, "backward": 8}
        note = ("gather-bound (L1 / shared-memory data path and issue), not HBM-bound: the "
                "compulsory bytes fit in L2; samples_per_s is the efficiency figure")
    else:
        nvox = wl["n"] ** 3
        nrays = len(g["angles"]) * g["det_shape"][0] * g["det_shape"][1]
        s_fwd = cone_sample_count(g)
        gather = {"forward": 32, "backward": 16}
        note = (f"gather-bound (L1 load and texture pipes), not HBM-bound: the {nvox * 4 >> 20} "
                "MiB volume's quad copies are re-read from L2 per sample; from 512^3 the "
                "resident blocks' working set exceeds L2 (89 % L2 hit) but DRAM runs at a few "
                "percent of its peak; samples_per_s is the efficiency figure")
    s_bwd = nvox * len(g["angles"])
    b_alg = {"forward": 4 * (nvox + nrays), "backward": 4 * (nrays + 2 * nvox)}
    dom = "forward" if ms_fwd >= ms_bwd else "backward"
    t_dom = (ms_fwd if dom == "forward" else ms_bwd) / 1e3
    kernel = KERNELS.get((wl["kind"], dom, algos[dom]), dom)
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    achieved = b_alg[dom] / t_dom / 1e9
    samples = s_fwd if dom == "forward" else s_bwd
    return {"bound": "hbm", "kernel": kernel, "operator": dom,
            "achieved": round(achieved, 3), "peak": peak, "peak_source": peak_src,
            "unit": "GB/s", "frac": achieved / peak,
            # DRAM bytes per launch come from an ncu capture of the same
            # kernel, kept with the profiles, not from this run
            "traffic": None, "algorithmic_bytes": b_alg[dom],
            "samples_per_s": samples / t_dom,
            "gather_GBps": samples * gather[dom] / t_dom / 1e9, "note": note}


def run_ours(args, rank, world, local_rank):
    import torch

    import curadon_gb300 as cg
    from curadon_gb300 import _build
    from curadon_gb300.backend import raise_on_wait_timeouts

    _build.build()
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    wl = workload(args.workload)
    geom, vol, sino, vbp = make_problem(wl, dev, local_rank)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    launches_per_step = kernels_per_step(wl, geom)

    def fwd():
        cg.forward(vol, sino, geom)

    def bwd():
        vbp.zero_()
        cg.backward(sino, vbp, geom)

    sampler = ClockSampler(local_rank) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.2)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    t_fwd, t_bwd = time_steps(fwd, bwd, args.steps, args.warmup, flush, stream)
    if world > 1:
        torch.distributed.barrier()
    total_ms = sum(t_fwd) + sum(t_bwd)

    # end to end: pinned host volume in, sinogram and backprojection out
    host_vol = torch.empty(vol.shape, dtype=torch.float32, pin_memory=True)
    host_vol.copy_(vol.cpu())
    host_sino = torch.empty(sino.shape, dtype=torch.float32, pin_memory=True)
    host_vbp = torch.empty(vol.shape, dtype=torch.float32, pin_memory=True)
    dvol = torch.empty_like(vol)
    h2d = host_vol.numel() * 4
    d2h = (host_sino.numel() + host_vbp.numel()) * 4

    def e2e_step():
        dvol.copy_(host_vol, non_blocking=True)
        cg.forward(dvol, sino, geom)
        vbp.zero_()
        cg.backward(sino, vbp, geom)
        host_sino.copy_(sino, non_blocking=True)
        host_vbp.copy_(vbp, non_blocking=True)

    for _ in range(args.warmup):
        e2e_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e_ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        e_ev[k][0].record(stream)
        e2e_step()
        e_ev[k][1].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    e2e_ms = sum(a.elapsed_time(b) for a, b in e_ev)
    clocks = sampler.stop() if sampler else None
    raise_on_wait_timeouts()

    total_ms, e2e_ms, fwd_ms, bwd_ms = reduce_max([total_ms, e2e_ms, sum(t_fwd), sum(t_bwd)],
                                                  world, dev)
    if rank != 0:
        return None

    ops = 2 * args.steps * world
    value = ops / (total_ms / 1e3)
    ms_fwd = fwd_ms / args.steps
    ms_bwd = bwd_ms / args.steps
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    algos = plan_algorithms(geom)

    line = {
        "metric": "fwd/bwd proj ops/s", "value": value, "unit": "ops/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipse phantom)",
        "config": dict(wl["config"], l2="flushed between timed steps (512 MiB write, outside "
                                          "the per-step events)", parallelism=f"replicas{world}"),
        "fwd_ops_s": args.steps * world / (fwd_ms / 1e3),
        "bwd_ops_s": args.steps * world / (bwd_ms / 1e3),
        "ms_forward": ms_fwd, "ms_backward": ms_bwd,
        "algorithms": algos,
        "e2e": {"value": ops / (e2e_ms / 1e3), "unit": "ops/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": roofline_of(wl, ms_fwd, ms_bwd, algos, peaks),
        "clocks": clocks,
    }
    if world == 1 and not args.no_reference_gpu:
        line.update(reference_gpu_comparison(args, wl, vol, sino, flush, stream, ms_fwd,
                                             ms_bwd))
        if wl["name"] != "cone512":
            line["cone512"] = cone512_comparison(args, dev, flush, stream)
    return line


def reference_gpu_comparison(args, wl, vol, sino, flush, stream, ms_fwd, ms_bwd):
    """The reference's own CUDA operators on the same workload, the same
    steps and the same clock (the drop-in comparison), and the relative L2
    distance between its sinogram and ours."""
    ref, why = reference_ops()
    if ref is None:
        return {"reference_gpu": {"unavailable": why}}
    tf, tb, s_ref = time_reference_gpu(ref, wl, vol, args.steps, args.warmup, flush, stream)
    rf, rb = sum(tf) / len(tf), sum(tb) / len(tb)
    rel = float((sino - s_ref).norm() / s_ref.norm())
    return {
        "reference_gpu": {"ms_forward": rf, "ms_backward": rb, "ms_per_step": rf + rb,
                          "ops_s": 2e3 / (rf + rb), "steps": args.steps,
                          "warmup": args.warmup,
                          "timing": "CUDA events around each synchronous reference call, "
                                    "L2 flushed before each step (as this library's)",
                          "forward_rel_l2_vs_ours": rel},
        "ref_gpu_ms_forward": rf, "ref_gpu_ms_backward": rb,
        "vs_ref_gpu": {"forward": rf / ms_fwd, "backward": rb / ms_bwd,
                       "step": (rf + rb) / (ms_fwd + ms_bwd)},
    }


def cone512_comparison(args, dev, flush, stream):
    """The 3D 512^3 workload (720 views, 768^2 cells): this library's default
    operators and the reference's, a few steps each, with the SM clock
    sampled meanwhile."""
    import torch

    import curadon_gb300 as cg
    from curadon_gb300.backend import raise_on_wait_timeouts

    wl = workload("cone512")
    steps, warmup = 5, 2
    sampler = ClockSampler(dev.index or 0)
    sampler.start()
    time.sleep(0.2)
    geom, vol, sino, vbp = make_problem(wl, dev, dev.index or 0)

    def fwd():
        cg.forward(vol, sino, geom)

    def bwd():
        vbp.zero_()
        cg.backward(sino, vbp, geom)

    tf, tb = time_steps(fwd, bwd, steps, warmup, flush, stream)
    raise_on_wait_timeouts()
    mf, mb = sum(tf) / steps, sum(tb) / steps
    algos = plan_algorithms(geom)
    out = {"workload": wl["config"]["workload"], "steps": steps, "warmup": warmup,
           "ms_forward": mf, "ms_backward": mb, "ms_per_step": mf + mb,
           "ops_s": 2e3 / (mf + mb), "algorithms": algos,
           "samples_per_s_forward": cone_sample_count(wl["geom"]) / (mf / 1e3)}
    ref, why = reference_ops()
    if ref is None:
        out["reference_gpu"] = {"unavailable": why}
    else:
        del geom  # the reference allocates its own arrays
        torch.cuda.empty_cache()
        rf_, rb_, s_ref = time_reference_gpu(ref, wl, vol, steps, warmup, flush, stream)
        rf, rb = sum(rf_) / steps, sum(rb_) / steps
        hit = s_ref != 0
        rel = float((sino[hit] - s_ref[hit]).norm() / s_ref[hit].norm())
        out["reference_gpu"] = {"ms_forward": rf, "ms_backward": rb, "ms_per_step": rf + rb,
                                "ops_s": 2e3 / (rf + rb), "forward_rel_l2_vs_ours": rel}
        out["vs_ref_gpu"] = {"forward": rf / mf, "backward": rb / mb,
                             "step": (rf + rb) / (mf + mb)}
    out["clocks"] = sampler.stop()
    return out


# ------------------------------------------------------------ CPU (oracle)

def _sub_geom(g, kind, views):
    h = dict(g)
    h["angles"] = np.asarray(g["angles"])[:views]
    if kind == "fan":
        h["DSO"] = np.asarray(g["DSO"])[:views]
        h["DSD"] = np.asarray(g["DSD"])[:views]
    return h


def cpu_sample(wl, budget_s: float, threads: int):
    """Times the oracle on the first v views of forward and backprojection,
    v sized to the budget, and scales to full operators.  Returns
    (ops_per_s, description)."""
    import oracle
    from curadon_gb300.phantom import ellipses_2d, ellipsoids_3d

    g = wl["geom"]
    kind = wl["kind"]
    nviews = len(g["angles"])
    if kind == "fan":
        vol = ellipses_2d(wl["n"], wl["seed"]).numpy()
        fwd, bwd = oracle.fwd2d, oracle.bwd2d
    else:
        vol = ellipsoids_3d(wl["n"], wl["seed"]).numpy()
        fwd, bwd = oracle.fwd3d, oracle.bwd3d

    def run(v):
        h = _sub_geom(g, kind, v)
        t0 = time.perf_counter()
        s = fwd(h, vol, nthreads=threads)
        t1 = time.perf_counter()
        bwd(h, s.astype(np.float32), nthreads=threads)
        t2 = time.perf_counter()
        return t1 - t0, t2 - t1

    tf1, tb1 = run(1)
    per_view = max(tf1 + tb1, 1e-4)
    v = int(max(1, min(nviews, budget_s / per_view)))
    tf, tb = run(v)
    full = (tf + tb) * nviews / v
    return 2.0 / full, (f"forward and backprojection over the first {v} of {nviews} views, "
                        f"FP64 oracle, scaled by {nviews}/{v}")


def run_reference_cpu(args, rank, world):
    """The reference has no CPU path: its operators as restated by the FP64
    oracle on all host cores.  Each timed step is one full forward and one
    full backprojection of the workload; warm-up steps run on an eighth of
    the views (they only warm the threads and caches)."""
    if rank != 0:
        return None
    import oracle
    from curadon_gb300.phantom import ellipses_2d, ellipsoids_3d

    wl = workload(args.workload)
    g = wl["geom"]
    kind = wl["kind"]
    threads = os.cpu_count() or 1
    if kind == "fan":
        vol = ellipses_2d(wl["n"], wl["seed"]).numpy()
        fwd, bwd = oracle.fwd2d, oracle.bwd2d
    else:
        vol = ellipsoids_3d(wl["n"], wl["seed"]).numpy()
        fwd, bwd = oracle.fwd3d, oracle.bwd3d
    nviews = len(g["angles"])
    warm = _sub_geom(g, kind, max(1, nviews // 8))
    for _ in range(args.warmup):
        bwd(warm, fwd(warm, vol, nthreads=threads).astype(np.float32), nthreads=threads)
    per_step = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        s = fwd(g, vol, nthreads=threads)
        bwd(g, s.astype(np.float32), nthreads=threads)
        per_step.append(time.perf_counter() - t0)
    total = sum(per_step)
    value = 2 * args.steps / total
    desc = (f"full forward + backprojection per step ({nviews} views), FP64 oracle, "
            f"{threads} threads (the reference has no CPU path; its operators restated)")
    return {
        "impl": "reference", "metric": "fwd/bwd proj ops/s", "value": value, "unit": "ops/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ellipse phantom)",
        "config": dict(wl["config"], parallelism="host cores"),
        "cpu_baseline": {"value": value, "unit": "ops/s", "cores": threads, "kind": "port",
                         "sample": desc},
        "e2e": {"value": value, "unit": "ops/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def run_reference_gpu(args, rank, world, local_rank):
    """The reference's own CUDA operators (the oracle/_ref shim) alone, with
    this library's clock: CUDA events around each synchronous call."""
    if rank != 0:
        return None
    import torch

    ref, why = reference_ops()
    if ref is None:
        return {"impl": "reference-gpu", "unavailable": why}
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    wl = workload(args.workload)
    from curadon_gb300.phantom import ellipses_2d, ellipsoids_3d

    vol = (ellipses_2d(wl["n"], wl["seed"], device=dev) if wl["kind"] == "fan"
           else ellipsoids_3d(wl["n"], wl["seed"], device=dev)).contiguous()
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    tf, tb, _ = time_reference_gpu(ref, wl, vol, args.steps, args.warmup, flush,
                                   torch.cuda.current_stream(dev))
    total = (sum(tf) + sum(tb)) / 1e3
    return {
        "impl": "reference-gpu", "metric": "fwd/bwd proj ops/s",
        "value": 2 * args.steps / total, "unit": "ops/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipse phantom)", "config": wl["config"],
        "fwd_ops_s": args.steps / (sum(tf) / 1e3), "bwd_ops_s": args.steps / (sum(tb) / 1e3),
        "ms_forward": sum(tf) / args.steps, "ms_backward": sum(tb) / args.steps,
        "timing": "CUDA events around each synchronous reference call, L2 flushed per step",
    }


# ------------------------------------------------------------ n-sweep

def run_sweep(args):
    """The 2D n-sweep against the reference's own CUDA operators: for n in
    64 .. 2048 (n x n image, n views, ceil(sqrt(2) n) cells of 1.5, DSO 2n,
    DSD 3n), forward and backprojection timed separately, 50 runs after 3
    warm-ups each (the reference benchmark's protocol, benchmark/bench.py:
    51-75), CUDA events around every call on both sides, L2 flushed before
    every call; relative L2 of our outputs against the reference's (the
    backprojection only up to 1024 views, above which the reference's chunks
    race)."""
    import torch

    import curadon_gb300 as cg
    from curadon_gb300 import _build
    from curadon_gb300.backend import raise_on_wait_timeouts

    _build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    ref, why = reference_ops()
    runs, warm = 50, 3

    def timed(fn):
        for _ in range(warm):
            fn()
        torch.cuda.synchronize()
        ts = []
        for _ in range(runs):
            flush.zero_()
            a_, b_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a_.record(stream)
            fn()
            b_.record(stream)
            b_.synchronize()
            ts.append(a_.elapsed_time(b_))
        return sum(ts) / len(ts)

    rows = []
    for n in [int(v) for v in args.sweep_sizes.split(",")]:
        wl = workload(f"fan{n}")
        geom, vol, sino, vbp = make_problem(wl, dev)
        row = {"n": n, "views": n, "det": wl["geom"]["det_shape"],
               "algorithms": plan_algorithms(geom)}
        row["ms_forward"] = timed(lambda: cg.forward(vol, sino, geom))
        row["ms_backward"] = timed(lambda: cg.backward(sino, vbp, geom))
        raise_on_wait_timeouts()
        if ref is not None:
            h, nv = ref.plan2d(wl["geom"])
            s_ref = torch.zeros_like(sino)
            b_ref = torch.zeros_like(vol)
            row["ref_ms_forward"] = timed(lambda: ref.forward2d(h, vol.data_ptr(),
                                                                s_ref.data_ptr()))
            row["ref_ms_backward"] = timed(lambda: ref.backward2d(h, b_ref.data_ptr(),
                                                                  s_ref.data_ptr()))
            cg.forward(vol, sino, geom)
            row["forward_rel_l2"] = float((sino - s_ref).norm() / s_ref.norm())
            if nv <= 1024:
                b_ref.zero_()
                ref.backward2d(h, b_ref.data_ptr(), s_ref.data_ptr())
                b = torch.zeros_like(vol)
                cg.backward(s_ref, b, geom)
                row["backward_rel_l2"] = float((b - b_ref).norm() / b_ref.norm())
            ref.destroy2d(h)
            row["vs_ref_forward"] = row["ref_ms_forward"] / row["ms_forward"]
            row["vs_ref_backward"] = row["ref_ms_backward"] / row["ms_backward"]
        rows.append(row)
        print(json.dumps(row), file=sys.stderr, flush=True)
        del geom, vol, sino, vbp
        torch.cuda.empty_cache()
    return {"metric": "fwd/bwd proj ops/s (n-sweep)", "unit": "ms per call",
            "protocol": f"{runs} runs after {warm} warm-ups per operator, CUDA events, L2 "
                        "flushed per call", "reference": why or "oracle/_ref shim (sm_103a)",
            "rows": rows}


# ------------------------------------------------------------ serving

def serve_requests(n_req: int, dev, seed: int = 4000, kinds=("fbp", "sirt", "cgls")):
    """A seeded request mix of the served stream: 70 % 2D FBP (n log-uniform
    over 128..2048, n views), 25 % 2D SIRT-20 (n log-uniform over
    128..1024), 5 % 3D CGLS-30 (128^3..256^3, 180..360 views, 1.5 n cells);
    sizes drawn from log-spaced sets so geometries repeat as in a clinic's
    protocols.  ``kinds`` keeps a sub-mix (the others are redrawn).
    Sinograms are projections of seeded phantoms, in pinned host memory."""
    import torch

    from curadon_gb300 import ConeGeometry, FanGeometry, forward
    from curadon_gb300.phantom import cone_config, ellipses_2d, ellipsoids_3d, fan_config
    from curadon_gb300.serve import Request

    rng = np.random.default_rng(seed)
    fbp_sizes = [128, 181, 256, 362, 512, 724, 1024, 1448, 2048]
    sirt_sizes = [128, 181, 256, 362, 512, 724, 1024]
    cone_sizes = [128, 160, 192, 224, 256]
    cone_views = [180, 270, 360]
    geoms, reqs = {}, []
    while len(reqs) < n_req:
        u = rng.random()
        if u < 0.70:
            kind, n, nv = "fbp", int(rng.choice(fbp_sizes)), 0
        elif u < 0.95:
            kind, n, nv = "sirt", int(rng.choice(sirt_sizes)), 0
        else:
            kind, n, nv = "cgls", int(rng.choice(cone_sizes)), int(rng.choice(cone_views))
        seed_k = int(rng.integers(1 << 30))
        if kind not in kinds:
            continue
        key = (kind == "cgls", n, nv)
        if key not in geoms:
            if kind == "cgls":
                geoms[key] = ConeGeometry(**cone_config(n, nv, int(1.5 * n)))
            else:
                geoms[key] = FanGeometry(**fan_config(n))
        g = geoms[key]
        ph = (ellipsoids_3d(n, seed_k, device=dev) if kind == "cgls"
              else ellipses_2d(n, seed_k, device=dev)).contiguous()
        y = torch.zeros(g.sinogram_shape(), device=dev)
        forward(ph, y, g)
        iters = {"fbp": 0, "sirt": 20, "cgls": 30}[kind]
        reqs.append(Request(kind, g, y.cpu().pin_memory(), iters=iters))
    torch.cuda.synchronize()
    return reqs


def _serve_pass(reqs, rate: float, seed: int = 7, batching: bool = True, count: int = 0):
    """Submits ``reqs`` (``count`` submissions cycling through them, default
    each once) with Poisson arrivals at ``rate`` per second to a new server
    (after a warm-up pass of residency) and returns its stats."""
    import threading

    from curadon_gb300.serve import Server

    srv = Server(device=0, slots=8, batching=batching)
    for f in [srv.submit(r) for r in reqs]:  # warm-up: slot and class-batch residency
        f.result()
    srv.latencies.clear()
    srv.latencies_by_kind.clear()
    srv.completed, srv.t_first, srv.t_last = 0, None, None
    rng = np.random.default_rng(seed)
    count = count or len(reqs)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, count))
    futs = []
    sampler = ClockSampler(0)
    sampler.start()

    def client():
        t_start = time.perf_counter()
        for k, ta in enumerate(arrivals):
            r = reqs[k % len(reqs)]
            delay = t_start + ta - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            futs.append(srv.submit(r))

    th = threading.Thread(target=client)
    th.start()
    th.join()
    for f in futs:
        f.result()
    batches = srv.batches_run
    srv.close()
    st = srv.stats()
    st["clocks"] = sampler.stop()
    st["batches"] = batches
    st["arrival_span_s"] = float(arrivals[-1])
    return st


def run_serve(args):
    """The served reconstruction stream: requests of the served mix at their
    specified sizes with Poisson arrivals at 200/s, solves/s and p50 / p99
    latency, against the plain loop (one request at a time, each solved and
    read back before the next); again at an arrival rate below capacity
    (latency without a growing queue); and the 2D part of the mix alone,
    where coalescing applies."""
    import torch

    from curadon_gb300 import _build
    from curadon_gb300.fbp import fbp
    from curadon_gb300.solvers import cgls, sirt

    _build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)

    def plain_rate(reqs):
        def plain(r):
            y = r.sinogram.to(dev)
            x = (fbp(y, r.geom) if r.kind == "fbp" else
                 sirt(r.geom, y, r.iters) if r.kind == "sirt" else cgls(r.geom, y, r.iters))
            return x.cpu()

        for r in reqs:  # warm-up: plans and filters of the plain path
            plain(r)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for r in reqs:
            plain(r)
        return len(reqs) / (time.perf_counter() - t0)

    n_req = args.serve_requests
    reqs = serve_requests(n_req, dev)
    kinds = {k: sum(r.kind == k for r in reqs) for k in ("fbp", "sirt", "cgls")}
    plain_all = plain_rate(reqs)
    served = _serve_pass(reqs, args.serve_rate)
    sub_rate = max(1.0, 0.7 * served["solves_per_s"])
    relaxed = _serve_pass(reqs, sub_rate, seed=8)
    # the 2D part alone (FBP and SIRT, coalesced into class batches), at an
    # arrival rate above its capacity so that solves/s measures the server
    reqs2d = serve_requests(n_req, dev, seed=4001, kinds=("fbp", "sirt"))
    plain_2d = plain_rate(reqs2d)
    rate_2d = 10 * args.serve_rate
    served_2d = _serve_pass(reqs2d, rate_2d)
    unbatched_2d = _serve_pass(reqs2d, rate_2d, batching=False)
    sustained = None
    if args.serve_seconds > 0:
        # the specified mix for serve_seconds of arrivals at 0.7x the capacity
        # measured above (the specified 200/s exceeds it)
        n_sub = int(sub_rate * args.serve_seconds)
        t0 = time.perf_counter()
        st = _serve_pass(reqs, sub_rate, seed=9, count=n_sub)
        sustained = {"rate_per_s": sub_rate, "requests": n_sub,
                     "arrival_span_s": st["arrival_span_s"],
                     "wall_s": time.perf_counter() - t0, "solves_per_s": st["solves_per_s"],
                     "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"], "batches": st["batches"],
                     "latency_by_kind": st["by_kind"], "clocks": st["clocks"]}
    line = {
        "metric": "served solves/s", "value": served["solves_per_s"], "unit": "solves/s",
        "n_gpus": 1, "steps": len(reqs), "warmup": len(reqs),
        "ms_per_step": 1e3 / served["solves_per_s"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded phantoms, projected by the forward operator)",
        "config": {"workload": f"served stream of {len(reqs)} requests, Poisson arrivals at "
                               f"{args.serve_rate:.0f}/s: {kinds['fbp']} 2D FBP (n 128..2048), "
                               f"{kinds['sirt']} 2D SIRT-20 (n 128..1024), {kinds['cgls']} 3D "
                               "CGLS-30 (128^3..256^3, 180..360 views), 8 slots, 2D requests "
                               "below 704^2 pixels coalesced into class batches of up to 16",
                   "parallelism": "one GPU, concurrent streams"},
        "p50_ms": served["p50_ms"], "p99_ms": served["p99_ms"],
        "latency_by_kind": served["by_kind"], "clocks": served["clocks"],
        "batches": served["batches"],
        "plain_loop_solves_per_s": plain_all,
        "speedup_vs_plain_loop": served["solves_per_s"] / plain_all,
        "below_capacity": {"rate_per_s": sub_rate, "solves_per_s": relaxed["solves_per_s"],
                           "p50_ms": relaxed["p50_ms"], "p99_ms": relaxed["p99_ms"],
                           "latency_by_kind": relaxed["by_kind"]},
        "mix_2d_only": {"requests": len(reqs2d), "rate_per_s": rate_2d,
                        "solves_per_s": served_2d["solves_per_s"],
                        "p50_ms": served_2d["p50_ms"], "p99_ms": served_2d["p99_ms"],
                        "batches": served_2d["batches"],
                        "plain_loop_solves_per_s": plain_2d,
                        "speedup_vs_plain_loop": served_2d["solves_per_s"] / plain_2d,
                        "without_coalescing_solves_per_s": unbatched_2d["solves_per_s"]},
    }
    if sustained is not None:
        line["sustained"] = sustained
    return line


def batch_problems(dev, count: int = 64):
    """The batched workload: ``count`` fan-beam problems, n ~ U{128, 192, 256,
    384, 512, 768, 1024}, 180..720 views, per-view Gaussian jitter (sigma 0.5
    px) on source and detector positions in full vector form, data
    y = A x + Poisson noise (I0 = 1e4) from a seeded ellipse phantom."""
    import torch

    from curadon_gb300 import FanGeometry, FanVecGeometry, forward
    from curadon_gb300.phantom import ellipses_2d, fan_config, seed_for

    rng = np.random.default_rng(seed_for(3, 0))
    sizes = [128, 192, 256, 384, 512, 768, 1024]
    out = []
    for k in range(count):
        n = int(rng.choice(sizes))
        nangles = int(rng.integers(180, 721))
        g = fan_config(n, nangles)
        v = np.asarray(FanGeometry(**g).to_vec())
        v[:, 4:] *= g["det_spacing"]
        v[:, :4] += rng.normal(0.0, 0.5, (nangles, 4))
        geom = FanVecGeometry(g["vol_shape"], g["det_shape"], v, device=dev.index or 0)
        x = ellipses_2d(n, seed_for(3, k + 1), device=dev).contiguous()
        s = torch.zeros(geom.sinogram_shape(), device=dev)
        forward(x, s, geom)
        mu = 2.5 / float(s.max())  # line integrals up to 2.5 attenuation lengths
        counts = torch.poisson(1e4 * torch.exp(-mu * s)).clamp_min(1.0)
        y = -torch.log(counts / 1e4) / mu
        out.append((geom, n, y))
    return out


def fwd_kernels(algo: str, sizes) -> int:
    """Kernels of one batched forward: the texture march 1 (plus array
    copies); the register march 2 (re-layout, rays); each plan's own 1 for
    the texture problems and 2 (re-layout, bundles) for the chunked ones."""
    if algo == "texture":
        return 1
    if algo == "registers":
        return 2
    big = [n * n >= 704 * 704 for n in sizes]
    return (1 if not all(big) else 0) + (2 if any(big) else 0)


def time_batched_gd(proj, Y, iters: int, steps: int, warmup: int):
    """Times ``steps`` steps of ``iters`` unrolled gradient-descent iterations
    x <- x - a grad 1/2 ||A x - y||^2 through torch.autograd on a batched
    projector, one iteration captured in a CUDA graph and replayed (CUDA
    events around each step); a = 1 / lambda_i per problem, lambda_i the
    largest eigenvalue of B_i A_i (B the projector's backward operator: the
    drop-in backprojector is not scaled like A^T) by power iteration
    (untimed).  Returns (ms per step, relative
    residual, a)."""
    import torch

    dev = proj.device
    v = torch.rand_like(proj.X)
    lam = None
    for _ in range(10):
        v = torch.cat([(t / t.norm().clamp_min(1e-20)).reshape(-1)
                       for t in proj.split_volumes(v)])
        with torch.no_grad():
            v = proj.adjoint(proj(v))
        lam = [float(t.norm()) for t in proj.split_volumes(v)]
    A = torch.cat([torch.full((int(np.prod(sh)),), 1.0 / max(l_, 1e-20), device=dev)
                   for sh, l_ in zip(proj.vol_shapes, lam)])
    x = torch.zeros_like(proj.X)

    def iteration():
        xr = x.detach().requires_grad_(True)
        r = proj(xr) - Y
        (g,) = torch.autograd.grad(0.5 * (r * r).sum(), xr)
        x.sub_(A * g)

    for _ in range(max(3, warmup)):
        iteration()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    cap = torch.cuda.Stream()
    cap.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(cap), torch.cuda.graph(graph, stream=cap):
        iteration()
    torch.cuda.current_stream().wait_stream(cap)
    for _ in range(max(3, warmup)):
        graph.replay()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(steps)]
    for k in range(steps):
        x.zero_()
        ev[k][0].record()
        for _ in range(iters):
            graph.replay()
        ev[k][1].record()
    torch.cuda.synchronize()
    ms = sum(a_.elapsed_time(b_) for a_, b_ in ev) / steps
    with torch.no_grad():
        res = float(torch.linalg.vector_norm(proj(x) - Y) / torch.linalg.vector_norm(Y))
    return ms, res, A


def time_plain_gd(geoms, ys, av, iters: int):
    """The same gradient-descent iterations as a plain loop of single-problem
    calls through the drop-in autograd function (one problem per launch
    chain); ms for ``iters`` iterations after three warm-up iterations."""
    import torch

    from curadon_gb300 import TorchForward

    dev = ys[0].device
    xs = [torch.zeros(tuple(int(v) for v in g.vol_shape), device=dev) for g in geoms]

    def plain_iteration():
        for i, g in enumerate(geoms):
            xr = xs[i].detach().requires_grad_(True)
            r = TorchForward.apply(xr, g) - ys[i]
            (gr,) = torch.autograd.grad(0.5 * (r * r).sum(), xr)
            xs[i].sub_(av[i] * gr)

    for _ in range(3):
        plain_iteration()
    torch.cuda.synchronize()
    for t in xs:
        t.zero_()
    a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_ev.record()
    for _ in range(iters):
        plain_iteration()
    b_ev.record()
    torch.cuda.synchronize()
    return a_ev.elapsed_time(b_ev)


def run_batch(args):
    """The batched, differentiable workload: 10 unrolled gradient-descent steps
    x <- x - a grad 1/2 ||A x - y||^2 over all 64 problems, each step through
    torch.autograd on the batched projector (one forward and one gradient for
    the whole batch, a few launches each), one step captured in a CUDA graph
    and replayed.  ``value`` counts operator calls (two per problem and step)
    per second.  Beside it: the same steps as a plain loop of single-problem
    calls through the same autograd functions (one problem per launch), and
    the reference's own CUDA operators in the same plain loop (its geometry
    holds no per-view jitter, so it runs the unjittered circular problems of
    the same sizes: the same work).  ``matched`` repeats the batched steps
    with the exact gradient (register forward, batched matched adjoint)."""
    import torch

    from curadon_gb300 import _build
    from curadon_gb300.batch import BatchProjector

    _build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    probs = batch_problems(dev)
    count = len(probs)
    geoms = [g for g, _, _ in probs]
    iters = 10
    steps = max(1, args.steps // 10)  # a step = the 10 unrolled iterations

    def batched(matched: bool):
        proj = BatchProjector(geoms, dev, forward=args.batch_forward, matched=matched)
        Y = torch.cat([y.reshape(-1) for _, _, y in probs])
        ms, res, A = time_batched_gd(proj, Y, iters, steps, args.warmup)
        return ms, res, proj, A

    batch_ms, residual, proj, A = batched(False)
    matched_ms, matched_res, _, _ = batched(True)

    # plain loop: the same autograd steps problem by problem (single-problem calls)
    ys = [y for _, _, y in probs]
    av = proj.split_volumes(A)
    plain_ms = time_plain_gd(geoms, ys, av, iters)
    a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    # the reference's operators in the same plain loop (circular problems of the same sizes)
    ref, why = reference_ops()
    ref_ms = None
    if ref is not None:
        from curadon_gb300.phantom import fan_config

        handles, rx, rs, rg = [], [], [], []
        for g, n, y in probs:
            h, _ = ref.plan2d(fan_config(n, int(y.shape[0])))
            handles.append(h)
            rx.append(torch.zeros((n, n), device=dev))
            rs.append(torch.zeros_like(y))
            rg.append(torch.zeros((n, n), device=dev))

        def ref_iteration():
            for i in range(count):
                ref.forward2d(handles[i], rx[i].data_ptr(), rs[i].data_ptr())
                torch.sub(rs[i], ys[i], out=rs[i])
                rg[i].zero_()
                ref.backward2d(handles[i], rg[i].data_ptr(), rs[i].data_ptr())
                rx[i].sub_(av[i] * rg[i])

        ref_iteration()
        torch.cuda.synchronize()
        a_ev.record()
        for _ in range(iters):
            ref_iteration()
        b_ev.record()
        torch.cuda.synchronize()
        ref_ms = a_ev.elapsed_time(b_ev)
        for h in handles:
            ref.destroy2d(h)

    ops = 2 * count * iters
    value = ops / (batch_ms / 1e3)
    plain_value = ops / (plain_ms / 1e3)
    kinds = sorted({n for _, n, _ in probs})
    line = {
        "metric": "fwd/bwd proj ops/s", "value": value, "unit": "ops/s", "n_gpus": 1,
        "steps": steps, "warmup": max(3, args.warmup),
        "ms_per_step": batch_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipse phantoms, jittered vector geometries, Poisson noise)",
        "config": {"workload": f"batched differentiable gradient descent: {count} 2D fan-beam "
                               f"problems, n in {kinds}, 180..720 views, per-view jitter sigma "
                               "0.5 px in vector form, y = Ax + Poisson noise (I0 1e4); a step = "
                               "10 unrolled iterations x - a grad 1/2||Ax - y||^2 through "
                               "torch.autograd over all problems, one iteration graph-captured",
                   "l2": "the working set (0.3-1 GB) exceeds L2", "parallelism": "one GPU"},
        "gpu_launches": (2 + fwd_kernels(proj._fwd.forward_algorithm, [n for _, n, _ in probs]))
                        * iters * steps,
        "gradient": "drop-in (the backprojector, as the reference's autograd function)",
        "relative_residual_after_10": residual,
        "plain_loop_ops_per_s": plain_value, "speedup_vs_plain_loop": value / plain_value,
        "matched": {"ops_per_s": ops / (matched_ms / 1e3), "ms_per_step": matched_ms,
                    "speedup_vs_plain_loop": (ops / (matched_ms / 1e3)) / plain_value,
                    "relative_residual_after_10": matched_res,
                    "gradient": "exact (register forward, batched matched adjoint)"},
    }
    if ref_ms is not None:
        line["reference_plain_loop_ops_per_s"] = ops / (ref_ms / 1e3)
        line["speedup_vs_reference_plain_loop"] = value / (ops / (ref_ms / 1e3))
    else:
        line["reference_plain_loop"] = {"unavailable": why}
    return line


def batch3d_problems(dev, count: int = 24, sizes=(48, 64, 96, 128)):
    """The 3D batched workload: ``count`` circular cone-beam problems, n ~
    U{sizes} (n^3 volumes; default 48, 64, 96, 128), 90..360 views,
    ceil(1.5 n)^2 cells of 1.5, source-isocentre 2n, isocentre-detector n,
    data y = A x + Poisson noise (I0 = 1e4) from a seeded ellipsoid
    phantom."""
    import torch

    from curadon_gb300 import ConeGeometry, forward
    from curadon_gb300.phantom import cone_config, ellipsoids_3d, seed_for

    rng = np.random.default_rng(seed_for(5, 0))
    out = []
    for k in range(count):
        n = int(rng.choice(list(sizes)))
        nangles = int(rng.integers(90, 361))
        cfg = cone_config(n, nangles, int(np.ceil(1.5 * n)))
        geom = ConeGeometry(**cfg, device=dev.index or 0)
        x = ellipsoids_3d(n, seed_for(5, k + 1), device=dev).contiguous()
        s = torch.zeros(geom.sinogram_shape(), device=dev)
        forward(x, s, geom)
        mu = 2.5 / float(s.max())
        counts = torch.poisson(1e4 * torch.exp(-mu * s)).clamp_min(1.0)
        y = -torch.log(counts / 1e4) / mu
        out.append((geom, cfg, y))
    return out


def run_batch3d(args):
    """The batched, differentiable workload on 3D problems: 10 unrolled
    gradient-descent iterations over all problems through torch.autograd on
    the batched 3D projector (three forward launches and two backprojection
    launches for the whole batch per iteration), one iteration captured in a
    CUDA graph; beside it the same iterations as a plain loop of
    single-problem calls through the drop-in autograd function, and the
    reference's own CUDA operators in the same plain loop."""
    import torch

    from curadon_gb300 import _build
    from curadon_gb300.batch import BatchProjector

    _build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    probs = batch3d_problems(dev, args.batch3d_count,
                             tuple(int(v) for v in args.batch3d_sizes.split(",")))
    count = len(probs)
    geoms = [g for g, _, _ in probs]
    ys = [y for _, _, y in probs]
    iters = 10
    steps = max(1, args.steps // 10)
    proj = BatchProjector(geoms, dev)
    Y = torch.cat([y.reshape(-1) for y in ys])
    batch_ms, residual, A = time_batched_gd(proj, Y, iters, steps, args.warmup)
    av = proj.split_volumes(A)
    plain_ms = time_plain_gd(geoms, ys, av, iters)
    mproj = BatchProjector(geoms, dev, matched=True)
    matched_ms, matched_res, _ = time_batched_gd(mproj, Y, iters, steps, args.warmup)
    del mproj

    ref, why = reference_ops()
    ref_ms = None
    if ref is not None:
        rx = [torch.zeros(tuple(int(v) for v in g.vol_shape), device=dev) for g in geoms]
        rs = [torch.zeros_like(y) for y in ys]
        rg = [torch.zeros_like(x) for x in rx]

        def ref_iteration():
            for i, (_, cfg, _) in enumerate(probs):
                rs[i].zero_()  # the forward writes only the rays that hit the box
                ref.forward3d(cfg, rx[i].data_ptr(), rs[i].data_ptr())
                torch.sub(rs[i], ys[i], out=rs[i])
                rg[i].zero_()
                ref.backward3d(cfg, rg[i].data_ptr(), rs[i].data_ptr())
                rx[i].sub_(av[i] * rg[i])

        ref_iteration()
        torch.cuda.synchronize()
        a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a_ev.record()
        for _ in range(iters):
            ref_iteration()
        b_ev.record()
        torch.cuda.synchronize()
        ref_ms = a_ev.elapsed_time(b_ev)

    ops = 2 * count * iters
    value = ops / (batch_ms / 1e3)
    plain_value = ops / (plain_ms / 1e3)
    sizes = sorted({int(g.vol_shape[0]) for g in geoms})
    line = {
        "metric": "fwd/bwd proj ops/s", "value": value, "unit": "ops/s", "n_gpus": 1,
        "steps": steps, "warmup": max(3, args.warmup), "ms_per_step": batch_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipsoid phantoms, Poisson noise)",
        "config": {"workload": f"batched differentiable gradient descent: {count} 3D cone-beam "
                               f"problems, n^3 with n in {sizes}, 90..360 views, ceil(1.5 n)^2 "
                               "cells, y = Ax + Poisson noise (I0 1e4); a step = 10 unrolled "
                               "iterations x - a grad 1/2||Ax - y||^2 through torch.autograd "
                               "over all problems, one iteration graph-captured",
                   "parallelism": "one GPU"},
        # per iteration: two quad re-layouts and the forward, the projections'
        # re-layout and the axial backprojection (circular orbits)
        "gpu_launches": 5 * iters * steps,
        "gradient": "drop-in (the backprojector, as the reference's autograd function)",
        "relative_residual_after_10": residual,
        "residual_note": "in 3D the drop-in gradient is not the transpose of the ray-driven "
                         "forward (B A has eigen-directions with negative real part): the "
                         "residual falls for the first iterations, then grows; the matched "
                         "gradient converges",
        "plain_loop_ops_per_s": plain_value, "speedup_vs_plain_loop": value / plain_value,
        "matched": {"ops_per_s": ops / (matched_ms / 1e3), "ms_per_step": matched_ms,
                    "speedup_vs_plain_loop": (ops / (matched_ms / 1e3)) / plain_value,
                    "relative_residual_after_10": matched_res,
                    "gradient": "exact (quad forward, batched matched adjoint)"},
    }
    if ref_ms is not None:
        line["reference_plain_loop_ops_per_s"] = ops / (ref_ms / 1e3)
        line["speedup_vs_reference_plain_loop"] = value / (ops / (ref_ms / 1e3))
    else:
        line["reference_plain_loop"] = {"unavailable": why}
    return line


def main():
    global CONE_VIEWS
    args = parse()
    CONE_VIEWS = args.cone_views
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "sweep":
        line = run_sweep(args) if rank == 0 else None
    elif args.workload == "serve":
        line = run_serve(args) if rank == 0 else None
    elif args.workload == "batch":
        line = run_batch(args) if rank == 0 else None
    elif args.workload == "batch3d":
        line = run_batch3d(args) if rank == 0 else None
    elif args.impl == "reference":
        line = run_reference_cpu(args, rank, world)
    elif args.impl == "reference-gpu":
        line = run_reference_gpu(args, rank, world, local_rank)
    else:
        if world > 1:
            import torch
            import torch.distributed as dist

            torch.cuda.set_device(local_rank)
            dist.init_process_group("nccl", device_id=torch.device("cuda", local_rank))
        line = run_ours(args, rank, world, local_rank)
        if line is not None and world == 1 and not args.no_cpu_baseline:
            wl = workload(args.workload)
            threads = os.cpu_count() or 1
            ops_s, desc = cpu_sample(wl, args.cpu_seconds, threads)
            line["cpu_baseline"] = {"value": ops_s, "unit": "ops/s", "cores": threads,
                                    "kind": "port", "sample": desc}
        if world > 1:
            import torch.distributed as dist

            dist.destroy_process_group()
    if line is not None:
        print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
