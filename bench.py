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

# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum) from
# the ncu captures summarised in profiles/, by workload and kernel; None
# where not captured.
NCU_TRAFFIC = {
    ("fan2048", "k_fwd2d_cslab"): 83_357_440,  # profiles/k_fwd2d_cslab_fan2048.md capture
    ("fan2048", "k_bwd2d_smem"): 64_185_344,   # profiles/k_bwd2d_smem_fan2048.md
    ("fan2048", "k_fwd2d_tex"): 17_007_744,    # the texture-unit forward (algorithm 1)
    ("cone256", "k_fwd3d_quad"): 2_015_147_008,  # profiles/k_fwd3d_quad_cone256.md (algorithm 5)
    ("cone256", "k_bwd3d_ax"): 500_470_784,      # profiles/k_bwd3d_ax_cone256.md
    ("cone256", "k_fwd3d_tex3"): 1_281_753_856,  # profiles/k_bwd3d_cone256.md
    ("cone256", "k_bwd3d"): 504_137_984,
}

# Main kernel of each operator by the plan's algorithm name.
KERNELS = {
    ("fan", "forward", "texture"): "k_fwd2d_tex", ("fan", "forward", "chunked"): "k_fwd2d_cslab",
    ("fan", "forward", "registers"): "k_fwd2d", ("fan", "forward", "hybrid"): "k_fwd2d_hyb",
    ("fan", "forward", "slab"): "k_fwd2d_slab", ("fan", "backward", "shared"): "k_bwd2d_smem",
    ("fan", "backward", "registers"): "k_bwd2d", ("fan", "backward", "texture"): "k_bwd2d_tex",
    ("cone", "forward", "texture"): "k_fwd3d_tex3", ("cone", "forward", "layered"): "k_fwd3d_tex2l",
    ("cone", "forward", "registers"): "k_fwd3d", ("cone", "forward", "slab"): "k_fwd3d_slab",
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
                        "(served reconstruction stream vs the plain loop) or batch (64 "
                        "jittered problems, batched gradient descent vs the plain loop)")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--batch-forward", default="texture", choices=["texture", "registers"],
                   help="forward algorithm of the batch workload")
    p.add_argument("--cpu-seconds", type=float, default=12.0,
                   help="CPU work budget of the cpu_baseline sample")
    return p.parse_args()


# ------------------------------------------------------------ workloads

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


def cone_sample_estimate(g) -> int:
    n = g["vol_shape"][0]
    nangles = len(g["angles"])
    det = g["det_shape"][0]
    # rays through the volume ~ detector cells covering its shadow, ~n samples each
    return int(nangles * det * det * 0.6 * n)


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
        # forward: texture 1; split: re-layout + texture share + chunked rest;
        # others: re-layout + kernel
        f = {"texture": 1, "split": 3}.get(fwd, 2)
        # backprojection: texture one per 2048 views; split: re-layout +
        # texture rows + staged rows; others: re-layout + kernel
        b = {"texture": -(-nv // 2048), "split": 3}.get(bwd, 2)
        return f + b
    # forward: texture 1; layered: transpose + kernel; registers, slab, quad,
    # mixed: two re-layouts + kernel
    f = {"texture": 1, "layered": 2}.get(fwd, 3)
    # backprojection: re-layout + one kernel (axial: one per 768 views)
    b = 1 + (-(-nv // 768) if bwd == "axial" else 1)
    return f + b


def run_ours(args, rank, world, local_rank):
    import torch

    import curadon_gb300 as cg
    from curadon_gb300 import _build
    from curadon_gb300.phantom import ellipses_2d, ellipsoids_3d

    _build.build()
    dev = torch.device("cuda", local_rank)
    torch.cuda.set_device(dev)
    wl = workload(args.workload)
    g = wl["geom"]
    if wl["kind"] == "fan":
        geom = cg.FanGeometry(**g, device=local_rank)
        vol = ellipses_2d(wl["n"], wl["seed"], device=dev).contiguous()
    else:
        geom = cg.ConeGeometry(**g, device=local_rank)
        vol = ellipsoids_3d(wl["n"], wl["seed"], device=dev).contiguous()
    sino = torch.zeros(geom.sinogram_shape(), device=dev)
    vbp = torch.zeros_like(vol)
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    launches_per_step = kernels_per_step(wl, geom)

    def step():
        cg.forward(vol, sino, geom)
        vbp.zero_()
        cg.backward(sino, vbp, geom)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    sampler = ClockSampler(local_rank) if rank == 0 else None
    if sampler:
        sampler.start()
        time.sleep(0.2)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        e0, e1, e2 = ev[k]
        e0.record(stream)
        cg.forward(vol, sino, geom)
        e1.record(stream)
        vbp.zero_()
        cg.backward(sino, vbp, geom)
        e2.record(stream)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    t_fwd = [ev[k][0].elapsed_time(ev[k][1]) for k in range(args.steps)]
    t_bwd = [ev[k][1].elapsed_time(ev[k][2]) for k in range(args.steps)]
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

    total_ms, e2e_ms, fwd_ms, bwd_ms = reduce_max([total_ms, e2e_ms, sum(t_fwd), sum(t_bwd)],
                                                  world, dev)
    if rank != 0:
        return None

    ops = 2 * args.steps * world
    value = ops / (total_ms / 1e3)
    ms_fwd = fwd_ms / args.steps
    ms_bwd = bwd_ms / args.steps

    # roofline of the dominant operator: compulsory bytes per call / its time
    if wl["kind"] == "fan":
        nvox = wl["n"] * wl["n"]
        nrays = len(g["angles"]) * g["det_shape"]
        s_fwd = fan_sample_count(g)
        s_bwd = nvox * len(g["angles"])
        gather = {"forward": 16, "backward": 8}
    else:
        nvox = wl["n"] ** 3
        nrays = len(g["angles"]) * g["det_shape"][0] * g["det_shape"][1]
        s_fwd = cone_sample_estimate(g)
        s_bwd = nvox * len(g["angles"])
        gather = {"forward": 32, "backward": 16}
    b_alg = {"forward": 4 * (nvox + nrays), "backward": 4 * (nrays + 2 * nvox)}
    dom = "forward" if ms_fwd >= ms_bwd else "backward"
    t_dom = (ms_fwd if dom == "forward" else ms_bwd) / 1e3
    algos = dict(zip(("forward", "backward"), geom.plan.algorithm))
    kernel = KERNELS.get((wl["kind"], dom, algos[dom]), dom)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    peak = peaks.get("hbm_gbs")
    peak_src = "measured" if peak else "fallback"
    peak = peak or 6800.0
    achieved = b_alg[dom] / t_dom / 1e9
    samples = s_fwd if dom == "forward" else s_bwd
    traffic = NCU_TRAFFIC.get((wl["name"], kernel))
    roofline = {"bound": "hbm", "kernel": kernel, "operator": dom,
                "achieved": round(achieved, 3), "peak": peak,
                "peak_source": peak_src, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "algorithmic_bytes": b_alg[dom],
                "samples_per_s": samples / t_dom,
                "gather_GBps": samples * gather[dom] / t_dom / 1e9,
                "note": "gather-bound (L1/issue), not HBM-bound: the compulsory bytes are "
                        "L2-resident; samples_per_s is the efficiency figure"}

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
        "e2e": {"value": ops / (e2e_ms / 1e3), "unit": "ops/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": launches_per_step * args.steps,
        "roofline": roofline,
        "clocks": clocks,
    }
    return line


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
    if rank != 0:
        return None
    wl = workload(args.workload)
    threads = os.cpu_count() or 1
    per_step = []
    desc = ""
    budget = 2.0
    for k in range(args.warmup + args.steps):
        ops_s, desc = cpu_sample(wl, budget, threads)
        if k >= args.warmup:
            per_step.append(2.0 / ops_s)
    total = sum(per_step)
    value = 2 * args.steps / total
    return {
        "impl": "reference", "metric": "fwd/bwd proj ops/s", "value": value, "unit": "ops/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": total / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded ellipse phantom)",
        "config": dict(wl["config"], parallelism="host cores"),
        "cpu_baseline": {"value": value, "unit": "ops/s", "cores": threads, "kind": "port",
                         "sample": desc + " (the reference has no CPU path; its operators "
                                          "restated by the oracle)"},
        "e2e": {"value": value, "unit": "ops/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }


def run_reference_gpu(args, rank, world, local_rank):
    if rank != 0:
        return None
    import torch

    import oracle
    from oracle import build_ref
    from curadon_gb300.phantom import ellipses_2d, ellipsoids_3d

    if build_ref.build() is None or not oracle.ref_available():
        return {"impl": "reference-gpu", "unavailable": "reference headers not staged/built"}
    ref = oracle.RefOps()
    dev = torch.device("cuda", local_rank)
    wl = workload(args.workload)
    g = wl["geom"]
    tf, tb = [], []
    if wl["kind"] == "fan":
        vol = ellipses_2d(wl["n"], wl["seed"], device=dev).contiguous()
        h, n = ref.plan2d(g)
        sino = torch.zeros((n, g["det_shape"]), device=dev)
        vbp = torch.zeros_like(vol)

        def fwd():
            ref.forward2d(h, vol.data_ptr(), sino.data_ptr())

        def bwd():
            vbp.zero_()
            ref.backward2d(h, vbp.data_ptr(), sino.data_ptr())
    else:
        vol = ellipsoids_3d(wl["n"], wl["seed"], device=dev).contiguous()
        n = len(g["angles"])
        sino = torch.zeros((n, *g["det_shape"]), device=dev)
        vbp = torch.zeros_like(vol)

        def fwd():
            ref.forward3d(g, vol.data_ptr(), sino.data_ptr())

        def bwd():
            vbp.zero_()
            ref.backward3d(g, vbp.data_ptr(), sino.data_ptr())
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    for _ in range(args.warmup):
        fwd(), bwd()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        fwd()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        bwd()
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        tf.append(t1 - t0)
        tb.append(t2 - t1)
    total = sum(tf) + sum(tb)
    return {
        "impl": "reference-gpu", "metric": "fwd/bwd proj ops/s",
        "value": 2 * args.steps / total, "unit": "ops/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipse phantom)", "config": wl["config"],
        "fwd_ops_s": args.steps / sum(tf), "bwd_ops_s": args.steps / sum(tb),
        "ms_forward": sum(tf) / args.steps * 1e3, "ms_backward": sum(tb) / args.steps * 1e3,
        "timing": "wall clock around each synchronous reference call (its own protocol)",
    }


# ------------------------------------------------------------ serving

def serve_requests(n_req: int, dev, seed: int = 4000):
    """A seeded request mix in the proportions of the served stream: 70 %
    2D FBP (n log-uniform over 128..2048, n views), 25 % 2D SIRT-20 (n
    128..512), 5 % 3D CGLS-30 (n 64..128, 2n views); sizes drawn from a
    log-spaced set so geometries repeat as in a clinic.  Sinograms are
    projections of seeded phantoms, in pinned host memory."""
    import torch

    from curadon_gb300 import ConeGeometry, FanGeometry, forward
    from curadon_gb300.phantom import cone_config, ellipses_2d, ellipsoids_3d, fan_config
    from curadon_gb300.serve import Request

    rng = np.random.default_rng(seed)
    fbp_sizes = [128, 181, 256, 362, 512, 724, 1024, 1448, 2048]
    sirt_sizes = [128, 181, 256, 362, 512]
    cone_sizes = [64, 96, 128]
    geoms, reqs = {}, []
    for _ in range(n_req):
        u = rng.random()
        if u < 0.70:
            kind, n = "fbp", int(rng.choice(fbp_sizes))
        elif u < 0.95:
            kind, n = "sirt", int(rng.choice(sirt_sizes))
        else:
            kind, n = "cgls", int(rng.choice(cone_sizes))
        key = (kind == "cgls", n)
        if key not in geoms:
            if kind == "cgls":
                geoms[key] = ConeGeometry(**cone_config(n, 2 * n, int(1.5 * n)))
            else:
                geoms[key] = FanGeometry(**fan_config(n))
        g = geoms[key]
        ph = (ellipsoids_3d(n, int(rng.integers(1 << 30)), device=dev) if kind == "cgls"
              else ellipses_2d(n, int(rng.integers(1 << 30)), device=dev)).contiguous()
        y = torch.zeros(g.sinogram_shape(), device=dev)
        forward(ph, y, g)
        iters = {"fbp": 0, "sirt": 20, "cgls": 30}[kind]
        reqs.append(Request(kind, g, y.cpu().pin_memory(), iters=iters))
    torch.cuda.synchronize()
    return reqs


def run_serve(args):
    """Served solves/s with Poisson arrivals against the plain loop (one
    problem at a time, each solved and read back before the next)."""
    import threading

    import torch

    from curadon_gb300 import _build
    from curadon_gb300.fbp import fbp
    from curadon_gb300.serve import Server
    from curadon_gb300.solvers import cgls, sirt

    _build.build()
    dev = torch.device("cuda", 0)
    n_req = max(20, args.steps * 8)
    reqs = serve_requests(n_req, dev)

    def plain(r):
        y = r.sinogram.to(dev)
        x = (fbp(y, r.geom) if r.kind == "fbp" else
             sirt(r.geom, y, r.iters) if r.kind == "sirt" else cgls(r.geom, y, r.iters))
        return x.cpu()

    for r in reqs[:min(len(reqs), 30)]:  # warm-up: plans and filters of the plain path
        plain(r)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for r in reqs:
        plain(r)
    t_plain = time.perf_counter() - t0

    srv = Server(device=0, slots=8)
    for f in [srv.submit(r) for r in reqs[:min(len(reqs), 30)]]:  # warm-up: slot residency
        f.result()
    srv.latencies.clear()
    srv.completed, srv.t_first, srv.t_last = 0, None, None
    rate = 200.0
    rng = np.random.default_rng(7)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
    futs = []

    def client():
        t_start = time.perf_counter()
        for r, ta in zip(reqs, arrivals):
            delay = t_start + ta - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            futs.append(srv.submit(r))

    th = threading.Thread(target=client)
    th.start()
    th.join()
    for f in futs:
        f.result()
    srv.close()
    st = srv.stats()
    plain_rate = len(reqs) / t_plain
    kinds = {k: sum(r.kind == k for r in reqs) for k in ("fbp", "sirt", "cgls")}
    return {
        "metric": "served solves/s", "value": st["solves_per_s"], "unit": "solves/s",
        "n_gpus": 1, "steps": len(reqs), "warmup": 30, "ms_per_step": 1e3 / st["solves_per_s"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded phantoms, projected by the forward operator)",
        "config": {"workload": f"served stream of {len(reqs)} requests, Poisson arrivals at "
                               f"{rate:.0f}/s: {kinds['fbp']} 2D FBP (n 128..2048), "
                               f"{kinds['sirt']} 2D SIRT-20 (n 128..512), {kinds['cgls']} 3D "
                               "CGLS-30 (n 64..128, 2n views), 8 slots",
                   "parallelism": "one GPU, concurrent streams"},
        "p50_ms": st["p50_ms"], "p99_ms": st["p99_ms"],
        "plain_loop_solves_per_s": plain_rate, "speedup_vs_plain_loop": st["solves_per_s"] / plain_rate,
    }


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


def run_batch(args):
    """Gradient descent x <- x - a A^T (A x - y) on the batched workload: one
    iteration over all problems is a batched forward (one array copy per
    problem and one texture launch) and a batched backprojection (two
    launches) with two elementwise ops on flat buffers, captured once in a
    CUDA graph and replayed; against the plain loop (the single-problem
    operators, problem by problem).  The value counts operator calls (two
    per problem and iteration) per second."""
    import torch

    from curadon_gb300 import _build, backward, forward
    from curadon_gb300.batch import Batch2d

    _build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    probs = batch_problems(dev)
    count = len(probs)
    nv = [n * n for _, n, _ in probs]
    ns = [int(np.prod(y.shape)) for _, _, y in probs]
    X, G = torch.zeros(sum(nv), device=dev), torch.zeros(sum(nv), device=dev)
    S, R = torch.zeros(sum(ns), device=dev), torch.zeros(sum(ns), device=dev)
    Y = torch.cat([y.reshape(-1) for _, _, y in probs])
    A = torch.empty(sum(nv), device=dev)

    def views(flat, sizes, shapes):
        offs = np.cumsum([0] + sizes)
        return [flat[offs[i]:offs[i + 1]].view(shapes[i]) for i in range(len(sizes))]

    vshapes = [(n, n) for _, n, _ in probs]
    sshapes = [tuple(y.shape) for _, _, y in probs]
    xs, gs = views(X, nv, vshapes), views(G, nv, vshapes)
    ss, rs = views(S, ns, sshapes), views(R, ns, sshapes)
    geoms = [g for g, _, _ in probs]
    bf = Batch2d(geoms, xs, ss, forward=args.batch_forward)  # s_i = A_i x_i
    bb = Batch2d(geoms, gs, rs)  # g_i += A_i^T r_i
    # step sizes 1 / ||A_i^T A_i|| by power iteration (set-up, untimed)
    X.uniform_(0.0, 1.0)
    for _ in range(8):
        bf.forward()
        R.copy_(S)
        G.zero_()
        bb.backward()
        for x, g in zip(xs, gs):
            x.copy_(g / g.norm().clamp_min(1e-20))
    bf.forward()
    for a, s_ in zip(views(A, nv, vshapes), ss):
        a.fill_(1.0 / float(s_.norm() ** 2))
    X.zero_()

    def iteration():
        bf.forward()
        torch.sub(S, Y, out=R)
        G.zero_()
        bb.backward()
        X.addcmul_(A, G, value=-1.0)

    for _ in range(max(3, args.warmup)):
        iteration()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    cap = torch.cuda.Stream()
    cap.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(cap), torch.cuda.graph(graph, stream=cap):
        iteration()
    torch.cuda.current_stream().wait_stream(cap)
    X.zero_()
    iters = 10
    steps = max(1, args.steps // 10)  # a step = the 10 unrolled iterations
    for _ in range(max(3, args.warmup)):
        graph.replay()
    torch.cuda.synchronize()
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(steps)]
    for k in range(steps):
        X.zero_()
        ev[k][0].record()
        for _ in range(iters):
            graph.replay()
        ev[k][1].record()
    torch.cuda.synchronize()
    batch_ms = sum(a.elapsed_time(b) for a, b in ev)
    # the cost the iterations drive down (a check that the solver works)
    bf.forward()
    residual = float(torch.linalg.vector_norm(S - Y) / torch.linalg.vector_norm(Y))

    # plain loop: the single-problem operators problem by problem
    yv = views(Y, ns, sshapes)
    av = views(A, nv, vshapes)

    def plain_iteration():
        for i, g in enumerate(geoms):
            forward(xs[i], ss[i], g)
            torch.sub(ss[i], yv[i], out=rs[i])
            gs[i].zero_()
            backward(rs[i], gs[i], g)
            xs[i].addcmul_(av[i], gs[i], value=-1.0)

    for _ in range(3):
        plain_iteration()
    torch.cuda.synchronize()
    X.zero_()
    a_ev, b_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a_ev.record()
    for _ in range(iters):
        plain_iteration()
    b_ev.record()
    torch.cuda.synchronize()
    plain_ms = a_ev.elapsed_time(b_ev)

    ops = 2 * count * iters * steps
    value = ops / (batch_ms / 1e3)
    plain_value = 2 * count * iters / (plain_ms / 1e3)
    kinds = sorted({n for _, n, _ in probs})
    return {
        "metric": "fwd/bwd proj ops/s", "value": value, "unit": "ops/s", "n_gpus": 1,
        "steps": steps, "warmup": max(3, args.warmup),
        "ms_per_step": batch_ms / steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded ellipse phantoms, jittered vector geometries, Poisson noise)",
        "config": {"workload": f"batched gradient descent: {count} 2D fan-beam problems, n in "
                               f"{kinds}, 180..720 views, per-view jitter sigma 0.5 px in "
                               "vector form, y = Ax + Poisson noise (I0 1e4); a step = 10 "
                               "iterations x - a A^T(Ax - y) over all problems",
                   "l2": "the working set (0.3-1 GB) exceeds L2", "parallelism": "one GPU"},
        "gpu_launches": (2 + (1 if bf.forward_algorithm == "texture" else 2)) * iters * steps,
        "plain_loop_ops_per_s": plain_value, "speedup_vs_plain_loop": value / plain_value,
        "relative_residual_after_10": residual,
    }


def main():
    args = parse()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if args.workload == "serve":
        line = run_serve(args) if rank == 0 else None
    elif args.workload == "batch":
        line = run_batch(args) if rank == 0 else None
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
