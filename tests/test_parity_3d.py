"""GPU parity of the 3D cone-beam operators (through the C ABI).

Tolerance: relative L2 <= 1e-3 against the reference's operators and the
FP64 oracle; rays that miss the volume must stay unwritten exactly where the
reference leaves them unwritten."""
import numpy as np
import pytest
import torch

import oracle
from conftest import load_golden, max_abs, rel_l2
from curadon_gb300 import ConeGeometry, backward, backward_3d, forward, forward_3d
from curadon_gb300.backend import FORWARD_3D
from curadon_gb300.phantom import cone_config, ellipsoids_3d

pytestmark = pytest.mark.gpu
TOL = 1e-3
SENTINEL = -7.0


def make(g, dev):
    kw = {k: g[k] for k in ("DSD", "DSO", "angles", "vol_shape", "det_shape")}
    for k in ("det_spacing", "det_offset", "det_rotation", "vol_spacing", "vol_offset", "COR"):
        if k in g:
            kw[k] = g[k]
    return ConeGeometry(**kw, device=dev.index or 0)


def run_fwd(geom, vol, dev):
    v = torch.as_tensor(vol, device=dev).contiguous()
    s = torch.full(geom.sinogram_shape(), SENTINEL, device=dev)
    forward(v, s, geom)
    torch.cuda.synchronize()
    return s.cpu().numpy()


def run_bwd(geom, sino, dev, vol0):
    s = torch.as_tensor(sino, device=dev, dtype=torch.float32).contiguous()
    v = torch.as_tensor(vol0, device=dev, dtype=torch.float32).clone()
    backward(s, v, geom)
    torch.cuda.synchronize()
    return v.cpu().numpy()


def check_fwd(s, ref):
    """Same written/unwritten pattern as the reference and rel-L2 <= TOL.

    A ray that only grazes the box [-1, N+1]^3 can flip between hit and miss
    on the last bit of its slab test; it touches only the zero border, so
    where one side wrote it the value is exactly 0.  Such flips are allowed
    at a rate of at most one ray per million."""
    miss_ref, miss = ref == SENTINEL, s == SENTINEL
    flip = miss_ref != miss
    assert flip.sum() <= max(2, 1e-6 * flip.size), f"{flip.sum()} rays differ in hit/miss"
    assert np.all(ref[flip & ~miss_ref] == 0) and np.all(s[flip & ~miss] == 0)
    both = ~miss_ref & ~miss
    e = rel_l2(s[both], ref[both])
    print(f"fwd rel-L2 {e:.2e} max-abs {max_abs(s[both], ref[both]):.2e} flips {flip.sum()}")
    assert e < TOL


@pytest.mark.parametrize("case", ["cone_small", "cone_rot"])
def test_against_golden(cuda_device, case):
    z, g = load_golden(case)
    geom = make(g, cuda_device)
    check_fwd(run_fwd(geom, z["volume"], cuda_device), z["sino_ref"])
    b = run_bwd(geom, z["bwd_in"], cuda_device, np.ones(z["volume"].shape, np.float32))
    e = rel_l2(b, z["bwd_ref"])
    print(f"{case} bwd rel-L2 {e:.2e} max-abs {max_abs(b, z['bwd_ref']):.2e}")
    assert e < TOL


@pytest.mark.parametrize("shape,nangles,det", [((24, 24, 24), 16, 40), ((20, 28, 36), 33, 50)])
def test_against_oracle(cuda_device, shape, nangles, det):
    g = cone_config(shape[0], nangles, det)
    g["vol_shape"] = shape
    geom = make(g, cuda_device)
    ph = ellipsoids_3d(shape, 5).numpy()
    s = run_fwd(geom, ph, cuda_device)
    so = oracle.fwd3d(g, ph, sino0=np.full(geom.sinogram_shape(), SENTINEL))
    check_fwd(s, so)
    sin = np.where(so == SENTINEL, 0.0, so).astype(np.float32)
    b = run_bwd(geom, sin, cuda_device, np.zeros(shape, np.float32))
    bo = oracle.bwd3d(g, sin)
    assert rel_l2(b, bo) < TOL, rel_l2(b, bo)


@pytest.mark.parametrize("algo", FORWARD_3D)
@pytest.mark.parametrize("shape,nangles,det", [((40, 40, 40), 36, 64), ((20, 28, 36), 33, 90)])
def test_forward_algorithms(cuda_device, algo, shape, nangles, det):
    """Every selectable 3D forward agrees with the oracle, hit/miss included
    (the wide detector makes bundles whose rays change stepping axis)."""
    g = cone_config(shape[0], nangles, det)
    g["vol_shape"] = shape
    geom = make(g, cuda_device)
    geom.plan.set_algorithm(forward=algo)
    ph = ellipsoids_3d(shape, 5).numpy()
    s = run_fwd(geom, ph, cuda_device)
    print(algo, end=" ")
    check_fwd(s, oracle.fwd3d(g, ph, sino0=np.full(geom.sinogram_shape(), SENTINEL)))


@pytest.mark.parametrize("n,nangles,det", [(64, 90, 96), (128, 180, 192), (256, 360, 384),
                                           (512, 720, 768)])
def test_against_reference(cuda_device, ref_ops, n, nangles, det):
    g = cone_config(n, nangles, det)
    geom = make(g, cuda_device)
    v = ellipsoids_3d(n, n, device=cuda_device).contiguous()
    s_ref = torch.full(geom.sinogram_shape(), SENTINEL, device=cuda_device)
    ref_ops.forward3d(g, v.data_ptr(), s_ref.data_ptr())
    ref_ops.sync()
    s = torch.full_like(s_ref, SENTINEL)
    forward(v, s, geom)
    torch.cuda.synchronize()
    check_fwd(s.cpu().numpy(), s_ref.cpu().numpy())
    sin = torch.where(s_ref == SENTINEL, torch.zeros_like(s_ref), s_ref).contiguous()
    b_ref = torch.zeros_like(v)
    ref_ops.backward3d(g, b_ref.data_ptr(), sin.data_ptr())
    ref_ops.sync()
    b = torch.zeros_like(v)
    backward(sin, b, geom)
    torch.cuda.synchronize()
    e = rel_l2(b.cpu(), b_ref.cpu())
    print(f"n={n} bwd rel-L2 {e:.2e} max-abs {max_abs(b.cpu(), b_ref.cpu()):.2e}")
    assert e < TOL


def test_per_call_api_matches_plan(cuda_device):
    z, g = load_golden("cone_rot")
    geom = make(g, cuda_device)
    v = torch.as_tensor(z["volume"], device=cuda_device).contiguous()
    s1 = torch.full(geom.sinogram_shape(), SENTINEL, device=cuda_device)
    forward(v, s1, geom)
    s2 = torch.full_like(s1, SENTINEL)
    a = geom.angles
    forward_3d(v, geom.vol_shape, geom.vol_spacing, geom.vol_offset, s2, a[0], a[1], a[2],
               geom.det_shape, geom.det_spacing, geom.det_offset, geom.det_rotation, geom.DSO,
               geom.DSD, geom.COR)
    torch.cuda.synchronize()
    assert torch.equal(s1, s2)
    sin = torch.where(s1 == SENTINEL, torch.zeros_like(s1), s1).contiguous()
    b1, b2 = torch.ones_like(v), torch.ones_like(v)
    backward(sin, b1, geom)
    backward_3d(b2, geom.vol_shape, geom.vol_spacing, geom.vol_offset, sin, a[0], a[1], a[2],
                geom.det_shape, geom.det_spacing, geom.det_offset, geom.det_rotation, geom.DSO,
                geom.DSD, geom.COR)
    torch.cuda.synchronize()
    assert torch.equal(b1, b2)


def test_linearity_and_accumulation(cuda_device):
    g = cone_config(48, 40, 72)
    geom = make(g, cuda_device)
    x = ellipsoids_3d(48, 1).numpy()
    y = ellipsoids_3d(48, 2).numpy()
    a = run_fwd(geom, x, cuda_device)
    b = run_fwd(geom, y, cuda_device)
    hit = a != SENTINEL
    c = run_fwd(geom, 2 * x - y, cuda_device)
    assert rel_l2(c[hit], (2 * a - b)[hit]) < 1e-5
    sin = np.where(hit, a, 0).astype(np.float32)
    v0 = np.random.default_rng(0).uniform(0, 1, x.shape).astype(np.float32)
    b0 = run_bwd(geom, sin, cuda_device, np.zeros_like(x))
    b1 = run_bwd(geom, sin, cuda_device, v0)
    assert rel_l2(b1, b0 + v0) < 1e-6


BACKWARD_3D_VARIANTS = ["pair", "quad", "ax8m5"]


def backward_with(variant, monkeypatch, g, sin, dev, vol0):
    """Backprojection through a plan made while CURADON_GB300_ALGO selects
    ``bwd3d=variant`` (the variable is read when a plan is created)."""
    monkeypatch.setenv("CURADON_GB300_ALGO", f"bwd3d={variant}")
    geom = make(g, dev)
    geom.plan
    monkeypatch.delenv("CURADON_GB300_ALGO")
    return run_bwd(geom, sin, dev, vol0)


@pytest.mark.parametrize("variant", BACKWARD_3D_VARIANTS)
@pytest.mark.parametrize("shape,nangles,det,rot", [((20, 28, 36), 33, 50, None),
                                                   ((40, 40, 40), 36, 64, None),
                                                   ((33, 17, 29), 25, 48, (0.1, 0.0, 0.05))])
def test_backward_variants(cuda_device, monkeypatch, variant, shape, nangles, det, rot):
    """Every selectable 3D backprojection agrees with the oracle; the general
    kernel on row-pair quads (quad, the default) and on 8-byte pairs (pair,
    its fallback where the quads do not fit) read the same samples with the
    same arithmetic, so they agree bit for bit.  The axial runs (ax8m5) need
    every view to map y onto the detector's v axis; with a tilted detector
    the plan runs the general kernel instead."""
    g = cone_config(shape[0], nangles, det)
    g["vol_shape"] = shape
    if rot is not None:
        g["det_rotation"] = rot
    rng = np.random.default_rng(11)
    sin = rng.uniform(0, 1, (nangles, det, det)).astype(np.float32)
    v0 = np.zeros(shape, np.float32)
    b = backward_with(variant, monkeypatch, g, sin, cuda_device, v0)
    bo = oracle.bwd3d(g, sin)
    e = rel_l2(b, bo)
    print(f"{variant} bwd rel-L2 {e:.2e} max-abs {max_abs(b, bo):.2e}")
    assert e < TOL
    if variant == "quad":
        ref = backward_with("pair", monkeypatch, g, sin, cuda_device, v0)
        assert np.array_equal(b, ref)


def test_backward_algorithm_selection(cuda_device):
    """Circular orbits without detector tilt run the axial backprojector by
    default; a tilted detector or ``backward="registers"`` runs the general
    one, and both agree with the oracle."""
    g = cone_config(24, 20, 40)
    geom = make(g, cuda_device)
    assert geom.plan.algorithm[1] == "axial"
    rng = np.random.default_rng(5)
    sin = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    bo = oracle.bwd3d(g, sin)
    b_ax = run_bwd(geom, sin, cuda_device, np.zeros(g["vol_shape"], np.float32))
    geom.plan.set_algorithm(backward="registers")
    assert geom.plan.algorithm[1] == "registers"
    b_gen = run_bwd(geom, sin, cuda_device, np.zeros(g["vol_shape"], np.float32))
    assert rel_l2(b_ax, bo) < TOL and rel_l2(b_gen, bo) < TOL
    tilted = dict(g, det_rotation=(0.0, 0.02, 0.0))
    gt = make(tilted, cuda_device)
    assert gt.plan.algorithm[1] == "registers"


@pytest.mark.parametrize("variant", ["ax8m5", "quad"])
def test_backward_many_views(cuda_device, monkeypatch, variant):
    """More views than one launch of the axial kernel carries (768): the
    views are split over launches that accumulate."""
    g = cone_config(16, 1000, 24)
    g["vol_shape"] = (12, 16, 20)
    rng = np.random.default_rng(9)
    sin = rng.uniform(0, 1, (1000, 24, 24)).astype(np.float32)
    v0 = rng.uniform(0, 1, g["vol_shape"]).astype(np.float32)
    b = backward_with(variant, monkeypatch, g, sin, cuda_device, v0)
    bo = oracle.bwd3d(g, sin)
    e = rel_l2(b - v0, bo)
    print(f"{variant} 1000 views bwd rel-L2 {e:.2e}")
    assert e < TOL


@pytest.mark.parametrize("variant", ["mixed,fwd3d_tex=1", "mixed,fwd3d_tex=4",
                                     "mixed,fwd3d_tex=7", "mixed,fwd3d_tex=8"])
def test_forward_quad_variants(cuda_device, monkeypatch, variant):
    """The mixed forward with 1 to 8 of every 8 warps sampling through the
    texture unit (CURADON_GB300_ALGO fwd3d=mixed,fwd3d_tex=k), against the
    oracle."""
    shape, nangles, det = (20, 28, 36), 33, 90
    g = cone_config(shape[0], nangles, det)
    g["vol_shape"] = shape
    monkeypatch.setenv("CURADON_GB300_ALGO", f"fwd3d={variant}")
    geom = make(g, cuda_device)
    geom.plan
    monkeypatch.delenv("CURADON_GB300_ALGO")
    ph = ellipsoids_3d(shape, 5).numpy()
    s = run_fwd(geom, ph, cuda_device)
    check_fwd(s, oracle.fwd3d(g, ph, sino0=np.full(geom.sinogram_shape(), SENTINEL)))


def test_quad_buffers_fall_back_when_memory_is_short(cuda_device):
    """With the device nearly full, the default forward (mixed quads) and
    backprojection (axial quads) cannot allocate their 16-byte quad copies:
    the forward continues on the texture unit and the backprojection on the
    general kernel with 8-byte pairs, with the same results (no out-of-memory
    error)."""
    n, nangles, det = 96, 64, 128
    g = cone_config(n, nangles, det)
    ph = ellipsoids_3d(n, 6).numpy()
    ref_geom = make(g, cuda_device)
    s_ref = run_fwd(ref_geom, ph, cuda_device)
    sin = np.where(s_ref == SENTINEL, 0.0, s_ref).astype(np.float32)
    b_ref = run_bwd(ref_geom, sin, cuda_device, np.zeros(ph.shape, np.float32))

    geom = make(g, cuda_device)
    v = torch.as_tensor(ph, device=cuda_device).contiguous()
    s = torch.full(geom.sinogram_shape(), SENTINEL, device=cuda_device)
    b = torch.zeros_like(v)
    st = torch.as_tensor(sin, device=cuda_device)
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    free, _ = torch.cuda.mem_get_info()
    # leave about 24 MB: room for the texture array and the pair copies, not
    # for the quad copies (2 x 33 MB) or the projection quads (18 MB)
    filler = torch.empty(max(0, free - (24 << 20)), dtype=torch.uint8, device=cuda_device)
    try:
        forward(v, s, geom)
        backward(st, b, geom)
        torch.cuda.synchronize()
    finally:
        del filler
        torch.cuda.empty_cache()
    assert geom.plan.algorithm == ("texture", "registers")
    check_fwd(s.cpu().numpy(), s_ref)
    assert rel_l2(b.cpu().numpy(), b_ref) < TOL


@pytest.mark.parametrize("n,nangles,det", [(256, 360, 384), (512, 720, 768)])
def test_fp32_drift_along_rays(cuda_device, monkeypatch, n, nangles, det):
    """FP32 ray marches against the FP64 oracle on two views (0 and pi) of
    the 256^3 and 512^3 problems, quad forward (FP32 weights, no texture
    quantisation), with the reference's running sample parameter t += h
    ("step") and with t_k = tmin + k h ("exact", the default from 512
    voxels along an axis).  The running sum's rounding shifts the samples
    along the ray (at 256^3 up to 2.2e-4 of a ray's integral, relative);
    the exact parameters remove that drift.  What remains are a few rays
    whose FP32 sample count ceil((tmax - tmin) |d|) rounds to the other
    integer than in FP64 (the reference's set-up in FP32 operations) and
    so hold one sample more or less, ~1e-3 of their integral: the test
    bounds the 99.9th percentile of the per-ray error, the maximum is
    printed."""
    g = cone_config(n, nangles, det)
    g["angles"] = np.asarray(g["angles"])[:: nangles // 2].copy()
    ph = ellipsoids_3d(n, n).numpy()
    ref = None
    err = {}
    for mode in ("step", "exact"):
        monkeypatch.setenv("CURADON_GB300_ALGO", f"t3d={mode}")
        geom = make(g, cuda_device)
        geom.plan.set_algorithm(forward="quad")
        monkeypatch.delenv("CURADON_GB300_ALGO")
        s = run_fwd(geom, ph, cuda_device)
        if ref is None:
            ref = oracle.fwd3d(g, ph, sino0=np.full(geom.sinogram_shape(), SENTINEL))
        both = (s != SENTINEL) & (ref != SENTINEL)
        e = rel_l2(s[both], ref[both])
        big = both & (np.abs(ref) > 1e-2 * np.abs(ref[both]).max())
        r = np.abs(s[big] - ref[big]) / np.abs(ref[big])
        p999 = np.quantile(r, 0.999)
        err[mode] = (e, p999)
        print(f"n={n} {mode}: FP32 vs FP64 rel-L2 {e:.2e} max-abs "
              f"{max_abs(s[both], ref[both]):.2e} per-ray relative 99.9 % {p999:.2e} "
              f"max {r.max():.2e}")
        assert e < 1e-4
    assert err["exact"][0] <= err["step"][0]
    assert err["exact"][1] <= err["step"][1]
    assert err["exact"][0] < 4e-5 and err["exact"][1] < 1e-4


@pytest.mark.parametrize("algo", ["mixed", "quad"])
def test_forward_two_samples_per_iteration_same_bits(cuda_device, monkeypatch, algo):
    """The quad / mixed forward takes two samples per loop iteration with both
    samples' loads in flight (default); the same samples are summed in the
    same order as one per iteration (CURADON_GB300_ALGO fwd3d_unroll=1), so
    the sinograms are equal bit for bit, hit/miss included."""
    shape, nangles, det = (33, 40, 28), 37, 70
    g = cone_config(shape[0], nangles, det)
    g["vol_shape"] = shape
    ph = ellipsoids_3d(shape, 8).numpy()
    out = []
    for unroll in ("1", "2"):
        monkeypatch.setenv("CURADON_GB300_ALGO", f"fwd3d={algo},fwd3d_unroll={unroll}")
        geom = make(g, cuda_device)
        geom.plan
        monkeypatch.delenv("CURADON_GB300_ALGO")
        out.append(run_fwd(geom, ph, cuda_device))
    assert np.array_equal(out[0], out[1])
