"""GPU parity of the 2D fan-beam operators (through the C ABI).

Tolerance: relative L2 <= 1e-3 against the reference's own operators and
against the FP64 oracle (the bar of the drop-in contract); max abs error is
printed.  The per-view geometry tables must equal the reference's bit for
bit, because their rounding is amplified by the detector index."""
import numpy as np
import pytest
import torch

import oracle
from conftest import load_golden, max_abs, rel_l2
from curadon_gb300 import FanGeometry, backward, backward_2d, forward, forward_2d, plan_2d
from curadon_gb300.backend import BACKWARD_2D, FORWARD_2D
from curadon_gb300.phantom import ellipses_2d, fan_config

pytestmark = pytest.mark.gpu
TOL = 1e-3


def make(g, dev):
    kw = {k: g[k] for k in ("DSD", "DSO", "angles", "vol_shape", "det_shape")}
    for k in ("det_spacing", "det_offset", "vol_spacing", "vol_offset"):
        if k in g:
            kw[k] = g[k]
    return FanGeometry(**kw, device=dev.index or 0)


def run_fwd(geom, vol, dev):
    v = torch.as_tensor(vol, device=dev).contiguous()
    s = torch.full(geom.sinogram_shape(), 123.0, device=dev)
    forward(v, s, geom)
    torch.cuda.synchronize()
    return s.cpu().numpy()


def run_bwd(geom, sino, dev, vol0=None):
    s = torch.as_tensor(sino, device=dev, dtype=torch.float32).contiguous()
    v = (torch.zeros(tuple(geom.vol_shape), device=dev) if vol0 is None
         else torch.as_tensor(vol0, device=dev, dtype=torch.float32).clone())
    backward(s, v, geom)
    torch.cuda.synchronize()
    return v.cpu().numpy()


@pytest.mark.parametrize("case", ["fan_cfg0", "fan_var"])
def test_against_golden(cuda_device, case):
    z, g = load_golden(case)
    geom = make(g, cuda_device)
    src, u0, du = geom.plan.tables()
    assert np.array_equal(src, z["sources"]) and np.array_equal(u0, z["u_origins"])
    assert np.array_equal(du, z["delta_us"]), max_abs(du, z["delta_us"])
    s = run_fwd(geom, z["volume"], cuda_device)
    e = rel_l2(s, z["sino_ref"])
    print(f"{case} fwd rel-L2 {e:.2e} max-abs {max_abs(s, z['sino_ref']):.2e}")
    assert e < TOL
    b = run_bwd(geom, z["sino_ref"], cuda_device)
    e = rel_l2(b, z["bwd_ref"])
    print(f"{case} bwd rel-L2 {e:.2e} max-abs {max_abs(b, z['bwd_ref']):.2e}")
    assert e < TOL


@pytest.mark.parametrize("n,nangles", [(64, 360), (96, 50), (128, 128), (200, 1500)])
def test_against_oracle(cuda_device, n, nangles):
    g = fan_config(n, nangles)
    geom = make(g, cuda_device)
    ph = ellipses_2d(n, n).numpy()
    s = run_fwd(geom, ph, cuda_device)
    so = oracle.fwd2d(g, ph)
    assert rel_l2(s, so) < TOL, rel_l2(s, so)
    b = run_bwd(geom, so.astype(np.float32), cuda_device)
    bo = oracle.bwd2d(g, so.astype(np.float32))
    assert rel_l2(b, bo) < TOL, rel_l2(b, bo)


@pytest.mark.parametrize("algo", FORWARD_2D)
@pytest.mark.parametrize("n,nangles,det", [(300, 240, None), (180, 97, 700)])
def test_forward_algorithms(cuda_device, algo, n, nangles, det):
    """Every selectable forward agrees with the oracle (wide detectors give
    views whose rays change stepping axis inside one block)."""
    g = fan_config(n, nangles, det)
    geom = make(g, cuda_device)
    geom.plan.set_algorithm(forward=algo)
    ph = ellipses_2d(n, n).numpy()
    s = run_fwd(geom, ph, cuda_device)
    e = rel_l2(s, oracle.fwd2d(g, ph))
    print(f"{algo} n={n} fwd rel-L2 {e:.2e}")
    assert e < TOL


@pytest.mark.parametrize("algo", BACKWARD_2D)
@pytest.mark.parametrize("n,nangles", [(300, 240), (64, 2100)])
def test_backward_algorithms(cuda_device, algo, n, nangles):
    """Every selectable backprojection agrees with the oracle, including past
    the layered texture's 2048 views."""
    g = fan_config(n, nangles)
    geom = make(g, cuda_device)
    geom.plan.set_algorithm(backward=algo)
    rng = np.random.default_rng(n + nangles)
    sino = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    b = run_bwd(geom, sino, cuda_device)
    e = rel_l2(b, oracle.bwd2d(g, sino))
    print(f"{algo} n={n} views={nangles} bwd rel-L2 {e:.2e}")
    assert e < TOL


@pytest.mark.parametrize("n", [256, 512, 1024, 2048])
def test_against_reference_sweep(cuda_device, ref_ops, n):
    """The n-sweep workload at full size against the reference's kernels."""
    g = fan_config(n)
    geom = make(g, cuda_device)
    h, nv = ref_ops.plan2d(g)
    try:
        rs, ru, rd = ref_ops.plan2d_tables(h, nv)
        src, u0, du = geom.plan.tables()
        assert np.array_equal(src, rs) and np.array_equal(u0, ru) and np.array_equal(du, rd)
        v = ellipses_2d(n, n, device=cuda_device).contiguous()
        s_ref = torch.zeros(geom.sinogram_shape(), device=cuda_device)
        ref_ops.forward2d(h, v.data_ptr(), s_ref.data_ptr())
        ref_ops.sync()
        s = torch.zeros_like(s_ref)
        forward(v, s, geom)
        torch.cuda.synchronize()
        e = rel_l2(s.cpu(), s_ref.cpu())
        print(f"n={n} fwd rel-L2 {e:.2e} max-abs {max_abs(s.cpu(), s_ref.cpu()):.2e}")
        assert e < TOL
        # above 1024 views the reference's backprojection launches its chunks on
        # unordered streams that share one texture and the volume, so they race
        if nv <= 1024:
            b_ref = torch.zeros_like(v)
            ref_ops.backward2d(h, b_ref.data_ptr(), s_ref.data_ptr())
            ref_ops.sync()
            b = torch.zeros_like(v)
            backward(s_ref, b, geom)
            torch.cuda.synchronize()
            e = rel_l2(b.cpu(), b_ref.cpu())
            print(f"n={n} bwd rel-L2 {e:.2e} max-abs {max_abs(b.cpu(), b_ref.cpu()):.2e}")
            assert e < TOL
    finally:
        ref_ops.destroy2d(h)


def test_edge_geometries(cuda_device):
    cases = [
        dict(fan_config(1, 3, 1, 1.0, 10.0, 20.0)),                       # 1x1 image, 1 cell
        dict(fan_config(17, 1, 5, 0.5, 40.0, 60.0)),                      # one view, odd sizes
        dict(fan_config(33, 7, 64, 2.0, 60.0, 100.0), vol_shape=(33, 45),
             vol_spacing=(0.7, 1.3), vol_offset=(-4.0, 2.5), det_offset=3.0),
        dict(fan_config(40, 9, 30, 1.0, 500.0, 700.0), vol_offset=(1000.0, 0.0)),  # all miss
    ]
    for g in cases:
        geom = make(g, cuda_device)
        H, W = g["vol_shape"]
        ph = np.random.default_rng(H * W).uniform(0, 1, (H, W)).astype(np.float32)
        s = run_fwd(geom, ph, cuda_device)
        so = oracle.fwd2d(g, ph)
        if np.linalg.norm(so) == 0:
            assert np.all(s == 0)
        else:
            assert rel_l2(s, so) < TOL, (g["vol_shape"], rel_l2(s, so))
        b = run_bwd(geom, so.astype(np.float32), cuda_device)
        bo = oracle.bwd2d(g, so.astype(np.float32))
        assert rel_l2(b, bo) < TOL or np.linalg.norm(bo) == 0


def test_backward_accumulates_and_is_linear(cuda_device):
    g = fan_config(128, 96)
    geom = make(g, cuda_device)
    rng = np.random.default_rng(0)
    s1 = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    s2 = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    v0 = rng.uniform(0, 1, (128, 128)).astype(np.float32)
    b1, b2 = run_bwd(geom, s1, cuda_device), run_bwd(geom, s2, cuda_device)
    b12 = run_bwd(geom, 2 * s1 + 3 * s2, cuda_device)
    assert rel_l2(b12, 2 * b1 + 3 * b2) < 1e-5
    bacc = run_bwd(geom, s1, cuda_device, vol0=v0)
    assert rel_l2(bacc, b1 + v0) < 1e-6


def test_forward_linear_and_deterministic(cuda_device):
    g = fan_config(256)
    geom = make(g, cuda_device)
    x = ellipses_2d(256, 1).numpy()
    y = ellipses_2d(256, 2).numpy()
    a, b = run_fwd(geom, x, cuda_device), run_fwd(geom, y, cuda_device)
    assert rel_l2(run_fwd(geom, 2 * x - y, cuda_device), 2 * a - b) < 1e-5
    assert np.array_equal(a, run_fwd(geom, x, cuda_device))


def test_native_api_and_errors(cuda_device):
    g = fan_config(32, 8)
    plan = plan_2d(0, 32, (32, 32), (1.0, 1.0), (0.0, 0.0), 32, g["det_shape"], 1.5, 0.0,
                   g["DSO"], g["DSD"], g["angles"], 0.0, 0.0)
    v = torch.rand(32, 32, device=cuda_device)
    s = torch.zeros(8, g["det_shape"], device=cuda_device)
    forward_2d(v, s, plan)
    backward_2d(v, s, plan)
    plan.forward_block_y = 2
    plan.forward_block_x = 64
    assert (plan.forward_block_x, plan.forward_block_y) == (64, 2)
    forward_2d(v, s, plan)
    with pytest.raises(TypeError):
        forward_2d(v.double(), s, plan)
    with pytest.raises(TypeError):
        forward_2d(v.cpu(), s, plan)
    with pytest.raises(ValueError):
        forward_2d(v[:16].contiguous(), s, plan)
    with pytest.raises(TypeError):
        forward_2d(v.t(), s, plan)
    with pytest.raises(AttributeError):
        plan_2d(0, 8, (32, 32), (1.0, 1.0), (0.0, 0.0), 32, 10, 1.5, 0.0, [1.0], [2.0], [0.0])
    with pytest.raises(ValueError):
        plan.forward_block_x = 48


def test_runs_on_the_current_stream(cuda_device):
    g = fan_config(256)
    geom = make(g, cuda_device)
    x = ellipses_2d(256, 4, device=cuda_device)
    expect = torch.zeros(geom.sinogram_shape(), device=cuda_device)
    forward(x, expect, geom)
    st = torch.cuda.Stream()
    with torch.cuda.stream(st):
        y = x * 1.0
        s = torch.zeros_like(expect)
        forward(y, s, geom)
        r = s.sum()
    st.synchronize()
    assert torch.equal(s, expect) and float(r) == pytest.approx(float(expect.sum()), rel=1e-6)


def test_algorithm_override_variable(cuda_device):
    """CURADON_GB300_ALGO (comma-separated key=value tokens) sets the
    algorithms of plans made in that process; unknown tokens are ignored."""
    import os
    import subprocess
    import sys
    from pathlib import Path

    code = ("import curadon_gb300 as cg\n"
            "from curadon_gb300.phantom import fan_config\n"
            "print(cg.FanGeometry(**fan_config(64, 30)).plan.algorithm)\n")
    env = dict(os.environ, CURADON_GB300_ALGO="fwd2d=alu,bwd2d=tex,nonsense=1")
    out = subprocess.run([sys.executable, "-c", code], env=env, capture_output=True, text=True,
                         cwd=Path(__file__).resolve().parents[1], timeout=300)
    assert out.returncode == 0, out.stderr
    assert "('registers', 'texture')" in out.stdout, out.stdout


@pytest.mark.parametrize("shape", [27, 48, 68])
def test_staged_backprojector_shapes(cuda_device, monkeypatch, shape):
    """Every compiled variant of the staged backprojector (CURADON_GB300_ALGO
    bwd2d_minb=...: the default and the autotuner's other candidates)
    against the oracle."""
    n, nangles = 256, 150
    g = fan_config(n, nangles)
    monkeypatch.setenv("CURADON_GB300_ALGO", f"bwd2d=smem,bwd2d_minb={shape}")
    geom = FanGeometry(**g, device=cuda_device.index or 0)
    geom.plan
    monkeypatch.delenv("CURADON_GB300_ALGO")
    rng = np.random.default_rng(shape)
    sino = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    b = run_bwd(geom, sino, cuda_device)
    e = rel_l2(b, oracle.bwd2d(g, sino))
    print(f"shape {shape} bwd rel-L2 {e:.2e}")
    assert e < TOL


@pytest.mark.parametrize("shape", [443, 474, 484])
def test_chunked_forward_shapes(cuda_device, monkeypatch, shape):
    """Every compiled shape of the chunked forward (CURADON_GB300_ALGO
    fwd2d=cslab<shape>: the default and the autotuner's other candidates)
    against the oracle, on a wide detector whose bundles hold rays of both
    stepping classes."""
    n, nangles, det = 190, 77, 600
    g = fan_config(n, nangles, det)
    monkeypatch.setenv("CURADON_GB300_ALGO", f"fwd2d=cslab{shape}")
    geom = FanGeometry(**g, device=cuda_device.index or 0)
    assert geom.plan.algorithm[0] == "chunked"
    monkeypatch.delenv("CURADON_GB300_ALGO")
    ph = ellipses_2d(n, 4).numpy()
    s = run_fwd(geom, ph, cuda_device)
    e = rel_l2(s, oracle.fwd2d(g, ph))
    print(f"shape {shape} fwd rel-L2 {e:.2e}")
    assert e < TOL


@pytest.mark.parametrize("n", [1024, 2048])
def test_tma_staging_equals_cp_async_staging(cuda_device, monkeypatch, n):
    """Shape 484 stages the chunk windows with bulk copies of the tensor
    memory access unit (mbarrier completion) instead of per-lane cp.async
    (shape 474); the arithmetic is the same, so the sinograms must be equal
    bit for bit, and no bounded wait may have given up."""
    from curadon_gb300.backend import wait_timeouts

    g = fan_config(n, n // 2)
    ph = torch.as_tensor(ellipses_2d(n, 7).numpy(), device=cuda_device).contiguous()
    out = {}
    wait_timeouts()
    for shape in (474, 484):
        monkeypatch.setenv("CURADON_GB300_ALGO", f"fwd2d=cslab{shape}")
        geom = FanGeometry(**g, device=cuda_device.index or 0)
        geom.plan
        monkeypatch.delenv("CURADON_GB300_ALGO")
        s = torch.zeros(geom.sinogram_shape(), device=cuda_device)
        forward(ph, s, geom)
        torch.cuda.synchronize()
        out[shape] = s
    assert wait_timeouts() == 0
    assert torch.equal(out[474], out[484])


@pytest.mark.parametrize("n,nangles", [(1024, 512), (2048, 300), (333, 77)])
def test_bulk_staged_backprojector_equals_pairwise_staging(cuda_device, monkeypatch, n,
                                                           nangles):
    """Variant 68 stages the window rows with bulk copies (one per view,
    started on 16 bytes, so one pair wider) instead of pair by pair
    (variant 48); the samples and sums are the same, so the volumes must be
    equal bit for bit, and no bounded wait may have given up.  Odd detector
    widths put every other view row on an odd element."""
    from curadon_gb300.backend import wait_timeouts

    g = fan_config(n, nangles)
    rng = np.random.default_rng(n)
    sino = torch.as_tensor(rng.uniform(0, 1, (nangles, g["det_shape"])).astype(np.float32),
                           device=cuda_device)
    out = {}
    wait_timeouts()
    for variant in (48, 68):
        monkeypatch.setenv("CURADON_GB300_ALGO",
                           f"bwd2d=smem,bwd2d_minb={variant},bwd2d_sym=off")
        geom = FanGeometry(**g, device=cuda_device.index or 0)
        geom.plan
        monkeypatch.delenv("CURADON_GB300_ALGO")
        v = torch.zeros(tuple(geom.vol_shape), device=cuda_device)
        backward(sino, v, geom)
        torch.cuda.synchronize()
        out[variant] = v
    assert wait_timeouts() == 0
    assert torch.equal(out[48], out[68])


def test_full_size_backprojection_cross_check(cuda_device):
    """n=2048 with 2048 views, where the reference's backprojection cannot be
    run as a check (its chunks race above 1024 views): the default staged
    backprojector against this library's texture-unit one, an independent
    kernel with the reference's 8-bit texture weights; and linearity."""
    n = 2048
    g = fan_config(n)
    geom = make(g, cuda_device)
    rng = np.random.default_rng(2048)
    s1 = torch.as_tensor(rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32),
                         device=cuda_device)
    s2 = torch.as_tensor(rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32),
                         device=cuda_device)
    b1 = torch.zeros((n, n), device=cuda_device)
    backward(s1, b1, geom)
    other = make(g, cuda_device)
    other.plan.set_algorithm(backward="texture")
    bt = torch.zeros_like(b1)
    backward(s1, bt, other)
    b12 = torch.zeros_like(b1)
    backward(2 * s1 - s2, b12, geom)
    b2 = torch.zeros_like(b1)
    backward(s2, b2, geom)
    torch.cuda.synchronize()
    e = rel_l2(b1.cpu(), bt.cpu())
    print(f"n=2048 staged vs texture bwd rel-L2 {e:.2e} max-abs {max_abs(b1.cpu(), bt.cpu()):.2e}")
    assert e < TOL
    assert rel_l2(b12.cpu(), (2 * b1 - b2).cpu()) < 1e-5


def _bwd_with(g, sino, dev, monkeypatch, algo=None):
    if algo:
        monkeypatch.setenv("CURADON_GB300_ALGO", algo)
    geom = FanGeometry(**g, device=dev.index or 0)
    geom.plan
    if algo:
        monkeypatch.delenv("CURADON_GB300_ALGO")
    v = torch.zeros(tuple(geom.vol_shape), device=dev)
    backward(torch.as_tensor(sino, device=dev), v, geom)
    torch.cuda.synchronize()
    return v.cpu()


@pytest.mark.parametrize("n,nangles,reverse", [(64, 360, False), (256, 256, False),
                                               (1000, 500, False), (512, 512, True),
                                               (2048, 2048, False)])
def test_quarter_turn_backprojection(cuda_device, monkeypatch, n, nangles, reverse):
    """Circular orbits whose views come in quarter turns (n views spaced
    evenly over a full turn, n divisible by 4) on square centred images take
    the staged backprojection over the symmetry (one projective evaluation
    for four (pixel, view) pairs; reversed angles turn the other way): it
    differs from the per-view evaluation only in the last bits of the views'
    tables, and matches the oracle."""
    g = fan_config(n, nangles)
    if reverse:
        g["angles"] = np.ascontiguousarray(-g["angles"])
    rng = np.random.default_rng(n + nangles)
    sino = rng.uniform(0, 1, (nangles, g["det_shape"])).astype(np.float32)
    # forced on (by default only images whose first quadrant fills the GPU,
    # from about 1536^2 pixels, take it)
    sym = _bwd_with(g, sino, cuda_device, monkeypatch, "bwd2d_sym=on")
    per_view = _bwd_with(g, sino, cuda_device, monkeypatch, "bwd2d_sym=off")
    default = _bwd_with(g, sino, cuda_device, monkeypatch)
    assert torch.equal(default, sym if n >= 2048 else per_view)
    e = rel_l2(sym, per_view)
    print(f"n={n} views={nangles}: symmetric vs per-view rel-L2 {e:.2e} "
          f"max-abs {max_abs(sym, per_view):.2e}")
    assert not torch.equal(sym, per_view)  # the symmetric kernel ran
    assert e < 2e-5
    if n <= 512:
        eo = rel_l2(sym, oracle.bwd2d(g, sino))
        print(f"  vs oracle {eo:.2e}")
        assert eo < TOL


@pytest.mark.parametrize("case", ["views", "offset", "rect"])
def test_no_quarter_turn_without_the_symmetry(cuda_device, monkeypatch, case):
    """Geometries without the symmetry (views not in quarter turns, an
    off-centre image, a rectangular image) take the per-view kernel even
    when the symmetric one is forced on: equal bit for bit with it off."""
    if case == "views":
        g = fan_config(128, 90)
    elif case == "offset":
        g = dict(fan_config(128, 128), vol_offset=(3.0, -2.0))
    else:
        g = dict(fan_config(128, 128), vol_shape=(128, 96))
    rng = np.random.default_rng(7)
    sino = rng.uniform(0, 1, (len(g["angles"]), g["det_shape"])).astype(np.float32)
    a = _bwd_with(g, sino, cuda_device, monkeypatch, "bwd2d_sym=on")
    b = _bwd_with(g, sino, cuda_device, monkeypatch, "bwd2d_sym=off")
    assert torch.equal(a, b)
