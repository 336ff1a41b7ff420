"""Batched 3D operators (``Batch3d``, ``cg_batch3d_*``): a few launches per
direction for many cone-beam problems of mixed volume and detector sizes,
view counts and geometries.

The batched kernels run the single-problem block code (quad forward with the
plan's texture warps, axial or general backprojection) on each problem's
buffers with the problem's own block index, so results must equal the
single-problem operators bit for bit; CUDA-graph replay must equal direct
calls, and the autograd wrapper's gradient must be the batched
backprojection (or, matched, the batched adjoint, which passes the dot
test)."""
import numpy as np
import pytest
import torch

from curadon_gb300 import ConeGeometry
from curadon_gb300.batch import Batch3d, BatchProjector

pytestmark = pytest.mark.gpu


def _angles(n, tilt=0.0):
    a = np.linspace(0, 2 * np.pi, n, endpoint=False).astype(np.float32)
    if tilt == 0.0:
        return a
    return np.vstack([a, np.full(n, tilt, np.float32), np.zeros(n, np.float32)])


def mixed_problems(dev, seed=0):
    """Non-cubic volumes, other detector shapes and spacings, 800 views (the
    axial backprojection's views come in launches of 768), a tilted
    detector and a tilted orbit (the general backprojection), a plan set to
    the quad forward (no texture warps) and one set to the texture forward
    (the batch runs its quads)."""
    g = torch.Generator(device="cpu").manual_seed(seed)
    d = dev.index or 0
    specs = [
        dict(vol_shape=(40, 48, 56), det_shape=(64, 80), angles=_angles(72)),
        dict(vol_shape=(64, 64, 64), det_shape=(96, 96), angles=_angles(90)),
        dict(vol_shape=(24, 24, 24), det_shape=(36, 40), angles=_angles(800)),
        dict(vol_shape=(48, 40, 32), det_shape=(72, 64), angles=_angles(60),
             det_rotation=(0.02, 0.01, 0.03)),
        dict(vol_shape=(32, 32, 32), det_shape=(48, 48), angles=_angles(50, tilt=0.05)),
        dict(vol_shape=(33, 47, 29), det_shape=(50, 70), angles=_angles(45),
             det_spacing=(1.25, 1.75)),
        dict(vol_shape=(36, 36, 36), det_shape=(54, 54), angles=_angles(40)),
    ]
    forced = {5: "quad", 6: "texture"}
    geoms, vols, sinos = [], [], []
    for k, sp in enumerate(specs):
        n = max(sp["vol_shape"])
        kw = dict(DSD=3.0 * n, DSO=2.0 * n, det_spacing=(1.5, 1.5), device=d)
        kw.update(sp)
        geom = ConeGeometry(**kw)
        if k in forced:
            geom.plan.set_algorithm(forward=forced[k])
        geoms.append(geom)
        vols.append(torch.rand(sp["vol_shape"], generator=g).to(dev))
        sinos.append(torch.zeros(geom.sinogram_shape(), device=dev))
    return geoms, vols, sinos


def single_results(geoms, vols, sino_in, dev, zero_init=False):
    """The single-problem operators on fresh plans with the algorithms the
    batch runs (the quad forward where a plan was set to another); the
    backprojection adds into a copy of the volume (or into zeros)."""
    fw, bw = [], []
    for g, v, s_in in zip(geoms, vols, sino_in):
        p = g._make_plan()
        algo = g.plan.algorithm[0]
        p.set_algorithm(forward=algo if algo in ("quad", "mixed") else "quad")
        s = torch.zeros(g.sinogram_shape(), device=dev)
        p.forward(v, s)
        b = torch.zeros_like(v) if zero_init else v.clone()
        p.backward(b, s_in)
        fw.append(s)
        bw.append(b)
    torch.cuda.synchronize()
    return fw, bw


def test_batch3d_equals_single_problem_operators(cuda_device):
    geoms, vols, sinos = mixed_problems(cuda_device)
    sino_in = [torch.rand(s.shape, device=cuda_device) for s in sinos]
    fw, bw = single_results(geoms, vols, sino_in, cuda_device)
    b = Batch3d(geoms, vols, sinos)
    b.forward()
    torch.cuda.synchronize()
    for k, (s, r) in enumerate(zip(sinos, fw)):
        assert r.abs().max() > 0, k
        assert torch.equal(s, r), k
    outs = [v.clone() for v in vols]
    b2 = Batch3d(geoms, outs, sino_in)
    b2.backward()
    torch.cuda.synchronize()
    for k, (o, r) in enumerate(zip(outs, bw)):
        assert torch.equal(o, r), k


def test_batch3d_set_active(cuda_device):
    """Only problems [0, active) run."""
    geoms, vols, sinos = mixed_problems(cuda_device, seed=1)
    b = Batch3d(geoms, vols, sinos)
    b.set_active(3)
    b.forward()
    torch.cuda.synchronize()
    assert all(s.abs().max() > 0 for s in sinos[:3])
    assert all(s.abs().max() == 0 for s in sinos[3:])
    with pytest.raises(Exception):
        b.set_active(len(geoms) + 1)


def test_batch3d_graph_replay(cuda_device):
    """One forward + backprojection captured once and replayed (the texture
    warps' array copies are captured too) equals direct calls."""
    geoms, vols, sinos = mixed_problems(cuda_device, seed=2)
    outs = [torch.zeros_like(v) for v in vols]
    bf = Batch3d(geoms, vols, sinos)
    bb = Batch3d(geoms, outs, sinos)

    def step():
        bf.forward()
        bb.backward()

    step()
    torch.cuda.synchronize()
    want_s = [s.clone() for s in sinos]
    want_v = [o.clone() for o in outs]
    for o in outs:
        o.zero_()
    graph = torch.cuda.CUDAGraph()
    side = torch.cuda.Stream(cuda_device)
    side.wait_stream(torch.cuda.current_stream(cuda_device))
    with torch.cuda.stream(side):
        with torch.cuda.graph(graph, stream=side):
            step()
    torch.cuda.current_stream(cuda_device).wait_stream(side)
    for s in sinos:
        s.zero_()
    for o in outs:
        o.zero_()
    graph.replay()
    torch.cuda.synchronize()
    for s, w in zip(sinos, want_s):
        assert torch.equal(s, w)
    for o, w in zip(outs, want_v):
        assert torch.equal(o, w)


def test_batch3d_projector_autograd(cuda_device):
    """``BatchProjector`` over cone geometries: y = A x for every problem, and
    the gradient of <y, w> is the backprojection of w, problem by problem."""
    geoms, vols, _ = mixed_problems(cuda_device, seed=3)
    proj = BatchProjector(geoms, cuda_device)
    x = torch.cat([v.reshape(-1) for v in vols]).requires_grad_(True)
    y = proj(x)
    w = torch.rand_like(y)
    (y * w).sum().backward()
    torch.cuda.synchronize()
    ws = proj.split_sinograms(w)
    fw, bw = single_results(geoms, vols, ws, cuda_device, zero_init=True)
    for k, (ys, r) in enumerate(zip(proj.split_sinograms(y.detach()), fw)):
        assert torch.equal(ys, r), k
    for k, (gv, r) in enumerate(zip(proj.split_volumes(x.grad), bw)):
        assert torch.equal(gv, r), k


def test_batch3d_matched_adjoint(cuda_device):
    """The batched matched adjoint equals the single-problem one up to the
    order of its atomic additions and passes the dot test <A x, y> =
    <x, A^T y> per problem to 1e-5 relative (A the quad forward without
    texture warps); ``BatchProjector(..., matched=True)``'s gradient is it."""
    from curadon_gb300 import adjoint

    geoms, vols, _ = mixed_problems(cuda_device, seed=4)
    gen = torch.Generator(device="cpu").manual_seed(5)
    ys = [torch.rand(g.sinogram_shape(), generator=gen).to(cuda_device) for g in geoms]
    proj = BatchProjector(geoms, cuda_device, matched=True)
    x = torch.cat([v.reshape(-1) for v in vols]).requires_grad_(True)
    ax = proj(x)
    w = torch.cat([y.reshape(-1) for y in ys])
    (ax * w).sum().backward()
    torch.cuda.synchronize()
    for k, (g, v, y, a_x, aty) in enumerate(zip(geoms, vols, ys, proj.split_sinograms(ax.detach()),
                                                 proj.split_volumes(x.grad))):
        lhs = float((a_x.double() * y.double()).sum())
        rhs = float((v.double() * aty.double()).sum())
        assert abs(lhs - rhs) <= 1e-5 * abs(lhs), (k, lhs, rhs)
        single = adjoint(y, torch.zeros_like(v), g)
        torch.cuda.synchronize()
        assert torch.allclose(aty, single, rtol=1e-5, atol=1e-5 * float(single.abs().max())), k
