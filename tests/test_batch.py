"""Batched 2D operators (``Batch2d``, ``cg_batch2d_*``): one launch pair per
direction for many problems of mixed sizes and geometries.

The batched kernels run the same per-ray / per-tile code as the single-problem
texture or register forward and staged backprojection, so results must be
equal bit for bit; CUDA-graph replay of a batch must equal direct calls."""
import numpy as np
import pytest
import torch

from curadon_gb300 import FanGeometry, FanVecGeometry, backward, forward
from curadon_gb300.batch import Batch2d
from curadon_gb300.phantom import ellipses_2d, fan_config

pytestmark = pytest.mark.gpu


def mixed_problems(dev, seed=0):
    rng = np.random.default_rng(seed)
    geoms, vols, sinos = [], [], []
    for k, n in enumerate([128, 192, 256, 384, 130, 257, 96, 512]):
        nangles = int(rng.integers(60, 400))
        g = fan_config(n, nangles)
        if k % 3 == 2:  # a jittered vector geometry among the circular ones
            v = np.asarray(FanGeometry(**g).to_vec())
            v[:, 4:] *= g["det_spacing"]
            v[:, :4] += rng.normal(0, 0.5, (nangles, 4))
            geom = FanVecGeometry(g["vol_shape"], g["det_shape"], v, device=dev.index or 0)
        else:
            geom = FanGeometry(**g, device=dev.index or 0)
        geoms.append(geom)
        vols.append(ellipses_2d(n, k, device=dev).contiguous())
        sinos.append(torch.zeros(geom.sinogram_shape(), device=dev))
    return geoms, vols, sinos


def reference_results(geoms, vols, dev, forward_algo="texture"):
    """Single-problem operators with the batch's algorithms."""
    fw, bw = [], []
    for g, v in zip(geoms, vols):
        p = g._make_plan()
        p.set_algorithm(forward=forward_algo, backward="shared")
        from curadon_gb300.backend import backward_2d, forward_2d

        s = torch.zeros(g.sinogram_shape(), device=dev)
        forward_2d(v, s, p)
        b = v.clone()
        backward_2d(b, s, p)
        fw.append(s)
        bw.append(b)
    torch.cuda.synchronize()
    return fw, bw


@pytest.mark.parametrize("algo", ["texture", "registers"])
def test_batch_equals_single_problem_operators(cuda_device, algo):
    geoms, vols, sinos = mixed_problems(cuda_device)
    fw, bw = reference_results(geoms, vols, cuda_device, algo)
    b = Batch2d(geoms, vols, sinos, forward=algo)
    assert b.forward_algorithm == algo
    b.forward()
    torch.cuda.synchronize()
    for s, r in zip(sinos, fw):
        assert torch.equal(s, r)
    outs = [v.clone() for v in vols]
    b2 = Batch2d(geoms, outs, sinos)
    b2.backward()
    torch.cuda.synchronize()
    for o, r in zip(outs, bw):
        assert torch.equal(o, r)


@pytest.mark.parametrize("algo", ["texture", "registers"])
def test_batch_graph_replay(cuda_device, algo):
    """A forward + backprojection iteration captured once and replayed (the
    texture forward's per-problem array copies are captured too)."""
    geoms, vols, sinos = mixed_problems(cuda_device, seed=1)
    outs = [torch.zeros_like(v) for v in vols]
    bf = Batch2d(geoms, vols, sinos, forward=algo)
    bb = Batch2d(geoms, outs, sinos)
    # first calls outside capture (plans and scratch exist by now)
    bf.forward(), bb.backward()
    torch.cuda.synchronize()
    direct = [o.clone() for o in outs]
    for o in outs:
        o.zero_()
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(graph, stream=s):
            bf.forward()
            bb.backward()
    torch.cuda.current_stream().wait_stream(s)
    for o in outs:
        o.zero_()
    graph.replay()
    torch.cuda.synchronize()
    for o, d in zip(outs, direct):
        assert torch.equal(o, d)


def test_batch_plans_forward_equals_each_plans_default(cuda_device):
    """forward="plans": problems from 704^2 pixels through the batched chunked
    forward (one re-layout and one bundle launch for all of them), the others
    through the texture march -- each problem's result equal, bit for bit, to
    its plan's own default forward; also inside a CUDA graph."""
    rng = np.random.default_rng(12)
    geoms, vols, sinos = [], [], []
    for k, n in enumerate([1024, 128, 768, 256, 720, 96]):
        nangles = int(rng.integers(90, 240))
        g = fan_config(n, nangles)
        if k == 2:  # a jittered vector geometry among the big ones
            v = np.asarray(FanGeometry(**g).to_vec())
            v[:, 4:] *= g["det_spacing"]
            v[:, :4] += rng.normal(0, 0.5, (nangles, 4))
            geom = FanVecGeometry(g["vol_shape"], g["det_shape"], v, device=cuda_device.index or 0)
        else:
            geom = FanGeometry(**g, device=cuda_device.index or 0)
        geoms.append(geom)
        vols.append(ellipses_2d(n, k, device=cuda_device).contiguous())
        sinos.append(torch.zeros(geom.sinogram_shape(), device=cuda_device))
    expect = []
    for g, v in zip(geoms, vols):
        p = g._make_plan()
        assert p.algorithm[0] == ("chunked" if v.numel() >= 704 * 704 else "texture")
        from curadon_gb300.backend import forward_2d

        s = torch.zeros(g.sinogram_shape(), device=cuda_device)
        forward_2d(v, s, p)
        expect.append(s)
    b = Batch2d(geoms, vols, sinos, forward="plans")
    assert b.forward_algorithm == "plans"
    b.forward()
    torch.cuda.synchronize()
    for i, (s, e) in enumerate(zip(sinos, expect)):
        assert torch.equal(s, e), i
    for s in sinos:
        s.zero_()
    graph = torch.cuda.CUDAGraph()
    st = torch.cuda.Stream()
    st.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(st), torch.cuda.graph(graph, stream=st):
        b.forward()
    torch.cuda.current_stream().wait_stream(st)
    graph.replay()
    torch.cuda.synchronize()
    for i, (s, e) in enumerate(zip(sinos, expect)):
        assert torch.equal(s, e), i
    # the first problems only (a resident batch serving fewer requests)
    for s in sinos:
        s.zero_()
    b.set_active(3)
    b.forward()
    torch.cuda.synchronize()
    for i in range(3):
        assert torch.equal(sinos[i], expect[i]), i
    assert all(float(s.abs().sum()) == 0.0 for s in sinos[3:])


def test_batch_rejects_bad_input(cuda_device):
    g = FanGeometry(**fan_config(64, 30), device=cuda_device.index or 0)
    v = torch.zeros((64, 64), device=cuda_device)
    s = torch.zeros(g.sinogram_shape(), device=cuda_device)
    with pytest.raises(ValueError):
        Batch2d([g], [torch.zeros((32, 32), device=cuda_device)], [s])
    with pytest.raises(ValueError):
        Batch2d([], [], [])
    with pytest.raises(ValueError):
        Batch2d([g], [v], [s], forward="chunked")
    # the same geometry twice gets a private plan for its second use
    b = Batch2d([g, g], [v, v.clone()], [s, s.clone()])
    b.forward()
    torch.cuda.synchronize()


def jittered_batch(dev, count=8, seed=3):
    """``count`` fan-beam problems of the batched workload's kind: mixed n,
    180..720 views, per-view Gaussian jitter (sigma 0.5 px) on source and
    detector positions in full vector form."""
    rng = np.random.default_rng(seed)
    geoms = []
    for k in range(count):
        n = int(rng.choice([64, 96, 128, 192, 256]))
        nangles = int(rng.integers(180, 721))
        g = fan_config(n, nangles)
        v = np.asarray(FanGeometry(**g).to_vec())
        v[:, 4:] *= g["det_spacing"]
        v[:, :4] += rng.normal(0.0, 0.5, (nangles, 4))
        geoms.append(FanVecGeometry(g["vol_shape"], g["det_shape"], v, device=dev.index or 0))
    return geoms


def test_batch_matched_adjoint_dot_test(cuda_device):
    """<A x, y> = <x, A^T y> for the batched register forward and the batched
    matched adjoint on a jittered batch of 8 problems (float64 sums)."""
    from curadon_gb300.batch import BatchProjector

    geoms = jittered_batch(cuda_device)
    proj = BatchProjector(geoms, cuda_device, matched=True)
    g = torch.Generator(device=cuda_device).manual_seed(5)
    x = torch.rand(proj.X.shape, device=cuda_device, generator=g)
    y = torch.rand(proj.S.shape, device=cuda_device, generator=g)
    with torch.no_grad():
        ax = proj(x)
    aty = proj.adjoint(y)
    lhs = float((ax.double() * y.double()).sum())
    rhs = float((x.double() * aty.double()).sum())
    rel = abs(lhs - rhs) / abs(lhs)
    print(f"batched dot test: <Ax,y> {lhs:.8e} <x,A^T y> {rhs:.8e} rel {rel:.2e}")
    assert rel <= 1e-5
    # per problem: the dot test again and the single-problem adjoint
    from curadon_gb300.backend import adjoint_2d

    for i, geom in enumerate(geoms):
        xi, yi = proj.split_volumes(x)[i], proj.split_sinograms(y)[i]
        ai = proj.split_sinograms(ax)[i]
        ti = proj.split_volumes(aty)[i]
        l_, r_ = float((ai.double() * yi.double()).sum()), float((xi.double() * ti.double()).sum())
        assert abs(l_ - r_) / abs(l_) <= 1e-5, (i, l_, r_)
        single = torch.zeros_like(xi)
        adjoint_2d(single, yi.contiguous(), geom.plan)
        torch.cuda.synchronize()
        e = float((single - ti).norm() / single.norm())
        assert e <= 1e-5, (i, e)


def test_batch_autograd_gradient_against_finite_differences(cuda_device):
    """The gradient of L(x) = 1/2 ||A x - y||^2 through the batched autograd
    function (matched adjoint) against central finite differences along
    random directions, on a jittered batch of 8 problems."""
    from curadon_gb300.batch import BatchProjector

    geoms = jittered_batch(cuda_device, seed=4)
    proj = BatchProjector(geoms, cuda_device, matched=True)
    g = torch.Generator(device=cuda_device).manual_seed(6)
    x0 = torch.rand(proj.X.shape, device=cuda_device, generator=g)
    y = torch.rand(proj.S.shape, device=cuda_device, generator=g) * 50

    def loss(x):
        r = proj(x) - y
        return 0.5 * (r.double() ** 2).sum()

    x = x0.clone().requires_grad_(True)
    L = loss(x)
    L.backward()
    grad = x.grad.double()
    for k in range(3):
        d = torch.randn(proj.X.shape, device=cuda_device, generator=g)
        eps = 1e-2
        with torch.no_grad():
            fd = float((loss(x0 + eps * d) - loss(x0 - eps * d)) / (2 * eps))
        an = float((grad * d.double()).sum())
        rel = abs(fd - an) / abs(an)
        print(f"direction {k}: autograd {an:.6e} finite differences {fd:.6e} rel {rel:.2e}")
        assert rel <= 2e-3


def test_batch_unrolled_gradient_descent_graph_equals_eager(cuda_device):
    """Ten gradient-descent steps on 1/2 ||A x - y||^2 through torch.autograd
    over a jittered batch: one step captured in a CUDA graph and replayed
    gives the eager steps' iterates (to rounding), and the loss decreases."""
    from curadon_gb300.batch import BatchProjector

    geoms = jittered_batch(cuda_device, count=6, seed=7)
    proj = BatchProjector(geoms, cuda_device, matched=True)
    xt = torch.cat([ellipses_2d(int(gm.vol_shape[0]), k, device=cuda_device).reshape(-1)
                    for k, gm in enumerate(geoms)])
    with torch.no_grad():
        y = proj(xt).clone()
    # per-problem step 1 / ||A_i^T A_i|| from a few power iterations
    v = torch.rand_like(xt)
    for _ in range(6):
        with torch.no_grad():
            w = proj.adjoint(proj(v))
        v = torch.cat([(t / t.norm()).reshape(-1) for t in proj.split_volumes(w)])
    with torch.no_grad():
        av = proj(v)
    steps = torch.cat([torch.full((int(np.prod(s)),), 1.0 / float(a.norm() ** 2), device=cuda_device)
                       for s, a in zip(proj.vol_shapes, proj.split_sinograms(av))])

    def step(x):
        xr = x.detach().requires_grad_(True)
        r = proj(xr) - y
        (0.5 * (r * r).sum()).backward()
        return x - steps * xr.grad

    x = torch.zeros_like(xt)
    losses = []
    for _ in range(10):
        x = step(x)
        with torch.no_grad():
            losses.append(float(((proj(x) - y) ** 2).sum()))
    eager = x.clone()
    assert losses[-1] < 0.5 * losses[0], losses

    xs = torch.zeros_like(xt)
    step(xs)  # warm-up outside capture
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    cap = torch.cuda.Stream()
    cap.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(cap), torch.cuda.graph(graph, stream=cap):
        xr = xs.detach().requires_grad_(True)
        r = proj(xr) - y
        (gr,) = torch.autograd.grad(0.5 * (r * r).sum(), xr)
        xs.sub_(steps * gr)
    torch.cuda.current_stream().wait_stream(cap)
    xs.zero_()
    for _ in range(10):
        graph.replay()
    torch.cuda.synchronize()
    e = float((xs - eager).norm() / eager.norm())
    print(f"graph-replayed vs eager iterates: rel-L2 {e:.2e}; losses {losses[0]:.3e} -> "
          f"{losses[-1]:.3e}")
    assert e <= 1e-4


def test_batch_quarter_turn_backprojection(cuda_device, monkeypatch):
    """Problems whose plans take the quarter-turn backprojection (forced on
    here for small images) run it in the batch too: equal to the
    single-problem backprojection bit for bit, beside problems without the
    symmetry in the same launch."""
    monkeypatch.setenv("CURADON_GB300_ALGO", "bwd2d_sym=on")
    geoms, vols, sinos = [], [], []
    for k, (n, nangles) in enumerate([(128, 128), (256, 360), (130, 90), (192, 200), (96, 64)]):
        g = FanGeometry(**fan_config(n, nangles), device=cuda_device.index or 0)
        geoms.append(g)
        vols.append(ellipses_2d(n, 40 + k, device=cuda_device).contiguous())
        sinos.append(torch.zeros(g.sinogram_shape(), device=cuda_device))
    fw, bw = reference_results(geoms, vols, cuda_device)
    b = Batch2d(geoms, vols, sinos)
    b.forward()
    outs = [v.clone() for v in vols]
    Batch2d(geoms, outs, sinos).backward()
    torch.cuda.synchronize()
    for i, (o, r) in enumerate(zip(outs, bw)):
        assert torch.equal(o, r), i
