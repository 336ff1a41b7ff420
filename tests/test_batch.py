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
