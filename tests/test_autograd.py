"""GPU tests of the autograd functions (reference diffable.py semantics)."""
import numpy as np
import pytest
import torch

from curadon_gb300 import (ConeGeometry, FanGeometry, TorchBackprojection, TorchForward, backward,
                           forward)
from curadon_gb300.phantom import cone_config, ellipses_2d, fan_config

pytestmark = pytest.mark.gpu


def fan_geom():
    g = fan_config(64, 90)
    return FanGeometry(**g)


def test_forward_gradient_is_backprojection(cuda_device):
    geom = fan_geom()
    x = ellipses_2d(64, 0, device=cuda_device).requires_grad_(True)
    s = TorchForward.apply(x, geom)
    w = torch.rand_like(s)
    (s * w).sum().backward()
    expect = torch.zeros(64, 64, device=cuda_device)
    backward(w.contiguous(), expect, geom)
    assert torch.allclose(x.grad, expect, rtol=1e-6, atol=1e-4)
    ref = torch.zeros_like(s)
    forward(x.detach(), ref, geom)
    assert torch.equal(s.detach(), ref)


def test_backprojection_gradient_is_forward(cuda_device):
    geom = fan_geom()
    s = torch.rand(geom.sinogram_shape(), device=cuda_device, requires_grad=True)
    v = TorchBackprojection.apply(s, geom)
    w = torch.rand_like(v)
    (v * w).sum().backward()
    expect = torch.zeros(geom.sinogram_shape(), device=cuda_device)
    forward(w.contiguous(), expect, geom)
    assert torch.allclose(s.grad, expect, rtol=1e-6, atol=1e-4)


def test_cone_autograd(cuda_device):
    g = cone_config(24, 12, 40)
    geom = ConeGeometry(**g)
    x = torch.rand(24, 24, 24, device=cuda_device, requires_grad=True)
    s = TorchForward.apply(x, geom)
    s.sum().backward()
    expect = torch.zeros(24, 24, 24, device=cuda_device)
    backward(torch.ones_like(s), expect, geom)
    assert torch.allclose(x.grad, expect)


def test_gradient_descent_reduces_residual(cuda_device):
    geom = fan_geom()
    x_true = ellipses_2d(64, 3, device=cuda_device)
    y = torch.zeros(geom.sinogram_shape(), device=cuda_device)
    forward(x_true, y, geom)
    x = torch.zeros_like(x_true, requires_grad=True)
    losses = []
    for _ in range(10):
        r = TorchForward.apply(x, geom) - y
        loss = (r * r).sum()
        losses.append(float(loss))
        (g,) = torch.autograd.grad(loss, x)
        with torch.no_grad():
            # exact line search of ||A x - y||^2 along -g
            ag = torch.zeros_like(y)
            forward(g.contiguous(), ag, geom)
            alpha = (r.detach() * ag).sum() / (ag * ag).sum()
            x -= alpha * g
    assert losses[-1] < 0.2 * losses[0]
    assert np.all(np.diff(losses) < 0)
