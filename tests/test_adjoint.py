"""GPU tests of the matched adjoint: dot-product test <Ax, y> = <x, A^T y>
(relative 1e-5) and finite differences of the matched-gradient autograd."""
import numpy as np
import pytest
import torch

from curadon_gb300 import ConeGeometry, FanGeometry, TorchForward, adjoint, forward
from curadon_gb300.phantom import cone_config, ellipses_2d, ellipsoids_3d, fan_config

pytestmark = pytest.mark.gpu


def dot_test(geom, x, y, dev):
    x = torch.as_tensor(x, device=dev).contiguous()
    y = torch.as_tensor(y, device=dev).contiguous()
    ax = torch.zeros(geom.sinogram_shape(), device=dev)
    forward(x, ax, geom, exact=True)
    if isinstance(geom, ConeGeometry):
        # rays that miss are left unwritten: they are zero rows of A
        ax0 = torch.full_like(ax, 123.0)
        forward(x, ax0, geom, exact=True)
        ax = torch.where(ax0 == 123.0, torch.zeros_like(ax), ax)
    aty = torch.zeros_like(x)
    adjoint(y, aty, geom)
    torch.cuda.synchronize()
    lhs = float((ax.double() * y.double()).sum())
    rhs = float((x.double() * aty.double()).sum())
    return abs(lhs - rhs) / max(abs(lhs), abs(rhs))


@pytest.mark.parametrize("n,nangles", [(64, 90), (128, 200), (257, 301)])
def test_dot_product_2d(cuda_device, n, nangles):
    g = fan_config(n, nangles)
    geom = FanGeometry(**g)
    rng = np.random.default_rng(n)
    x = rng.uniform(0, 1, (n, n)).astype(np.float32)
    y = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    assert dot_test(geom, x, y, cuda_device) < 1e-5


def test_dot_product_2d_pair_accumulators(cuda_device):
    """Above ~1700^2 pixels the adjoint's accumulators no longer fit the L2
    as quads and it scatters into pairs instead: the same transpose."""
    n = 1800
    g = fan_config(n, 48)
    geom = FanGeometry(**g)
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 1, (n, n)).astype(np.float32)
    y = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    assert dot_test(geom, x, y, cuda_device) < 1e-5


def test_dot_product_2d_offsets(cuda_device):
    g = fan_config(48, 37, 70, 1.3, 90.0, 150.0)
    g.update(vol_shape=(48, 60), vol_spacing=(0.9, 1.2), vol_offset=(2.0, -3.0), det_offset=1.5)
    geom = FanGeometry(**g)
    rng = np.random.default_rng(1)
    x = rng.uniform(0, 1, (48, 60)).astype(np.float32)
    y = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    assert dot_test(geom, x, y, cuda_device) < 1e-5


@pytest.mark.parametrize("shape,nangles,det", [((24, 24, 24), 20, 40), ((20, 28, 36), 33, 50)])
def test_dot_product_3d(cuda_device, shape, nangles, det):
    g = cone_config(shape[0], nangles, det)
    g["vol_shape"] = shape
    geom = ConeGeometry(**g)
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 1, shape).astype(np.float32)
    y = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    assert dot_test(geom, x, y, cuda_device) < 1e-5


def test_matched_gradient_finite_differences(cuda_device):
    g = fan_config(64, 60)
    geom = FanGeometry(**g)
    x0 = ellipses_2d(64, 2, device=cuda_device).double()
    target = torch.zeros(geom.sinogram_shape(), device=cuda_device)
    forward(ellipses_2d(64, 9, device=cuda_device), target, geom, exact=True)

    def loss(x):
        s = TorchForward.apply(x.float(), geom, True)
        return ((s.double() - target.double()) ** 2).sum()

    x = x0.clone().float().requires_grad_(True)
    L = ((TorchForward.apply(x, geom, True) - target) ** 2).sum()
    (grad,) = torch.autograd.grad(L, x)
    rng = np.random.default_rng(0)
    d = torch.as_tensor(rng.normal(size=(64, 64)), device=cuda_device)
    eps = 1e-2
    fd = (float(loss(x0 + eps * d)) - float(loss(x0 - eps * d))) / (2 * eps)
    an = float((grad.double() * d).sum())
    assert abs(fd - an) / abs(fd) < 1e-3


@pytest.mark.parametrize("algo", ["registers", "chunked"])
def test_dot_product_2d_per_forward_algorithm(cuda_device, algo):
    """The FP32-weight forwards (registers, chunked) share the adjoint."""
    g = fan_config(200, 150)
    geom = FanGeometry(**g)
    geom.exact_plan.set_algorithm(forward=algo)
    rng = np.random.default_rng(5)
    x = rng.uniform(0, 1, (200, 200)).astype(np.float32)
    y = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    assert dot_test(geom, x, y, cuda_device) < 1e-5


@pytest.mark.parametrize("algo", ["registers", "quad"])
def test_dot_product_3d_per_forward_algorithm(cuda_device, algo):
    """The FP32-weight 3D forwards (registers, quad) share the adjoint."""
    g = cone_config(40, 36, 64)
    geom = ConeGeometry(**g)
    geom.exact_plan.set_algorithm(forward=algo)
    rng = np.random.default_rng(6)
    x = rng.uniform(0, 1, (40, 40, 40)).astype(np.float32)
    y = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    assert dot_test(geom, x, y, cuda_device) < 1e-5


@pytest.mark.parametrize("algo", ["registers", "quad"])
def test_dot_product_3d_exact_parameters(cuda_device, monkeypatch, algo):
    """With drift-free sample parameters (t3d=exact, the default from 512
    voxels along an axis) the forward and the matched adjoint still take the
    same samples."""
    g = cone_config(40, 36, 64)
    monkeypatch.setenv("CURADON_GB300_ALGO", "t3d=exact")
    geom = ConeGeometry(**g)
    geom.exact_plan.set_algorithm(forward=algo)
    monkeypatch.delenv("CURADON_GB300_ALGO")
    rng = np.random.default_rng(8)
    x = rng.uniform(0, 1, (40, 40, 40)).astype(np.float32)
    y = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    assert dot_test(geom, x, y, cuda_device) < 1e-5


def test_adjoint_accumulates(cuda_device):
    g = cone_config(24, 12, 40)
    geom = ConeGeometry(**g)
    y = torch.rand(geom.sinogram_shape(), device=cuda_device)
    a = torch.zeros(24, 24, 24, device=cuda_device)
    adjoint(y, a, geom)
    b = torch.ones_like(a)
    adjoint(y, b, geom)
    torch.cuda.synchronize()
    assert torch.allclose(b, a + 1.0, rtol=1e-6, atol=1e-5)


@pytest.mark.parametrize("variant", ["adj3d_merge=1", "adj3d_order=band",
                                     "adj3d_order=band,adj3d_merge=1",
                                     "adj3d=pair,adj3d_order=band", "adj3d=pair",
                                     "adj3d_agg=1", "adj3d_agg=1,adj3d_order=band"])
def test_dot_product_3d_scatter_variants(cuda_device, monkeypatch, variant):
    """Every shape of the 3D scatter (accumulators, block order, merged slice
    atomics, warp-aggregated atomics; CURADON_GB300_ALGO) is the transpose of
    the quad forward."""
    g = cone_config(40, 36, 64)
    monkeypatch.setenv("CURADON_GB300_ALGO", variant)
    geom = ConeGeometry(**g)
    geom.exact_plan
    monkeypatch.delenv("CURADON_GB300_ALGO")
    rng = np.random.default_rng(8)
    x = rng.uniform(0, 1, (40, 40, 40)).astype(np.float32)
    y = rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32)
    e = dot_test(geom, x, y, cuda_device)
    print(f"{variant}: dot-test relative error {e:.2e}")
    assert e < 1e-5
