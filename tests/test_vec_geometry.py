"""GPU parity of the full vector geometry (``FanVecGeometry``,
``cg_plan2d_create_vec``).

Tolerance: relative L2 <= 1e-3 against the FP64 vector oracle (which
intersects every pixel's ray with the detector line directly, independent of
the projective tables the kernels use) and against the circular plan for
vectors made from a circular geometry; max abs error printed."""
import numpy as np
import pytest
import torch

import oracle
from conftest import max_abs, rel_l2
from curadon_gb300 import FanGeometry, FanVecGeometry, backward, forward
from curadon_gb300.backend import FORWARD_2D
from curadon_gb300.phantom import ellipses_2d, fan_config

pytestmark = pytest.mark.gpu
TOL = 1e-3


def circular_vecs(g):
    vecs = np.asarray(FanGeometry(**g).to_vec())
    vecs[:, 4:] *= g["det_spacing"]  # u as the step between cell centres
    return vecs


def jittered_vecs(g, sigma, seed):
    """Per-view Gaussian jitter of source and detector positions."""
    rng = np.random.default_rng(seed)
    v = circular_vecs(g)
    v[:, 0:4] += rng.normal(0.0, sigma, (v.shape[0], 4))
    return v


def run(geom, vol, sino_in, dev):
    v = torch.as_tensor(vol, device=dev).contiguous()
    s = torch.zeros(geom.sinogram_shape(), device=dev)
    forward(v, s, geom)
    b = torch.zeros(tuple(int(x) for x in geom.vol_shape), device=dev)
    backward(torch.as_tensor(sino_in, device=dev).contiguous(), b, geom)
    torch.cuda.synchronize()
    return s.cpu().numpy(), b.cpu().numpy()


def test_circular_vectors_match_circular_plan(cuda_device):
    g = fan_config(256, 180)
    ph = ellipses_2d(256, 4).numpy()
    rng = np.random.default_rng(1)
    sino = rng.uniform(0, 1, (180, g["det_shape"])).astype(np.float32)
    vg = FanVecGeometry(g["vol_shape"], g["det_shape"], circular_vecs(g),
                        device=cuda_device.index or 0)
    cg = FanGeometry(**g, device=cuda_device.index or 0)
    vg.plan.set_algorithm(forward="registers")
    cg.plan.set_algorithm(forward="registers")
    s1, b1 = run(vg, ph, sino, cuda_device)
    s2, b2 = run(cg, ph, sino, cuda_device)
    # the circular plan keeps the reference's FP32 tables, whose per-cell step
    # carries the rounding of a difference of two numbers of size DSD; the
    # vector plan's tables are exact to FP32, so far cells differ slightly
    print(f"fwd rel-L2 {rel_l2(s1, s2):.2e} bwd rel-L2 {rel_l2(b1, b2):.2e}")
    assert rel_l2(s1, s2) < TOL and rel_l2(b1, b2) < TOL


@pytest.mark.parametrize("algo", FORWARD_2D)
def test_jittered_forward_against_oracle(cuda_device, algo):
    g = fan_config(192, 240)
    vecs = jittered_vecs(g, 0.5, 11)
    vg = FanVecGeometry(g["vol_shape"], g["det_shape"], vecs, device=cuda_device.index or 0)
    vg.plan.set_algorithm(forward=algo)
    ph = ellipses_2d(192, 6).numpy()
    v = torch.as_tensor(ph, device=cuda_device).contiguous()
    s = torch.zeros(vg.sinogram_shape(), device=cuda_device)
    forward(v, s, vg)
    torch.cuda.synchronize()
    so = oracle.fwd2d_vec(g, vecs, ph)
    e = rel_l2(s.cpu().numpy(), so)
    print(f"{algo}: fwd rel-L2 {e:.2e} max-abs {max_abs(s.cpu().numpy(), so):.2e}")
    assert e < TOL


@pytest.mark.parametrize("n,nangles", [(192, 240), (130, 77)])
def test_jittered_backward_against_oracle(cuda_device, n, nangles):
    g = fan_config(n, nangles)
    vecs = jittered_vecs(g, 0.5, n)
    vg = FanVecGeometry(g["vol_shape"], g["det_shape"], vecs, device=cuda_device.index or 0)
    rng = np.random.default_rng(3)
    sino = rng.uniform(0, 1, vg.sinogram_shape()).astype(np.float32)
    b = torch.zeros((n, n), device=cuda_device)
    backward(torch.as_tensor(sino, device=cuda_device), b, vg)
    torch.cuda.synchronize()
    bo = oracle.bwd2d_vec(g, vecs, sino)
    e = rel_l2(b.cpu().numpy(), bo)
    print(f"n={n}: bwd rel-L2 {e:.2e} max-abs {max_abs(b.cpu().numpy(), bo):.2e}")
    assert e < TOL
    with pytest.raises(Exception):
        vg.plan.set_algorithm(backward="texture")


def test_jittered_matched_adjoint(cuda_device):
    """<A x, y> = <x, A^T y> for a vector geometry (matched adjoint)."""
    from curadon_gb300 import adjoint

    g = fan_config(160, 120)
    vg = FanVecGeometry(g["vol_shape"], g["det_shape"], jittered_vecs(g, 0.5, 5),
                        device=cuda_device.index or 0)
    rng = np.random.default_rng(9)
    x = torch.as_tensor(rng.uniform(0, 1, (160, 160)).astype(np.float32), device=cuda_device)
    y = torch.as_tensor(rng.uniform(0, 1, vg.sinogram_shape()).astype(np.float32),
                        device=cuda_device)
    ax = torch.zeros_like(y)
    forward(x, ax, vg, exact=True)
    aty = torch.zeros_like(x)
    adjoint(y, aty, vg)
    torch.cuda.synchronize()
    lhs = float((ax.double() * y.double()).sum())
    rhs = float((x.double() * aty.double()).sum())
    print(f"dot test {abs(lhs - rhs) / abs(lhs):.2e}")
    assert abs(lhs - rhs) / abs(lhs) < 1e-5
