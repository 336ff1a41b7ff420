"""Parity at the benchmark workload itself, against the FP64 oracle.

The 2D fan-beam n=2048 problem timed by ``bench.py`` (2048 x 2048 image,
2048 views over [0, 2 pi), 2897 cells of 1.5, DSO 4096, DSD 6144): the
default backprojection over the whole image and all 2048 views, and the
default forward on a subset of views, each against the oracle's FP64
restatement of the reference (forward_2d.hpp:21-79, backward_2d.hpp:21-100).
The reference's own backprojection cannot serve as the check here: above
1024 views it launches its chunks on unordered streams that share one
texture and read-modify-write the volume (backward_2d.hpp:103-153).

Tolerance: relative L2 <= 1e-3 (the drop-in bar); max abs error printed.
The oracle runs on all host cores (a few seconds on 16)."""
import numpy as np
import pytest
import torch

import oracle
from conftest import max_abs, rel_l2
from curadon_gb300 import FanGeometry, backward, forward
from curadon_gb300.phantom import ellipses_2d, fan_config, seed_for

pytestmark = pytest.mark.gpu
TOL = 1e-3


@pytest.fixture(scope="module")
def headline(cuda_device):
    g = fan_config(2048)
    assert len(g["angles"]) == 2048 and g["det_shape"] == 2897
    geom = FanGeometry(**g)
    vol = ellipses_2d(2048, seed_for(1, 0), device=cuda_device).contiguous()
    sino = torch.zeros(geom.sinogram_shape(), device=cuda_device)
    forward(vol, sino, geom)
    torch.cuda.synchronize()
    return g, geom, vol, sino


def test_headline_backprojection_against_oracle(cuda_device, headline):
    g, geom, _, sino = headline
    assert geom.plan.algorithm[1] == "shared"  # the default, staged backprojector
    b = torch.zeros((2048, 2048), device=cuda_device)
    backward(sino, b, geom)
    torch.cuda.synchronize()
    s_host = sino.cpu().numpy()
    bo = oracle.bwd2d(g, s_host)
    bg = b.cpu().numpy()
    e = rel_l2(bg, bo)
    print(f"n=2048 x 2048 views backprojection: rel-L2 {e:.2e} max-abs {max_abs(bg, bo):.2e} "
          f"(max |oracle| {np.abs(bo).max():.3e})")
    assert e <= TOL


def test_headline_forward_against_oracle(cuda_device, headline):
    g, geom, vol, sino = headline
    assert geom.plan.algorithm[0] == "chunked"  # the default from 704^2 pixels
    views = np.arange(0, 2048, 8)  # 256 views spread over the whole orbit
    h = dict(g)
    h["angles"] = np.asarray(g["angles"])[views]
    h["DSO"] = np.asarray(g["DSO"])[views]
    h["DSD"] = np.asarray(g["DSD"])[views]
    so = oracle.fwd2d(h, vol.cpu().numpy())
    sg = sino.cpu().numpy()[views]
    e = rel_l2(sg, so)
    print(f"n=2048 forward ({len(views)} of 2048 views): rel-L2 {e:.2e} "
          f"max-abs {max_abs(sg, so):.2e} (max |oracle| {np.abs(so).max():.3e})")
    assert e <= TOL
