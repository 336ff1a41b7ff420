"""Autotuning of the 2D operators (``curadon_gb300.autotune``, ``cg_plan2d_set_shapes``)
and of the batched forward (``Batch2d(..., forward="auto")``).

Tuning may only change which parity-tested variant runs: results stay within
the 1e-3 relative-L2 bar against the oracle."""
import numpy as np
import pytest
import torch

import oracle
from conftest import rel_l2
from curadon_gb300 import FanGeometry, FanVecGeometry, autotune, backward, forward
from curadon_gb300.batch import Batch2d
from curadon_gb300.phantom import ellipses_2d, fan_config

pytestmark = pytest.mark.gpu
TOL = 1e-3


def test_unknown_shapes_are_rejected(cuda_device):
    geom = FanGeometry(**fan_config(64, 30), device=cuda_device.index or 0)
    before = geom.plan.shapes
    with pytest.raises(ValueError):
        geom.plan.set_shapes(forward=999)
    with pytest.raises(ValueError):
        geom.plan.set_shapes(backward=1)
    assert geom.plan.shapes == before
    geom.plan.set_shapes(forward=443, backward=27)
    assert geom.plan.shapes == (443, 27)


def test_tune_applies_the_fastest_candidate(cuda_device):
    autotune.clear_cache()
    g = fan_config(384, 200)
    geom = FanGeometry(**g, device=cuda_device.index or 0)
    choice = autotune.tune(geom, reps=2, warmup=1)
    fwd = {f"forward {n}{'' if s is None else f' {s}'}" for n, s in autotune.FORWARD_CANDIDATES}
    bwd = {f"backward {n}{'' if s is None else f' {s}'}" for n, s in autotune.BACKWARD_CANDIDATES}
    assert set(choice["ms"]) == fwd | bwd
    assert all(t > 0 for t in choice["ms"].values())
    name_f, shape_f = choice["forward"]
    name_b, shape_b = choice["backward"]
    assert geom.plan.algorithm == (name_f, name_b)
    assert geom.plan.shapes == (shape_f, shape_b)
    best_f = min((t, k) for k, t in choice["ms"].items() if k.startswith("forward"))[1]
    assert best_f.split()[1] == name_f
    print(choice)
    ph = ellipses_2d(384, 3).numpy()
    v = torch.as_tensor(ph, device=cuda_device).contiguous()
    s = torch.zeros(geom.sinogram_shape(), device=cuda_device)
    forward(v, s, geom)
    e = rel_l2(s.cpu().numpy(), oracle.fwd2d(g, ph))
    sino = s.cpu().numpy()
    b = torch.zeros_like(v)
    backward(s, b, geom)
    eb = rel_l2(b.cpu().numpy(), oracle.bwd2d(g, sino))
    print(f"tuned fwd rel-L2 {e:.2e} bwd rel-L2 {eb:.2e}")
    assert e < TOL and eb < TOL


def test_tune_reuses_the_class_choice(cuda_device):
    autotune.clear_cache()
    g = fan_config(256, 120)
    g1 = FanGeometry(**g, device=cuda_device.index or 0)
    c1 = autotune.tune(g1, reps=1, warmup=1)
    g2 = FanGeometry(**g, device=cuda_device.index or 0)
    g2.plan.set_algorithm(forward="registers", backward="registers")
    c2 = autotune.tune(g2)
    assert c2 is c1
    assert g2.plan.algorithm == (c1["forward"][0], c1["backward"][0])
    other = FanGeometry(**fan_config(256, 121), device=cuda_device.index or 0)
    assert autotune.geometry_class(other.plan) != autotune.geometry_class(g1.plan)


def test_tune_vector_geometry_skips_refused_candidates(cuda_device):
    autotune.clear_cache()
    g = fan_config(192, 90)
    v = np.asarray(FanGeometry(**g).to_vec())
    geom = FanVecGeometry(g["vol_shape"], g["det_shape"], v, device=cuda_device.index or 0)
    choice = autotune.tune(geom, reps=1, warmup=1)
    assert "backward texture" not in choice["ms"]
    assert choice["backward"][0] == "shared"


def test_batch_auto_forward_keeps_the_faster_and_restores_sinograms(cuda_device):
    geoms, vols, sinos = [], [], []
    for k, n in enumerate([128, 256, 192]):
        g = fan_config(n, 100 + 20 * k)
        geoms.append(FanGeometry(**g, device=cuda_device.index or 0))
        vols.append(ellipses_2d(n, k, device=cuda_device).contiguous())
        sinos.append(torch.rand(geoms[-1].sinogram_shape(), device=cuda_device))
    before = [s.clone() for s in sinos]
    b = Batch2d(geoms, vols, sinos, forward="auto")
    assert set(b.tuned_ms) == set(Batch2d.FORWARD)
    best = min(b.tuned_ms, key=b.tuned_ms.get)
    assert b.forward_algorithm == best
    for s, c in zip(sinos, before):
        assert torch.equal(s, c)
    with pytest.raises(ValueError):
        Batch2d(geoms, vols, sinos, forward="fastest")
