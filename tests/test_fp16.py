"""FP16 storage of the 2D operators (float16 volumes and/or sinograms).

The reference instantiates forward_2d / backward_2d for every pair of
float32 / float16 volume and sinogram (forward.cu:107-135, backward.cu:104-135)
and computes in FP32.  Tolerance: relative L2 <= 1e-3 against the
reference's own operators on the same half inputs, and against this
library's FP32 operators applied to the same (half-representable) values;
a half output carries one rounding to 11 significant bits (relative error
at most 4.9e-4 per element).  Max abs error is printed."""
import numpy as np
import pytest
import torch

from conftest import max_abs, rel_l2
from curadon_gb300 import FanGeometry, backward, forward
from curadon_gb300.phantom import ellipses_2d, fan_config

pytestmark = pytest.mark.gpu
TOL = 1e-3
DT = {16: torch.float16, 32: torch.float32}


def geometry(n, nangles, vol_prec, sino_prec, dev):
    g = fan_config(n, nangles)
    return g, FanGeometry(**g, vol_prec=vol_prec, sino_prec=sino_prec, device=dev.index or 0)


@pytest.mark.parametrize("vb,sb", [(16, 16), (16, 32), (32, 16)])
def test_forward_matches_reference(cuda_device, ref_ops, vb, sb):
    g, geom = geometry(256, 180, vb, sb, cuda_device)
    v = ellipses_2d(256, 3, device=cuda_device).to(DT[vb]).contiguous()
    s = torch.zeros(geom.sinogram_shape(), device=cuda_device, dtype=DT[sb])
    forward(v, s, geom)
    h, _ = ref_ops.plan2d(g, vol_prec=vb, det_prec=sb)
    try:
        s_ref = torch.zeros_like(s)
        ref_ops.forward2d_typed(h, v, s_ref)
        ref_ops.sync()
    finally:
        ref_ops.destroy2d(h)
    torch.cuda.synchronize()
    a, b = s.float().cpu(), s_ref.float().cpu()
    e = rel_l2(a, b)
    print(f"vol f{vb} sino f{sb}: fwd rel-L2 {e:.2e} max-abs {max_abs(a, b):.2e}")
    assert e < TOL


@pytest.mark.parametrize("vb,sb", [(16, 16), (16, 32), (32, 16)])
def test_backward_matches_reference(cuda_device, ref_ops, vb, sb):
    g, geom = geometry(256, 180, vb, sb, cuda_device)
    rng = np.random.default_rng(7)
    sino = torch.as_tensor(rng.uniform(0, 2, geom.sinogram_shape()).astype(np.float32),
                           device=cuda_device).to(DT[sb])
    v0 = torch.as_tensor(rng.uniform(0, 50, (256, 256)).astype(np.float32),
                         device=cuda_device).to(DT[vb])
    v = v0.clone()
    backward(sino, v, geom)
    h, _ = ref_ops.plan2d(g, vol_prec=vb, det_prec=sb)
    try:
        v_ref = v0.clone()
        ref_ops.backward2d_typed(h, v_ref, sino)
        ref_ops.sync()
    finally:
        ref_ops.destroy2d(h)
    torch.cuda.synchronize()
    a, b = (v - v0).float().cpu(), (v_ref - v0).float().cpu()
    e = rel_l2(a, b)
    print(f"vol f{vb} sino f{sb}: bwd rel-L2 {e:.2e} max-abs {max_abs(a, b):.2e}")
    assert e < TOL


def test_half_storage_matches_fp32(cuda_device):
    """Half in, half out = the FP32 operators on the same values, rounded."""
    g, g16 = geometry(200, 150, 16, 16, cuda_device)
    g32 = FanGeometry(**g, device=cuda_device.index or 0)
    v16 = ellipses_2d(200, 5, device=cuda_device).half().contiguous()
    s16 = torch.zeros(g16.sinogram_shape(), device=cuda_device, dtype=torch.float16)
    s32 = torch.zeros(g32.sinogram_shape(), device=cuda_device)
    forward(v16, s16, g16)
    forward(v16.float(), s32, g32)
    assert torch.equal(s16, s32.half())  # same FP32 sums, one rounding
    b16 = torch.zeros((200, 200), device=cuda_device, dtype=torch.float16)
    b32 = torch.zeros((200, 200), device=cuda_device)
    backward(s16, b16, g16)
    backward(s16.float(), b32, g32)
    torch.cuda.synchronize()
    assert torch.equal(b16, b32.half())


def test_precision_mismatch_raises(cuda_device):
    _, geom = geometry(64, 30, 32, 32, cuda_device)
    v = torch.zeros((64, 64), device=cuda_device, dtype=torch.float16)
    s = torch.zeros(geom.sinogram_shape(), device=cuda_device)
    with pytest.raises(AttributeError, match="precision"):
        forward(v, s, geom)
    with pytest.raises(TypeError):
        forward(v.double(), s, geom)
