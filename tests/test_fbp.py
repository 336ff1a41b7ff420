"""FBP row filter: the direct circular convolution equals the reference's
FFT formulation (examples/fbp.py:51-56), and FBP reconstructs a phantom."""
import numpy as np
import pytest

from curadon_gb300.fbp import filter_kernel, frequency_response


def fft_filter(rows, name, fs=1.0):
    """examples/fbp.py:_apply_filter in float64 numpy: the per-row DFT times
    fftshift(w), real part of the inverse DFT (its shifts along the angle
    axis cancel)."""
    w = frequency_response(rows.shape[-1], name, fs)
    return np.real(np.fft.ifft(np.fft.fft(rows, axis=-1) * np.fft.fftshift(w), axis=-1))


@pytest.mark.parametrize("N", [16, 91, 363, 1000])
@pytest.mark.parametrize("name", ["ram-lak", "shepp-logan", "hamming", "hann", "cosine"])
def test_convolution_equals_fft_filter(N, name):
    rng = np.random.default_rng(N)
    rows = rng.uniform(0, 1, (3, N))
    h = filter_kernel(N, name)
    idx = (np.arange(N)[:, None] - np.arange(N)[None, :]) % N
    direct = rows @ h[idx].T
    assert np.allclose(direct, fft_filter(rows, name), atol=1e-12)


def test_unknown_filter():
    with pytest.raises(RuntimeError):
        frequency_response(8, "box")


@pytest.mark.gpu
@pytest.mark.parametrize("shape", [(360, 91), (7, 2897), (50, 1)])
def test_gpu_filter_matches_fft(cuda_device, shape):
    import torch

    from curadon_gb300.fbp import filter_sinogram

    rng = np.random.default_rng(0)
    s = rng.uniform(0, 1, shape).astype(np.float32)
    out = filter_sinogram(torch.as_tensor(s, device=cuda_device), "ram-lak", scale=0.5)
    expect = 0.5 * fft_filter(s.astype(np.float64), "ram-lak")
    got = out.cpu().numpy()
    err = np.linalg.norm(got - expect) / np.linalg.norm(expect)
    assert err < 1e-5, err


@pytest.mark.gpu
def test_fbp_reconstructs_phantom(cuda_device):
    import torch

    from curadon_gb300 import FanGeometry, forward
    from curadon_gb300.fbp import fbp
    from curadon_gb300.phantom import ellipses_2d, fan_config

    n = 128
    g = fan_config(n, 360, 182, 1.0, 20.0 * n, 22.0 * n)  # near-parallel, as fbp.py's config
    geom = FanGeometry(**g)
    x = ellipses_2d(n, 4, device=cuda_device)
    s = torch.zeros(geom.sinogram_shape(), device=cuda_device)
    forward(x, s, geom)
    rec = fbp(s, geom)
    torch.cuda.synchronize()
    a = (rec - rec.mean()).flatten()
    b = (x - x.mean()).flatten()
    corr = float((a @ b) / (a.norm() * b.norm()))
    assert corr > 0.9, corr


@pytest.mark.gpu
def test_packed_filter_equals_scalar_filter(cuda_device, tmp_path):
    """The filter runs on pairs of rows with packed FMAs; its accumulation
    order per output is that of the one-row kernel (selected in a child
    process by CURADON_GB300_FILTER=scalar), so the results are equal bit
    for bit, odd row counts included."""
    import os
    import subprocess
    import sys

    import torch

    from curadon_gb300.fbp import filter_sinogram

    rng = np.random.default_rng(5)
    s = rng.uniform(0, 1, (37, 1449)).astype(np.float32)
    np.save(tmp_path / "s.npy", s)
    out = filter_sinogram(torch.as_tensor(s, device=cuda_device), "shepp-logan").cpu().numpy()
    code = ("import numpy as np, torch, sys\n"
            "from curadon_gb300.fbp import filter_sinogram\n"
            f"s = np.load(r'{tmp_path / 's.npy'}')\n"
            "o = filter_sinogram(torch.as_tensor(s, device='cuda'), 'shepp-logan').cpu().numpy()\n"
            f"np.save(r'{tmp_path / 'o.npy'}', o)\n")
    env = dict(os.environ, CURADON_GB300_FILTER="scalar")
    subprocess.run([sys.executable, "-c", code], check=True, env=env, timeout=300)
    assert np.array_equal(out, np.load(tmp_path / "o.npy"))
