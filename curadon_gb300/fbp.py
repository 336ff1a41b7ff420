"""Filtered backprojection, mirroring the reference's example
(examples/fbp.py:27-99): filter every sinogram row with a ramp-type response,
scale by pi / (2 nangles), backproject.

The filtering runs in the sm_103a kernel behind ``cg_filter_rows`` as a
direct circular convolution with h = Re(IDFT(fftshift(w))), which equals the
reference's ``_apply_filter`` (DFT of each row times fftshift(w), real part of
the inverse DFT) exactly in exact arithmetic.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Union

import numpy as np
import torch

from ._lib import check, load
from .backend import _check_tensor, _stream
from .geometry import ConeGeometry, FanGeometry
from .ops import backward

__all__ = ["frequency_response", "filter_kernel", "filter_sinogram", "fbp"]

_FILTERS = ("ram-lak", "shepp-logan", "cosine", "hamming", "hann", None)


def frequency_response(size: int, filter_name: Optional[str] = "ram-lak",
                       frequency_scaling: float = 1.0) -> np.ndarray:
    """The response of examples/fbp.py:27-48 in float64 (unshifted order:
    index i is frequency linspace(-1, 1, size)[i])."""
    W = np.linspace(-1, 1, size)
    w = np.abs(W)
    if filter_name == "ram-lak":
        pass
    elif filter_name == "shepp-logan":
        w = w * np.sinc(W / (2 * frequency_scaling))
    elif filter_name == "cosine":
        # the reference's branch names an undefined variable; the cosine
        # apodisation it intends is cos(pi W / (2 fs))
        w = w * np.cos(W * np.pi / (2 * frequency_scaling))
    elif filter_name == "hamming":
        w = w * (0.54 + 0.46 * np.cos(w * np.pi / frequency_scaling))
    elif filter_name == "hann":
        w = w * np.cos(w * np.pi / (2 * frequency_scaling)) ** 2
    elif filter_name is None:
        return np.ones(size)
    else:
        raise RuntimeError(f"Unknown Filter {filter_name}")
    return w * (W <= frequency_scaling)


def filter_kernel(size: int, filter_name: Optional[str] = "ram-lak",
                  frequency_scaling: float = 1.0) -> np.ndarray:
    """Spatial circular-convolution kernel h = Re(IDFT(fftshift(w)))."""
    w = frequency_response(size, filter_name, frequency_scaling)
    return np.real(np.fft.ifft(np.fft.fftshift(w)))


_kernel_cache: dict = {}


def _device_kernel(size, name, fs, device):
    key = (size, name, float(fs), str(device))
    h = _kernel_cache.get(key)
    if h is None:
        h = torch.as_tensor(filter_kernel(size, name, fs), dtype=torch.float32, device=device)
        _kernel_cache[key] = h
    return h


def filter_sinogram(sinogram: torch.Tensor, filter_name: Optional[str] = "ram-lak",
                    frequency_scaling: float = 1.0, scale: float = 1.0,
                    pre_weight: Optional[torch.Tensor] = None,
                    out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Filters the last axis of ``sinogram`` (2D: rows of cells; 3D: detector
    rows along u) and multiplies by ``scale``; ``pre_weight`` (one value per
    cell of the filtered axis) multiplies the input first."""
    _check_tensor(sinogram, "sinogram")
    N = sinogram.shape[-1]
    rows = sinogram.numel() // N
    if out is None:
        out = torch.empty_like(sinogram)
    _check_tensor(out, "out")
    if out.shape != sinogram.shape or out.data_ptr() == sinogram.data_ptr():
        raise ValueError("out must have the sinogram's shape and not alias it")
    h = _device_kernel(N, filter_name, frequency_scaling, sinogram.device)
    pre = C.c_void_p(0)
    if pre_weight is not None:
        _check_tensor(pre_weight, "pre_weight", 1)
        if pre_weight.numel() != N:
            raise ValueError("pre_weight needs one value per detector cell")
        pre = C.c_void_p(pre_weight.data_ptr())
    check(load().cg_filter_rows(C.c_void_p(sinogram.data_ptr()), C.c_void_p(out.data_ptr()),
                                C.c_void_p(h.data_ptr()), pre, rows, N, float(scale),
                                _stream(sinogram)))
    return out


def fbp(sinogram: torch.Tensor, geom: Union[FanGeometry, ConeGeometry],
        filter_name: Optional[str] = "ram-lak", frequency_scaling: float = 1.0,
        out: Optional[torch.Tensor] = None) -> torch.Tensor:
    """Filtered backprojection as in examples/fbp.py:87-94: filter, scale by
    pi / (2 nangles), backproject into ``out`` (zeros if not given)."""
    scale = np.pi / (2 * geom.nangles)
    fs = filter_sinogram(sinogram, filter_name, frequency_scaling, scale)
    if out is None:
        out = torch.zeros(tuple(int(v) for v in geom.vol_shape), device=sinogram.device,
                          dtype=torch.float32)
    return backward(fs, out, geom)
