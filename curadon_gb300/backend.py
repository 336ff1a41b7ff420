"""Python face of the C ABI, mirroring curadon's native module ``curadon_ext``.

Same names, argument order and meaning as the reference's bindings
(python/standalone/src/bind.cpp:58-66, plan.cu:34-58, forward.cu:138-143,
backward.cu:135-140).  Tensors are torch CUDA tensors, C-contiguous; 2D
volumes and sinograms are float32 or float16 (the volume's as the plan's
vol_prec), 3D ones float32.  Work is enqueued on torch's current stream of
the tensors' device.

Error behaviour follows the reference's: mismatched devices raise
``AttributeError`` (forward.cu:95-105), a volume whose dtype differs from the
plan's precision raises ``AttributeError`` (forward.cu:107-122), a dtype other
than float32/float16 raises ``TypeError`` (forward.cu:133-135), and
precisions other than 16/32 raise ``AttributeError`` (plan.cu:20-28).  Unlike
the reference, shapes are checked against the plan (the reference writes out
of bounds instead).
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np
import torch

from ._lib import check, load

__all__ = ["plan_2d", "plan_2d_vec", "plan_3d", "forward_2d", "backward_2d", "adjoint_2d",
           "forward_3d", "backward_3d", "wait_timeouts", "raise_on_wait_timeouts",
           "WaitTimeoutError"]


def _u64(a):
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.uint64).ravel())
    return arr, arr.ctypes.data_as(C.POINTER(C.c_uint64))


def _f32(a):
    arr = np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel())
    return arr, arr.ctypes.data_as(C.POINTER(C.c_float))


def _stream(t: torch.Tensor) -> C.c_void_p:
    return C.c_void_p(torch.cuda.current_stream(t.device).cuda_stream)


# algorithm names and the C ABI's codes (cg_plan2d/3d_set_algorithm)
FORWARD_2D = {"registers": 0, "texture": 1, "chunked": 4}
BACKWARD_2D = {"registers": 0, "texture": 1, "shared": 2}
FORWARD_3D = {"registers": 0, "texture": 1, "quad": 4, "mixed": 5}
BACKWARD_3D = {"registers": 0, "axial": 1}


def _algo_index(name, names, what):
    if name is None:
        return -1
    if name not in names:
        raise ValueError(f"{what} algorithm must be one of {tuple(names)}, got {name!r}")
    return names[name]


def _algo_name(code, names):
    return next(k for k, v in names.items() if v == code)


def _check_tensor(t, name: str, ndim: int | None = None, half: bool = False):
    if not isinstance(t, torch.Tensor):
        raise TypeError(f"{name} must be a torch.Tensor")
    if not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise TypeError(f"{name} must be C-contiguous")
    if ndim is not None and t.dim() != ndim:
        raise TypeError(f"{name} must have {ndim} dimensions, got {t.dim()}")
    if t.dtype == torch.float16 and not half:
        raise NotImplementedError(f"{name}: float16 is only built for the 2D operators")
    if t.dtype not in (torch.float32, torch.float16):
        raise TypeError("Only float32 is supported")


def _bits(t: torch.Tensor) -> int:
    return 16 if t.dtype == torch.float16 else 32


class plan_2d:
    """Fan-beam plan: ``plan_2d(device, vol_prec, vol_shape, vol_spacing,
    vol_offset, det_prec, det_count, det_spacing, det_offset, DSO, DSD,
    angles, det_pitch, COR)`` as in plan.cu:34-56 (shapes in Python order)."""

    def __init__(self, device, vol_prec, vol_shape, vol_spacing, vol_offset, det_prec, det_count,
                 det_spacing, det_offset, DSO, DSD, angles, det_pitch=0.0, COR=0.0):
        L = load()
        if int(vol_prec) not in (16, 32) or int(det_prec) not in (16, 32):
            raise AttributeError("Precision must either be f32 or f16")
        angles_a, angles_p = _f32(angles)
        n = angles_a.size
        dso_a, dso_p = _f32(np.broadcast_to(np.asarray(DSO, np.float32), (n,)))
        dsd_a, dsd_p = _f32(np.broadcast_to(np.asarray(DSD, np.float32), (n,)))
        shape_a, shape_p = _u64(vol_shape)
        sp_a, sp_p = _f32(vol_spacing)
        off_a, off_p = _f32(vol_offset)
        if shape_a.size != 2 or sp_a.size != 2 or off_a.size != 2:
            raise TypeError("vol_shape, vol_spacing and vol_offset must have 2 entries")
        h = C.c_void_p()
        check(L.cg_plan2d_create(C.byref(h), int(device), int(vol_prec), shape_p, sp_p, off_p,
                                 int(det_prec), int(det_count), float(det_spacing),
                                 float(det_offset), dso_p, dsd_p, angles_p, n, float(det_pitch),
                                 float(COR)))
        self._h = h
        self._L = L
        self.device_id = int(device)
        self.vol_prec = int(vol_prec)
        self.det_prec = int(det_prec)
        self.vol_shape = (int(shape_a[0]), int(shape_a[1]))
        self.det_count = int(det_count)
        self.nangles = n

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.cg_plan2d_destroy(h)
            self._h = None

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def _block(self):
        bx, by = C.c_uint64(), C.c_uint64()
        check(self._L.cg_plan2d_get_forward_block(self._h, C.byref(bx), C.byref(by)))
        return bx.value, by.value

    @property
    def forward_block_x(self) -> int:
        return self._block()[0]

    @forward_block_x.setter
    def forward_block_x(self, v):
        check(self._L.cg_plan2d_set_forward_block(self._h, int(v), self._block()[1]))

    @property
    def forward_block_y(self) -> int:
        return self._block()[1]

    @forward_block_y.setter
    def forward_block_y(self, v):
        check(self._L.cg_plan2d_set_forward_block(self._h, self._block()[0], int(v)))

    @property
    def algorithm(self):
        """(forward, backward) algorithm names of this plan."""
        f, b = C.c_int(), C.c_int()
        check(self._L.cg_plan2d_get_algorithm(self._h, C.byref(f), C.byref(b)))
        return _algo_name(f.value, FORWARD_2D), _algo_name(b.value, BACKWARD_2D)

    @property
    def quarter_turn(self) -> int:
        """+1 / -1 where the staged backprojection runs over the views'
        quarter-turn symmetry (one projective evaluation for four (pixel,
        view) pairs), else 0."""
        q = C.c_int()
        check(self._L.cg_plan2d_get_symmetry(self._h, C.byref(q)))
        return q.value

    def set_algorithm(self, forward=None, backward=None):
        """Selects the algorithms (names from FORWARD_2D / BACKWARD_2D)."""
        check(self._L.cg_plan2d_set_algorithm(
            self._h, _algo_index(forward, FORWARD_2D, "forward"),
            _algo_index(backward, BACKWARD_2D, "backward")))

    @property
    def shapes(self):
        """(chunked-forward shape, staged-backprojector variant) of this plan."""
        f, b = C.c_int(), C.c_int()
        check(self._L.cg_plan2d_get_shapes(self._h, C.byref(f), C.byref(b)))
        return f.value, b.value

    def set_shapes(self, forward=None, backward=None):
        """Selects the chunked forward's kernel shape and the staged
        backprojector's variant (``cg_plan2d_set_shapes``; None keeps)."""
        check(self._L.cg_plan2d_set_shapes(self._h, -1 if forward is None else int(forward),
                                           -1 if backward is None else int(backward)))

    def tables(self):
        """(sources, u_origins, delta_us), each (nangles, 2) float32."""
        out = [np.zeros(2 * self.nangles, np.float32) for _ in range(3)]
        check(self._L.cg_plan2d_tables(self._h, *(o.ctypes.data_as(C.POINTER(C.c_float))
                                                   for o in out)))
        return [o.reshape(self.nangles, 2) for o in out]


class plan_2d_vec(plan_2d):
    """Fan-beam plan from per-view vectors (``cg_plan2d_create_vec``):
    ``vecs`` is (nangles, 6) = [source.x, source.y, detector.x, detector.y,
    u.x, u.y] as FanGeometry.to_vec returns them (geometry.py:54-80)."""

    def __init__(self, device, vol_prec, vol_shape, vol_spacing, vol_offset, det_prec, det_count,
                 vecs):
        L = load()
        if int(vol_prec) not in (16, 32) or int(det_prec) not in (16, 32):
            raise AttributeError("Precision must either be f32 or f16")
        v = np.ascontiguousarray(np.asarray(vecs, np.float32).reshape(-1, 6))
        n = v.shape[0]
        shape_a, shape_p = _u64(vol_shape)
        sp_a, sp_p = _f32(vol_spacing)
        off_a, off_p = _f32(vol_offset)
        if shape_a.size != 2 or sp_a.size != 2 or off_a.size != 2:
            raise TypeError("vol_shape, vol_spacing and vol_offset must have 2 entries")
        h = C.c_void_p()
        check(L.cg_plan2d_create_vec(C.byref(h), int(device), int(vol_prec), shape_p, sp_p, off_p,
                                     int(det_prec), int(det_count),
                                     v.ctypes.data_as(C.POINTER(C.c_float)), n))
        self._h = h
        self._L = L
        self.device_id = int(device)
        self.vol_prec = int(vol_prec)
        self.det_prec = int(det_prec)
        self.vol_shape = (int(shape_a[0]), int(shape_a[1]))
        self.det_count = int(det_count)
        self.nangles = n


def _check_2d(vol, sino, plan: plan_2d):
    _check_tensor(vol, "volume", 2, half=True)
    _check_tensor(sino, "sinogram", 2, half=True)
    if vol.device != sino.device:
        raise AttributeError("Volume and sinogram must be on the same device")
    if vol.device.index != plan.device_id:
        raise AttributeError("Volume and plan are not on the same device")
    if _bits(vol) != plan.vol_prec:
        kind = "f16" if vol.dtype == torch.float16 else "f32"
        raise AttributeError(f"Plan precision does not match volume precision ({kind})")
    if tuple(vol.shape) != plan.vol_shape:
        raise ValueError(f"volume shape {tuple(vol.shape)} != plan {plan.vol_shape}")
    if tuple(sino.shape) != (plan.nangles, plan.det_count):
        raise ValueError(f"sinogram shape {tuple(sino.shape)} != plan "
                         f"{(plan.nangles, plan.det_count)}")


def wait_timeouts() -> int:
    """Thread blocks of this library's kernels on the current device whose
    bounded wait for their own bulk copies gave up since the last call
    (``cg_wait_timeouts``, which reads and clears the count; it waits for the
    device).  0 when all is well; otherwise the outputs of the launches in
    between are not to be trusted."""
    n = C.c_ulonglong()
    check(load().cg_wait_timeouts(C.byref(n)))
    return n.value


class WaitTimeoutError(RuntimeError):
    """A kernel's bounded wait for its own bulk copies gave up: the results
    computed since the previous check are not to be trusted."""


def raise_on_wait_timeouts() -> None:
    """Raises ``WaitTimeoutError`` when a bounded wait gave up since the last
    check (synchronises with the device).  The operators call it after every
    launch when the environment variable ``CURADON_GB300_CHECK_WAITS`` is 1."""
    n = wait_timeouts()
    if n:
        raise WaitTimeoutError(f"{n} thread block(s) gave up waiting for their bulk copies; "
                               "the results since the last check are not to be trusted")


_CHECK_WAITS = os.environ.get("CURADON_GB300_CHECK_WAITS", "0") == "1"


def _after_launch() -> None:
    if _CHECK_WAITS:
        raise_on_wait_timeouts()


def forward_2d(volume, sinogram, plan: plan_2d):
    """Overwrites ``sinogram`` (nangles, det) with the projection of ``volume``."""
    _check_2d(volume, sinogram, plan)
    check(plan._L.cg_forward_2d_ex(plan.handle, C.c_void_p(volume.data_ptr()),
                                   C.c_void_p(sinogram.data_ptr()), _bits(sinogram),
                                   _stream(volume)))
    _after_launch()


def backward_2d(volume, sinogram, plan: plan_2d):
    """Adds the backprojection of ``sinogram`` to ``volume``."""
    _check_2d(volume, sinogram, plan)
    check(plan._L.cg_backward_2d_ex(plan.handle, C.c_void_p(volume.data_ptr()),
                                    C.c_void_p(sinogram.data_ptr()), _bits(sinogram),
                                    _stream(volume)))
    _after_launch()


def adjoint_2d(volume, sinogram, plan: plan_2d):
    """Adds the matched adjoint (exact transpose of ``forward_2d``) of
    ``sinogram`` to ``volume`` (float32 only)."""
    _check_2d(volume, sinogram, plan)
    if volume.dtype != torch.float32 or sinogram.dtype != torch.float32:
        raise TypeError("the matched adjoint takes float32 tensors")
    check(plan._L.cg_adjoint_2d(plan.handle, C.c_void_p(volume.data_ptr()),
                                C.c_void_p(sinogram.data_ptr()), _stream(volume)))


class plan_3d:
    """Cone-beam plan over the argument list of ``forward_3d``/``backward_3d``;
    ``angles`` is (3, nangles) = (phi, theta, psi)."""

    def __init__(self, device, vol_shape, vol_spacing, vol_offset, angles, det_shape,
                 det_spacing, det_offset, det_rotation, DSO, DSD, COR=0.0):
        L = load()
        ang = np.asarray(angles, np.float32)
        if ang.ndim == 1:
            ang = np.vstack([ang, np.zeros_like(ang), np.zeros_like(ang)])
        keep = [_u64(vol_shape), _f32(vol_spacing), _f32(vol_offset), _f32(ang[0]), _f32(ang[1]),
                _f32(ang[2]), _u64(det_shape), _f32(det_spacing), _f32(det_offset),
                _f32(det_rotation)]
        p = [k[1] for k in keep]
        h = C.c_void_p()
        check(L.cg_plan3d_create(C.byref(h), int(device), p[0], p[1], p[2], p[3], p[4], p[5],
                                 ang.shape[1], p[6], p[7], p[8], p[9], float(DSO), float(DSD),
                                 float(COR)))
        self._h, self._L = h, L
        self.device_id = int(device)
        self.vol_shape = tuple(int(v) for v in keep[0][0])
        self.det_shape = tuple(int(v) for v in keep[6][0])
        self.nangles = ang.shape[1]

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            self._L.cg_plan3d_destroy(h)
            self._h = None

    @property
    def handle(self):
        return self._h

    @property
    def algorithm(self):
        f, b = C.c_int(), C.c_int()
        check(self._L.cg_plan3d_get_algorithm(self._h, C.byref(f), C.byref(b)))
        return _algo_name(f.value, FORWARD_3D), _algo_name(b.value, BACKWARD_3D)

    def set_algorithm(self, forward=None, backward=None):
        check(self._L.cg_plan3d_set_algorithm(
            self._h, _algo_index(forward, FORWARD_3D, "forward"),
            _algo_index(backward, BACKWARD_3D, "backward")))

    def _check(self, vol, sino):
        _check_tensor(vol, "volume", 3)
        _check_tensor(sino, "sinogram", 3)
        if vol.device != sino.device:
            raise AttributeError("Volume and sinogram must be on the same device")
        if vol.device.index != self.device_id:
            raise AttributeError("Volume and plan are not on the same device")
        if tuple(vol.shape) != self.vol_shape:
            raise ValueError(f"volume shape {tuple(vol.shape)} != plan {self.vol_shape}")
        if tuple(sino.shape) != (self.nangles, *self.det_shape):
            raise ValueError(f"sinogram shape {tuple(sino.shape)} != plan "
                             f"{(self.nangles, *self.det_shape)}")

    def forward(self, volume, sinogram):
        self._check(volume, sinogram)
        check(self._L.cg_forward_3d_plan(self._h, C.c_void_p(volume.data_ptr()),
                                         C.c_void_p(sinogram.data_ptr()), _stream(volume)))

    def backward(self, volume, sinogram):
        self._check(volume, sinogram)
        check(self._L.cg_backward_3d_plan(self._h, C.c_void_p(volume.data_ptr()),
                                          C.c_void_p(sinogram.data_ptr()), _stream(volume)))


    def adjoint(self, volume, sinogram):
        """Adds the matched adjoint of ``forward`` to ``volume``."""
        self._check(volume, sinogram)
        check(self._L.cg_adjoint_3d_plan(self._h, C.c_void_p(volume.data_ptr()),
                                         C.c_void_p(sinogram.data_ptr()), _stream(volume)))


def _call_3d(fn_name, x, vol_shape, vol_spacing, vol_offset, sinogram, a0, a1, a2, sino_shape,
             det_spacing, det_offset, det_rotation, DSO, DSD, COR):
    _check_tensor(x, "x", 3)
    _check_tensor(sinogram, "sinogram", 3)
    if x.device != sinogram.device:
        raise AttributeError("Volume and sinogram must be on the same device")
    keep = [_u64(vol_shape), _f32(vol_spacing), _f32(vol_offset), _f32(a0), _f32(a1), _f32(a2),
            _u64(sino_shape), _f32(det_spacing), _f32(det_offset), _f32(det_rotation)]
    n = keep[3][0].size
    if tuple(x.shape) != tuple(int(v) for v in keep[0][0]):
        raise ValueError("x shape does not match vol_shape")
    if tuple(sinogram.shape) != (n, *(int(v) for v in keep[6][0])):
        raise ValueError("sinogram shape does not match (nangles, *sino_shape)")
    p = [k[1] for k in keep]
    L = load()
    with torch.cuda.device(x.device):
        check(getattr(L, fn_name)(C.c_void_p(x.data_ptr()), p[0], p[1], p[2],
                                  C.c_void_p(sinogram.data_ptr()), p[3], p[4], p[5], n, p[6], p[7],
                                  p[8], p[9], float(DSO), float(DSD), float(COR), _stream(x)))


def forward_3d(x, vol_shape, vol_spacing, vol_offset, sinogram, psi, theta, phi, sino_shape,
               det_spacing, det_offset, det_rotation, DSO, DSD, COR):
    """Per-call 3D forward with the reference's argument list (forward.cu:141-143).

    The 6th argument is named ``psi`` there but is used as phi, as the
    reference does (forward.cu:60-66); ``curadon.forward`` passes
    ``geom.angles[0]`` in that position."""
    _call_3d("cg_forward_3d", x, vol_shape, vol_spacing, vol_offset, sinogram, psi, theta, phi,
             sino_shape, det_spacing, det_offset, det_rotation, DSO, DSD, COR)


def backward_3d(x, vol_shape, vol_spacing, vol_offset, sinogram, phi, theta, psi, sino_shape,
                det_spacing, det_offset, det_rotation, DSO, DSD, COR):
    """Per-call 3D backprojection (backward.cu:20-72, bound at :135-140),
    accumulating into x."""
    _call_3d("cg_backward_3d", x, vol_shape, vol_spacing, vol_offset, sinogram, phi, theta, psi,
             sino_shape, det_spacing, det_offset, det_rotation, DSO, DSD, COR)
