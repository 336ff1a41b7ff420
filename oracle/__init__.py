"""FP64 CPU oracle of curadon's projection operators (test infrastructure).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline /
reference leg may import this package, and only as the checker or as the
timed CPU baseline; the product path (``curadon_gb300``) never does.

``liboracle.so`` is ``oracle.c`` compiled with gcc; the functions below take
numpy arrays in Python axis order and a geometry given either as a dict or
as any object with the attributes of curadon's ``FanGeometry`` /
``ConeGeometry`` (vol_shape, vol_spacing, vol_offset, det_shape,
det_spacing, det_offset, angles, DSO, DSD, and for cones det_rotation, COR).

``RefOps`` drives the reference's own CUDA operators through
``oracle/_ref/libcuradon_ref.so`` (see ``build_ref.py``) where that library
could be built.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
LIB_PATH = ORACLE_DIR / "liboracle.so"
REF_DIR = ORACLE_DIR / "_ref"
REF_LIB = REF_DIR / "libcuradon_ref.so"

_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")


class Fan2d(C.Structure):
    _fields_ = [("W", C.c_int64), ("H", C.c_int64), ("sx", C.c_double), ("sy", C.c_double),
                ("ox", C.c_double), ("oy", C.c_double), ("det_count", C.c_int64),
                ("det_spacing", C.c_double), ("det_offset", C.c_double),
                ("nangles", C.c_int64), ("angles", C.c_void_p), ("DSO", C.c_void_p),
                ("DSD", C.c_void_p)]


class Cone3d(C.Structure):
    _fields_ = [("X", C.c_int64), ("Y", C.c_int64), ("Z", C.c_int64), ("sx", C.c_double),
                ("sy", C.c_double), ("sz", C.c_double), ("ox", C.c_double), ("oy", C.c_double),
                ("oz", C.c_double), ("U", C.c_int64), ("V", C.c_int64), ("su", C.c_double),
                ("sv", C.c_double), ("offu", C.c_double), ("offv", C.c_double),
                ("pitch", C.c_double), ("roll", C.c_double), ("yaw", C.c_double),
                ("DSO", C.c_double), ("DSD", C.c_double), ("COR", C.c_double),
                ("nangles", C.c_int64), ("phi", C.c_void_p), ("theta", C.c_void_p),
                ("psi", C.c_void_p)]


def build(force: bool = False) -> Path:
    src = ORACLE_DIR / "oracle.c"
    if force or not LIB_PATH.exists() or LIB_PATH.stat().st_mtime < max(
            src.stat().st_mtime, (ORACLE_DIR / "oracle.h").stat().st_mtime):
        tmp = LIB_PATH.with_suffix(".so.tmp")
        subprocess.run(["gcc", "-O2", "-std=c11", "-shared", "-fPIC", "-pthread", "-o", str(tmp),
                        str(src), "-lm"], check=True)
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB_PATH))
        for name, st in (("or_fwd2d", Fan2d), ("or_bwd2d", Fan2d)):
            f = getattr(L, name)
            f.argtypes = [C.POINTER(st), _f32p, _f64p, C.c_int, C.c_int]
            f.restype = C.c_int
        for name in ("or_fwd3d", "or_bwd3d"):
            f = getattr(L, name)
            f.argtypes = [C.POINTER(Cone3d), _f32p, _f64p, C.c_int, C.c_int]
            f.restype = C.c_int
        L.or_fan2d_tables.argtypes = [C.POINTER(Fan2d), _f64p, _f64p, _f64p]
        L.or_fan2d_vec_tables.argtypes = [C.POINTER(Fan2d), _f64p, _f64p, _f64p, _f64p]
        L.or_fwd2d_vec.argtypes = [C.POINTER(Fan2d), _f64p, _f32p, _f64p, C.c_int, C.c_int]
        L.or_bwd2d_vec.argtypes = [C.POINTER(Fan2d), _f64p, _f32p, _f64p, C.c_int, C.c_int]
        L.or_fwd2d_vec.restype = L.or_bwd2d_vec.restype = C.c_int
        L.or_cone3d_fwd_tables.argtypes = [C.POINTER(Cone3d), _f64p, _f64p, _f64p, _f64p]
        L.or_cone3d_bwd_tables.argtypes = [C.POINTER(Cone3d)] + [_f64p] * 5
        _lib = L
    return _lib


def default_threads() -> int:
    return max(1, os.cpu_count() or 1)


def _get(g, name):
    return g[name] if isinstance(g, dict) else getattr(g, name)


def _opt(g, name, default):
    try:
        v = _get(g, name)
    except (KeyError, AttributeError):
        return default
    return default if v is None else v


def _f32(a):
    return np.ascontiguousarray(np.asarray(a, dtype=np.float32).ravel())


def fan_struct(g):
    """(struct, keep-alive arrays) for a fan geometry in Python axis order."""
    H, W = (int(v) for v in _get(g, "vol_shape"))
    sy, sx = (float(v) for v in _opt(g, "vol_spacing", (1.0, 1.0)))
    oy, ox = (float(v) for v in _opt(g, "vol_offset", (0.0, 0.0)))
    angles = _f32(_get(g, "angles"))
    n = angles.size
    DSO = _f32(np.broadcast_to(np.asarray(_get(g, "DSO"), np.float32), (n,)))
    DSD = _f32(np.broadcast_to(np.asarray(_get(g, "DSD"), np.float32), (n,)))
    det = int(_get(g, "det_shape"))
    s = Fan2d(W, H, sx, sy, ox, oy, det, float(_opt(g, "det_spacing", 1.0)),
              float(_opt(g, "det_offset", 0.0)), n, angles.ctypes.data, DSO.ctypes.data,
              DSD.ctypes.data)
    return s, (angles, DSO, DSD)


def cone_struct(g):
    Z, Y, X = (int(v) for v in _get(g, "vol_shape"))
    sz, sy, sx = (float(v) for v in _opt(g, "vol_spacing", (1.0, 1.0, 1.0)))
    oz, oy, ox = (float(v) for v in _opt(g, "vol_offset", (0.0, 0.0, 0.0)))
    V, U = (int(v) for v in _get(g, "det_shape"))
    sv, su = (float(v) for v in _opt(g, "det_spacing", (1.0, 1.0)))
    ov, ou = (float(v) for v in _opt(g, "det_offset", (0.0, 0.0)))
    pitch, roll, yaw = (float(v) for v in _opt(g, "det_rotation", (0.0, 0.0, 0.0)))
    ang = np.asarray(_get(g, "angles"), dtype=np.float32)
    if ang.ndim == 1:
        ang = np.vstack([ang, np.zeros_like(ang), np.zeros_like(ang)])
    phi, theta, psi = (_f32(a) for a in ang)
    s = Cone3d(X, Y, Z, sx, sy, sz, ox, oy, oz, U, V, su, sv, ou, ov, pitch, roll, yaw,
               float(_get(g, "DSO")), float(_get(g, "DSD")), float(_opt(g, "COR", 0.0)),
               phi.size, phi.ctypes.data, theta.ctypes.data, psi.ctypes.data)
    return s, (phi, theta, psi)


def fwd2d(g, vol, quant: int = 0, nthreads: int | None = None) -> np.ndarray:
    """Sinogram (nangles, det) in float64 of a (H, W) volume."""
    s, keep = fan_struct(g)
    v = np.ascontiguousarray(vol, dtype=np.float32)
    assert v.shape == (s.H, s.W), (v.shape, (s.H, s.W))
    out = np.zeros((s.nangles, s.det_count), np.float64)
    lib().or_fwd2d(C.byref(s), v, out, quant, nthreads or default_threads())
    del keep
    return out


def bwd2d(g, sino, vol0=None, quant: int = 0, nthreads: int | None = None) -> np.ndarray:
    """Volume (H, W) float64: vol0 (default 0) plus the backprojection."""
    s, keep = fan_struct(g)
    sg = np.ascontiguousarray(sino, dtype=np.float32)
    assert sg.shape == (s.nangles, s.det_count), (sg.shape, (s.nangles, s.det_count))
    out = (np.zeros((s.H, s.W), np.float64) if vol0 is None
           else np.array(vol0, dtype=np.float64, copy=True))
    lib().or_bwd2d(C.byref(s), sg, out, quant, nthreads or default_threads())
    del keep
    return out


def _vec_struct(g, vecs):
    """Fan struct for per-view vectors (nangles, 6); det_spacing = |u| of view 0."""
    v = np.ascontiguousarray(np.asarray(vecs, np.float64).reshape(-1, 6))
    n = v.shape[0]
    h = dict(g)
    h["angles"] = np.zeros(n, np.float32)
    h["DSO"] = np.ones(n, np.float32)
    h["DSD"] = np.full(n, 2.0, np.float32)
    h["det_spacing"] = float(np.hypot(v[0, 4], v[0, 5]))
    h["det_offset"] = 0.0
    s, keep = fan_struct(h)
    return s, keep, v


def fan_vec_tables(g, vecs):
    """FP64 (sources, u_origins, delta_us) of a vector geometry, each (nangles, 2)."""
    s, keep, v = _vec_struct(g, vecs)
    n = s.nangles
    src, u0, du = (np.zeros(2 * n) for _ in range(3))
    lib().or_fan2d_vec_tables(C.byref(s), v, src, u0, du)
    del keep
    return src.reshape(n, 2), u0.reshape(n, 2), du.reshape(n, 2)


def fwd2d_vec(g, vecs, vol, quant: int = 0, nthreads: int | None = None) -> np.ndarray:
    """Forward projection of a (H, W) volume through per-view vectors
    [S.x, S.y, C.x, C.y, U.x, U.y]; g supplies vol_shape, det_shape and the
    voxel spacing / offset."""
    s, keep, v = _vec_struct(g, vecs)
    vv = np.ascontiguousarray(vol, dtype=np.float32)
    out = np.zeros((s.nangles, s.det_count), np.float64)
    lib().or_fwd2d_vec(C.byref(s), v, vv, out, quant, nthreads or default_threads())
    del keep
    return out


def bwd2d_vec(g, vecs, sino, vol0=None, quant: int = 0,
              nthreads: int | None = None) -> np.ndarray:
    """Backprojection through per-view vectors (direct ray / detector-line
    intersection per pixel and view)."""
    s, keep, v = _vec_struct(g, vecs)
    sg = np.ascontiguousarray(sino, dtype=np.float32)
    out = (np.zeros((s.H, s.W), np.float64) if vol0 is None
           else np.array(vol0, dtype=np.float64, copy=True))
    lib().or_bwd2d_vec(C.byref(s), v, sg, out, quant, nthreads or default_threads())
    del keep
    return out


def fwd3d(g, vol, sino0=None, quant: int = 0, nthreads: int | None = None) -> np.ndarray:
    """Sinogram (nangles, V, U) float64; rays that miss keep sino0 (default 0)."""
    s, keep = cone_struct(g)
    v = np.ascontiguousarray(vol, dtype=np.float32)
    assert v.shape == (s.Z, s.Y, s.X), (v.shape, (s.Z, s.Y, s.X))
    out = (np.zeros((s.nangles, s.V, s.U), np.float64) if sino0 is None
           else np.array(sino0, dtype=np.float64, copy=True))
    lib().or_fwd3d(C.byref(s), v, out, quant, nthreads or default_threads())
    del keep
    return out


def bwd3d(g, sino, vol0=None, quant: int = 0, nthreads: int | None = None) -> np.ndarray:
    s, keep = cone_struct(g)
    sg = np.ascontiguousarray(sino, dtype=np.float32)
    assert sg.shape == (s.nangles, s.V, s.U), (sg.shape, (s.nangles, s.V, s.U))
    out = (np.zeros((s.Z, s.Y, s.X), np.float64) if vol0 is None
           else np.array(vol0, dtype=np.float64, copy=True))
    lib().or_bwd3d(C.byref(s), sg, out, quant, nthreads or default_threads())
    del keep
    return out


def fan_tables(g):
    """FP64 (sources, u_origins, delta_us), each (nangles, 2)."""
    s, keep = fan_struct(g)
    n = s.nangles
    src, u0, du = (np.zeros(2 * n) for _ in range(3))
    lib().or_fan2d_tables(C.byref(s), src, u0, du)
    del keep
    return src.reshape(n, 2), u0.reshape(n, 2), du.reshape(n, 2)


# ------------------------------------------------------------ reference ops

class RefOps:
    """The reference's CUDA operators via ``oracle/_ref/libcuradon_ref.so``.

    Arguments are torch CUDA tensors (or raw device pointers) in Python axis
    order; each call is synchronous, as the reference's are.
    """

    def __init__(self, path: Path = REF_LIB):
        if not Path(path).exists():
            raise FileNotFoundError(f"reference shim not built: {path}")
        L = C.CDLL(str(path))
        u64p, f32p = C.POINTER(C.c_uint64), C.POINTER(C.c_float)
        L.ref_plan2d_create.restype = C.c_void_p
        L.ref_plan2d_create.argtypes = [C.c_uint64, u64p, f32p, f32p, C.c_uint64, C.c_float,
                                        C.c_float, f32p, f32p, f32p, C.c_uint64, C.c_float,
                                        C.c_float, C.c_uint32, C.c_uint32]
        L.ref_plan2d_destroy.argtypes = [C.c_void_p]
        L.ref_plan2d_tables.argtypes = [C.c_void_p, f32p, f32p, f32p]
        L.ref_forward2d.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_backward2d.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_forward2d_t.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        L.ref_backward2d_t.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int]
        args3 = [C.c_void_p, u64p, f32p, f32p, C.c_void_p, f32p, f32p, f32p, C.c_uint64, u64p,
                 f32p, f32p, f32p, C.c_float, C.c_float, C.c_float]
        L.ref_forward3d.argtypes = args3
        L.ref_backward3d.argtypes = args3
        L.ref_sync.restype = C.c_int
        self.L = L

    @staticmethod
    def _arr(a, ct, dt):
        a = np.ascontiguousarray(np.asarray(a, dtype=dt).ravel())
        return a, a.ctypes.data_as(C.POINTER(ct))

    def plan2d(self, g, vol_prec: int = 32, det_prec: int = 32):
        H, W = (int(v) for v in _get(g, "vol_shape"))
        keep = []

        def a(v, ct=C.c_float, dt=np.float32):
            arr, p = self._arr(v, ct, dt)
            keep.append(arr)
            return p

        angles = _f32(_get(g, "angles"))
        n = angles.size
        DSO = np.broadcast_to(np.asarray(_get(g, "DSO"), np.float32), (n,))
        DSD = np.broadcast_to(np.asarray(_get(g, "DSD"), np.float32), (n,))
        h = self.L.ref_plan2d_create(
            0, a([H, W], C.c_uint64, np.uint64), a(_opt(g, "vol_spacing", (1.0, 1.0))),
            a(_opt(g, "vol_offset", (0.0, 0.0))), int(_get(g, "det_shape")),
            float(_opt(g, "det_spacing", 1.0)), float(_opt(g, "det_offset", 0.0)), a(DSO), a(DSD),
            a(angles), n, float(_opt(g, "det_rotation", 0.0)), 0.0, vol_prec, det_prec)
        return h, n

    def plan2d_tables(self, h, n):
        out = [np.zeros(2 * n, np.float32) for _ in range(3)]
        self.L.ref_plan2d_tables(h, *(o.ctypes.data_as(C.POINTER(C.c_float)) for o in out))
        return [o.reshape(n, 2) for o in out]

    def forward2d(self, h, vol_ptr, sino_ptr):
        self.L.ref_forward2d(h, vol_ptr, sino_ptr)

    def backward2d(self, h, vol_ptr, sino_ptr):
        self.L.ref_backward2d(h, vol_ptr, sino_ptr)

    def forward2d_typed(self, h, vol, sino):
        """Forward with the tensors' element types (float32 / float16)."""
        bits = lambda t: 16 if t.element_size() == 2 else 32  # noqa: E731
        self.L.ref_forward2d_t(h, vol.data_ptr(), sino.data_ptr(), bits(vol), bits(sino))

    def backward2d_typed(self, h, vol, sino):
        bits = lambda t: 16 if t.element_size() == 2 else 32  # noqa: E731
        self.L.ref_backward2d_t(h, vol.data_ptr(), sino.data_ptr(), bits(vol), bits(sino))

    def destroy2d(self, h):
        self.L.ref_plan2d_destroy(h)

    def _call3d(self, fn, g, vol_ptr, sino_ptr):
        keep = []

        def a(v, ct=C.c_float, dt=np.float32):
            arr, p = self._arr(v, ct, dt)
            keep.append(arr)
            return p

        ang = np.asarray(_get(g, "angles"), np.float32)
        if ang.ndim == 1:
            ang = np.vstack([ang, np.zeros_like(ang), np.zeros_like(ang)])
        fn(vol_ptr, a(_get(g, "vol_shape"), C.c_uint64, np.uint64),
           a(_opt(g, "vol_spacing", (1, 1, 1))), a(_opt(g, "vol_offset", (0, 0, 0))), sino_ptr,
           a(ang[0]), a(ang[1]), a(ang[2]), ang.shape[1],
           a(_get(g, "det_shape"), C.c_uint64, np.uint64), a(_opt(g, "det_spacing", (1, 1))),
           a(_opt(g, "det_offset", (0, 0))), a(_opt(g, "det_rotation", (0, 0, 0))),
           float(_get(g, "DSO")), float(_get(g, "DSD")), float(_opt(g, "COR", 0.0)))

    def forward3d(self, g, vol_ptr, sino_ptr):
        self._call3d(self.L.ref_forward3d, g, vol_ptr, sino_ptr)

    def backward3d(self, g, vol_ptr, sino_ptr):
        self._call3d(self.L.ref_backward3d, g, vol_ptr, sino_ptr)

    def sync(self):
        return self.L.ref_sync()


def ref_available() -> bool:
    return REF_LIB.exists()
