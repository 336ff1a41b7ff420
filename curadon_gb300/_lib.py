"""Loads ``libcuradon_gb300.so`` (the sm_103a kernels behind the C ABI).

There is no fallback: if the library is missing, importing an operator fails
with the build command to run.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

_LIB_PATH = Path(__file__).resolve().parent / "libcuradon_gb300.so"
_lib = None

u64p = C.POINTER(C.c_uint64)
f32p = C.POINTER(C.c_float)

# (name, restype, argtypes) of every function declared in include/curadon_gb300.h
SIGNATURES = [
    ("cg_last_error", C.c_char_p, []),
    ("cg_version", C.c_int, []),
    ("cg_plan2d_create", C.c_int,
     [C.POINTER(C.c_void_p), C.c_int, C.c_uint32, u64p, f32p, f32p, C.c_uint32, C.c_uint64,
      C.c_float, C.c_float, f32p, f32p, f32p, C.c_uint64, C.c_float, C.c_float]),
    ("cg_plan2d_create_vec", C.c_int,
     [C.POINTER(C.c_void_p), C.c_int, C.c_uint32, u64p, f32p, f32p, C.c_uint32, C.c_uint64,
      f32p, C.c_uint64]),
    ("cg_plan2d_destroy", C.c_int, [C.c_void_p]),
    ("cg_plan2d_get_forward_block", C.c_int, [C.c_void_p, u64p, u64p]),
    ("cg_plan2d_set_forward_block", C.c_int, [C.c_void_p, C.c_uint64, C.c_uint64]),
    ("cg_plan2d_set_algorithm", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("cg_plan2d_get_algorithm", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("cg_plan2d_get_symmetry", C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    ("cg_plan2d_set_shapes", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("cg_wait_timeouts", C.c_int, [C.POINTER(C.c_ulonglong)]),
    ("cg_plan2d_get_shapes", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("cg_plan2d_tables", C.c_int, [C.c_void_p, f32p, f32p, f32p]),
    ("cg_forward_2d", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cg_backward_2d", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cg_forward_2d_ex", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("cg_backward_2d_ex", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("cg_adjoint_2d", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cg_plan3d_create", C.c_int,
     [C.POINTER(C.c_void_p), C.c_int, u64p, f32p, f32p, f32p, f32p, f32p, C.c_uint64, u64p, f32p,
      f32p, f32p, C.c_float, C.c_float, C.c_float]),
    ("cg_plan3d_destroy", C.c_int, [C.c_void_p]),
    ("cg_plan3d_set_algorithm", C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    ("cg_plan3d_get_algorithm", C.c_int, [C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    ("cg_forward_3d_plan", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cg_backward_3d_plan", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cg_adjoint_3d_plan", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("cg_forward_3d", C.c_int,
     [C.c_void_p, u64p, f32p, f32p, C.c_void_p, f32p, f32p, f32p, C.c_uint64, u64p, f32p, f32p,
      f32p, C.c_float, C.c_float, C.c_float, C.c_void_p]),
    ("cg_backward_3d", C.c_int,
     [C.c_void_p, u64p, f32p, f32p, C.c_void_p, f32p, f32p, f32p, C.c_uint64, u64p, f32p, f32p,
      f32p, C.c_float, C.c_float, C.c_float, C.c_void_p]),
    ("cg_backward_2d_static", C.c_int,
     [C.c_void_p, C.c_void_p, u64p, f32p, f32p, C.c_uint64, C.c_float, f32p, f32p, f32p,
      C.c_uint64, C.c_void_p]),
    ("cg_filter_rows", C.c_int,
     [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint64, C.c_uint64, C.c_float,
      C.c_void_p]),
    ("cg_batch2d_create", C.c_int,
     [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
      C.POINTER(C.c_void_p), C.c_int]),
    ("cg_batch2d_destroy", C.c_int, [C.c_void_p]),
    ("cg_batch2d_forward", C.c_int, [C.c_void_p, C.c_void_p]),
    ("cg_batch2d_backward", C.c_int, [C.c_void_p, C.c_void_p]),
    ("cg_batch2d_adjoint", C.c_int, [C.c_void_p, C.c_void_p]),
    ("cg_batch2d_set_active", C.c_int, [C.c_void_p, C.c_int]),
    ("cg_batch2d_set_forward", C.c_int, [C.c_void_p, C.c_int]),
    ("cg_batch2d_get_forward", C.c_int, [C.c_void_p, C.POINTER(C.c_int)]),
    ("cg_batch3d_create", C.c_int,
     [C.POINTER(C.c_void_p), C.POINTER(C.c_void_p), C.POINTER(C.c_void_p),
      C.POINTER(C.c_void_p), C.c_int]),
    ("cg_batch3d_destroy", C.c_int, [C.c_void_p]),
    ("cg_batch3d_forward", C.c_int, [C.c_void_p, C.c_void_p]),
    ("cg_batch3d_backward", C.c_int, [C.c_void_p, C.c_void_p]),
    ("cg_batch3d_adjoint", C.c_int, [C.c_void_p, C.c_void_p]),
    ("cg_batch3d_set_active", C.c_int, [C.c_void_p, C.c_int]),
]

CG_OK, CG_ERR_INVALID, CG_ERR_CUDA, CG_ERR_NOMEM, CG_ERR_UNSUPPORTED = range(5)


class CuradonError(RuntimeError):
    """A C-ABI call returned an error status."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def lib_path() -> Path:
    return _LIB_PATH


def load() -> C.CDLL:
    global _lib
    if _lib is None:
        if not _LIB_PATH.exists():
            raise ImportError(
                f"{_LIB_PATH.name} is not built; run `python -m curadon_gb300._build` "
                "(or __graft_entry__.build()) on a machine with nvcc")
        L = C.CDLL(str(_LIB_PATH))
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(rc: int) -> None:
    if rc != CG_OK:
        msg = load().cg_last_error().decode(errors="replace")
        if rc == CG_ERR_INVALID:
            raise ValueError(msg)
        if rc == CG_ERR_UNSUPPORTED:
            raise NotImplementedError(msg)
        if rc == CG_ERR_NOMEM:
            raise MemoryError(msg)
        raise CuradonError(rc, msg)
