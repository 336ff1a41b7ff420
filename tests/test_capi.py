"""CPU tests of the C-ABI library: it builds, loads, exports every function
the header declares, and rejects bad arguments before touching the GPU."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

from curadon_gb300 import _build, _lib

HEADER = Path(__file__).resolve().parents[1] / "include" / "curadon_gb300.h"


@pytest.fixture(scope="module")
def lib():
    _build.build()
    return _lib.load()


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(cg_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_boundary():
    names = declared_functions()
    for required in ("cg_plan2d_create", "cg_forward_2d", "cg_backward_2d", "cg_forward_3d",
                     "cg_backward_3d", "cg_last_error"):
        assert required in names


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name


def test_python_signatures_cover_the_header():
    assert sorted(n for n, _, _ in _lib.SIGNATURES) == declared_functions()


def test_version(lib):
    assert lib.cg_version() == 10000


def _plan_args(**over):
    n = 4
    a = dict(device=0, vol_prec=32, shape=np.array([8, 8], np.uint64),
             sp=np.ones(2, np.float32), off=np.zeros(2, np.float32), det_prec=32, det=12,
             ds=1.0, doff=0.0, dso=np.full(n, 20, np.float32), dsd=np.full(n, 30, np.float32),
             ang=np.linspace(0, 3, n).astype(np.float32), n=n)
    a.update(over)
    return a


def _create(lib, a):
    h = C.c_void_p()
    f = C.POINTER(C.c_float)
    rc = lib.cg_plan2d_create(C.byref(h), a["device"], a["vol_prec"],
                              a["shape"].ctypes.data_as(C.POINTER(C.c_uint64)),
                              a["sp"].ctypes.data_as(f), a["off"].ctypes.data_as(f),
                              a["det_prec"], a["det"], a["ds"], a["doff"],
                              a["dso"].ctypes.data_as(f), a["dsd"].ctypes.data_as(f),
                              a["ang"].ctypes.data_as(f), a["n"], 0.0, 0.0)
    return rc, h


def test_invalid_precision_is_rejected(lib):
    rc, h = _create(lib, _plan_args(vol_prec=8))
    assert rc == _lib.CG_ERR_INVALID and not h.value
    assert b"Precision" in lib.cg_last_error()


def test_precisions(lib):
    """16 and 32 pass argument validation (without a GPU the device check is
    what fails), any other width is rejected (plan.cu:20-28)."""
    for prec in (16, 32):
        rc, _ = _create(lib, _plan_args(det_prec=prec))
        assert rc != _lib.CG_ERR_INVALID or b"device" in lib.cg_last_error()
    rc, _ = _create(lib, _plan_args(det_prec=8))
    assert rc == _lib.CG_ERR_INVALID and b"f32 or f16" in lib.cg_last_error()


def test_nonfinite_geometry_is_rejected(lib):
    a = _plan_args()
    a["ang"][1] = np.nan
    rc, _ = _create(lib, a)
    assert rc == _lib.CG_ERR_INVALID and b"finite" in lib.cg_last_error()


def test_zero_views_rejected(lib):
    rc, _ = _create(lib, _plan_args(n=0))
    assert rc == _lib.CG_ERR_INVALID


def test_null_plan_calls_fail_cleanly(lib):
    assert lib.cg_forward_2d(None, None, None, None) == _lib.CG_ERR_INVALID
    assert lib.cg_backward_2d(None, None, None, None) == _lib.CG_ERR_INVALID
    assert lib.cg_forward_2d_ex(None, None, None, 16, None) == _lib.CG_ERR_INVALID
    assert lib.cg_backward_2d_ex(None, None, None, 16, None) == _lib.CG_ERR_INVALID
    assert lib.cg_forward_3d_plan(None, None, None, None) == _lib.CG_ERR_INVALID
    h = C.c_void_p()
    assert lib.cg_batch2d_create(C.byref(h), None, None, None, 1) == _lib.CG_ERR_INVALID
    assert lib.cg_batch2d_forward(None, None) == _lib.CG_ERR_INVALID
    assert lib.cg_batch2d_destroy(None) == _lib.CG_OK
    assert lib.cg_plan2d_destroy(None) == _lib.CG_OK


def test_no_gpu_is_an_error_not_a_crash(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    rc, h = _create(lib, _plan_args())
    assert rc == _lib.CG_ERR_CUDA and not h.value
    assert len(lib.cg_last_error()) > 0


def test_check_maps_codes_to_exceptions(lib):
    with pytest.raises(ValueError):
        _lib.check(_lib.CG_ERR_INVALID)
    with pytest.raises(NotImplementedError):
        _lib.check(_lib.CG_ERR_UNSUPPORTED)
    with pytest.raises(_lib.CuradonError):
        _lib.check(_lib.CG_ERR_CUDA)


def test_batch_entry_points_reject_null(lib):
    """The batch calls check their handle before touching the GPU."""
    assert lib.cg_batch2d_forward(None, None) == _lib.CG_ERR_INVALID
    assert lib.cg_batch2d_backward(None, None) == _lib.CG_ERR_INVALID
    assert lib.cg_batch2d_adjoint(None, None) == _lib.CG_ERR_INVALID
    assert lib.cg_batch2d_set_active(None, 1) == _lib.CG_ERR_INVALID
    assert lib.cg_batch2d_set_forward(None, 2) == _lib.CG_ERR_INVALID
    assert lib.cg_batch2d_destroy(None) == _lib.CG_OK
    h = C.c_void_p()
    assert lib.cg_batch3d_create(C.byref(h), None, None, None, 1) == _lib.CG_ERR_INVALID
    assert lib.cg_batch3d_forward(None, None) == _lib.CG_ERR_INVALID
    assert lib.cg_batch3d_backward(None, None) == _lib.CG_ERR_INVALID
    assert lib.cg_batch3d_adjoint(None, None) == _lib.CG_ERR_INVALID
    assert lib.cg_batch3d_set_active(None, 1) == _lib.CG_ERR_INVALID
    assert lib.cg_batch3d_destroy(None) == _lib.CG_OK
