"""The allocation-free backprojection entry point, cg_backward_2d_static.

It exists for callers that cannot call cudaMalloc (a server whose device
memory is reserved up front by its own pool, a real-time loop that must not
wait on the allocator, a plugin host that forbids library allocations): all
its scratch sits in a fixed 16 MiB device array inside the library.  These
tests call it through the C ABI and compare it with the plan-based
cg_backward_2d on the same inputs, twice in a row with different problems
(the array keeps the previous call's contents and must be fully rewritten).
This file is collected last so a failure here cannot hide other results."""
import ctypes as C

import numpy as np
import pytest

from conftest import max_abs, rel_l2
from curadon_gb300 import _build, _lib
from curadon_gb300.phantom import fan_config

TOL = 1e-3


def _call_static(L, vol, sino, g, stream):
    H, W = g["vol_shape"]
    keep = [np.array([H, W], np.uint64), np.ones(2, np.float32), np.zeros(2, np.float32),
            np.ascontiguousarray(g["DSO"], np.float32), np.ascontiguousarray(g["DSD"], np.float32),
            np.ascontiguousarray(g["angles"], np.float32)]
    f = lambda a: a.ctypes.data_as(C.POINTER(C.c_float))
    return L.cg_backward_2d_static(
        C.c_void_p(vol), C.c_void_p(sino), keep[0].ctypes.data_as(C.POINTER(C.c_uint64)),
        f(keep[1]), f(keep[2]), int(g["det_shape"]), float(g["det_spacing"]), f(keep[3]),
        f(keep[4]), f(keep[5]), len(g["angles"]), C.c_void_p(stream))


@pytest.mark.gpu
def test_static_backprojection_matches_plan_twice(cuda_device):
    import torch

    from curadon_gb300 import FanGeometry, backward_2d

    L = _lib.load()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    for call, (n, nangles) in enumerate([(256, 180), (200, 97)]):
        g = fan_config(n, nangles)
        geom = FanGeometry(**g)
        rng = np.random.default_rng(call)
        sino = torch.as_tensor(rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32),
                               device=cuda_device)
        v0 = torch.as_tensor(rng.uniform(0, 1, (n, n)).astype(np.float32), device=cuda_device)
        expect = v0.clone()
        backward_2d(expect, sino, geom.plan)
        got = v0.clone()
        rc = _call_static(L, got.data_ptr(), sino.data_ptr(), g, stream)
        assert rc == _lib.CG_OK, L.cg_last_error()
        torch.cuda.synchronize()
        e = rel_l2(got.cpu(), expect.cpu())
        print(f"call {call}: n={n} rel-L2 {e:.2e} max-abs {max_abs(got.cpu(), expect.cpu()):.2e}")
        assert e <= TOL


def test_static_rejects_problems_beyond_its_scratch():
    _build.build()
    L = _lib.load()
    g = fan_config(2048)  # 2048 views x 2901 cells x 8 B > 16 MiB
    rc = _call_static(L, 1 << 20, 1 << 20, g, 0)
    assert rc == _lib.CG_ERR_INVALID
    assert b"static scratch" in L.cg_last_error()


@pytest.mark.gpu
@pytest.mark.parametrize("algo", ["bwd2d=tex", "bwd2d=alu", "bwd2d=smem,bwd2d_minb=27"])
def test_static_backprojection_under_algorithm_override(cuda_device, monkeypatch, algo):
    """An override naming a backprojector that would allocate (the texture
    unit) or another staged variant must not change the result: the entry
    point runs a kernel that needs only its own scratch, on the sinogram
    copy that kernel reads."""
    import torch

    from curadon_gb300 import FanGeometry, backward_2d

    L = _lib.load()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    g = fan_config(192, 150)
    geom = FanGeometry(**g)  # plan made before the override: the default kernels
    rng = np.random.default_rng(11)
    sino = torch.as_tensor(rng.uniform(0, 1, geom.sinogram_shape()).astype(np.float32),
                           device=cuda_device)
    expect = torch.zeros((192, 192), device=cuda_device)
    backward_2d(expect, sino, geom.plan)
    monkeypatch.setenv("CURADON_GB300_ALGO", algo)
    for _ in range(2):
        got = torch.zeros_like(expect)
        rc = _call_static(L, got.data_ptr(), sino.data_ptr(), g, stream)
        assert rc == _lib.CG_OK, L.cg_last_error()
        torch.cuda.synchronize()
        e = rel_l2(got.cpu(), expect.cpu())
        print(f"{algo}: rel-L2 {e:.2e}")
        assert e <= TOL
