"""Host-side logic of serving (no GPU): geometry keys for resident plans and
the memory estimate admission uses."""
import numpy as np
import torch

from curadon_gb300 import ConeGeometry, FanGeometry, FanVecGeometry
from curadon_gb300.phantom import cone_config, fan_config
from curadon_gb300.serve import Request, _geom_key, request_bytes


def test_geometry_keys():
    a = FanGeometry(**fan_config(128, 90))
    b = FanGeometry(**fan_config(128, 90))
    c = FanGeometry(**fan_config(128, 91))
    assert _geom_key(a) == _geom_key(b) != _geom_key(c)
    v = np.asarray(a.to_vec())
    assert _geom_key(FanVecGeometry((128, 128), a.det_shape, v)) != _geom_key(a)
    assert _geom_key(ConeGeometry(**cone_config(32, 20, 48))) != _geom_key(a)


def test_memory_estimate_grows_with_the_problem():
    def req(kind, n):
        g = FanGeometry(**fan_config(n, n))
        return Request(kind, g, torch.zeros(g.sinogram_shape()))

    small, large = request_bytes(req("fbp", 128)), request_bytes(req("fbp", 1024))
    assert 0 < small < large
    # the volume and sinogram alone are a lower bound
    assert large >= 4 * (1024 * 1024 + 1024 * 1449)
    assert request_bytes(req("sirt", 256)) > request_bytes(req("fbp", 256))


def test_coalescing_classes():
    """2D FBP / SIRT requests below 704^2 pixels coalesce by geometry, kind,
    iteration count and filter; larger 2D and all 3D requests run alone."""
    from curadon_gb300.serve import _batchable, _class_key

    small = FanGeometry(**fan_config(256, 90))
    same = FanGeometry(**fan_config(256, 90))
    big = FanGeometry(**fan_config(1024, 90))
    cone = ConeGeometry(**cone_config(32, 20, 48))

    def req(kind, g, iters=20, filt="ram-lak"):
        return Request(kind, g, torch.zeros(g.sinogram_shape()), iters=iters, filter_name=filt)

    assert _batchable(req("fbp", small)) and _batchable(req("sirt", small))
    assert not _batchable(req("fbp", big)) and not _batchable(req("cgls", cone))
    assert not _batchable(req("cgls", small))
    assert _class_key(req("fbp", small)) == _class_key(req("fbp", same))
    assert _class_key(req("fbp", small)) != _class_key(req("sirt", small))
    assert _class_key(req("sirt", small, 20)) != _class_key(req("sirt", small, 10))
    assert _class_key(req("fbp", small)) != _class_key(req("fbp", small, filt="hann"))
    # FBP ignores the iteration count
    assert _class_key(req("fbp", small, 0)) == _class_key(req("fbp", small, 20))


def test_heavy_requests_are_the_3d_ones():
    from curadon_gb300.serve import _heavy

    fan = FanGeometry(**fan_config(2048, 90))
    cone = ConeGeometry(**cone_config(32, 20, 48))
    assert _heavy(Request("cgls", cone, torch.zeros(cone.sinogram_shape())))
    assert not _heavy(Request("sirt", fan, torch.zeros(fan.sinogram_shape())))
