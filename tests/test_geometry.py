"""CPU tests of the geometry objects (reference geometry.py semantics)."""
import numpy as np
import pytest

from curadon_gb300 import ConeGeometry, FanGeometry, geom_to_str


def fan(**kw):
    a = dict(DSD=np.full(8, 30.0), DSO=np.full(8, 20.0),
             angles=np.linspace(0, 2 * np.pi, 8, endpoint=False), vol_shape=(16, 16),
             det_shape=24)
    a.update(kw)
    return FanGeometry(**a)


def test_defaults():
    g = fan()
    assert g.det_spacing == 1.0 and g.det_offset == 0.0 and g.det_rotation == 0.0
    assert np.array_equal(g.vol_spacing, [1, 1]) and np.array_equal(g.vol_offset, [0, 0])
    assert g.sinogram_shape() == (8, 24)


def test_scalar_dso_is_replaced_by_dsd_like_the_reference():
    g = fan(DSD=30.0, DSO=20.0)
    assert np.all(g.DSO == 30.0) and np.all(g.DSD == 30.0)


@pytest.mark.parametrize("kw,exc", [
    (dict(angles=np.zeros((2, 2))), AttributeError),
    (dict(DSD=np.ones(3)), AttributeError),
    (dict(DSO=np.ones(3)), AttributeError),
    (dict(vol_shape=(1, 2, 3)), AttributeError),
    (dict(det_shape="x"), AttributeError),
    (dict(det_spacing="x"), TypeError),
    (dict(det_offset=[1, 2]), TypeError),
    (dict(vol_spacing=(1, 2, 3)), AttributeError),
    (dict(vol_offset=(1,)), AttributeError),
])
def test_fan_validation(kw, exc):
    with pytest.raises(exc):
        fan(**kw)


def test_to_vec_from_vec_round_trip():
    rng = np.random.default_rng(0)
    n = 12
    g = fan(DSD=rng.uniform(50, 60, n), DSO=rng.uniform(20, 30, n),
            angles=np.sort(rng.uniform(0, 2 * np.pi, n)), det_spacing=1.0)
    vecs = g.to_vec()
    assert len(vecs) == n and len(vecs[0]) == 6
    h = FanGeometry.from_vec((16, 16), 24, vecs)
    assert np.allclose(h.DSD, g.DSD) and np.allclose(h.DSO, g.DSO)
    assert np.allclose(np.mod(h.angles, 2 * np.pi), np.mod(g.angles, 2 * np.pi))
    assert h.det_spacing == pytest.approx(1.0)


def test_from_vec_rejects_unequal_spacing():
    v = fan().to_vec()
    v[1][4] *= 2
    with pytest.raises(AttributeError):
        FanGeometry.from_vec((16, 16), 24, v)


def test_cone_angles_forms():
    g = ConeGeometry(DSD=300, DSO=200, angles=np.linspace(0, 1, 5), vol_shape=(8, 8, 8),
                     det_shape=(10, 12))
    assert g.angles.shape == (3, 5) and g.nangles == 5
    assert g.sinogram_shape() == (5, 10, 12)
    with pytest.raises(AttributeError):
        ConeGeometry(DSD=3, DSO=2, angles=np.zeros((2, 5)), vol_shape=(8, 8, 8),
                     det_shape=(10, 12))
    with pytest.raises(TypeError):
        ConeGeometry(DSD="a", DSO=2, angles=[0.0], vol_shape=(8, 8, 8), det_shape=(10, 12))
    with pytest.raises(AttributeError):
        ConeGeometry(DSD=3, DSO=2, angles=[0.0], vol_shape=(8, 8), det_shape=(10, 12))


def test_str():
    assert "DSD" in geom_to_str(fan())
    assert "vol_shape" in str(ConeGeometry(DSD=3, DSO=2, angles=[0.0], vol_shape=(8, 8, 8),
                                           det_shape=(10, 12)))


def test_vec_geometry_keeps_the_vectors():
    from curadon_gb300 import FanVecGeometry

    g = FanGeometry(DSD=300.0, DSO=[200.0] * 4, angles=[0.0, 0.5, 1.0, 2.0], vol_shape=(32, 32),
                    det_shape=40, det_spacing=1.0)
    vecs = np.asarray(g.to_vec())
    vecs[:, 0] += 0.25  # a source shift the angle/DSO/DSD reduction cannot hold
    vg = FanGeometry.from_vec((32, 32), 40, vecs, lossless=True)
    assert isinstance(vg, FanVecGeometry) and isinstance(vg, FanGeometry)
    assert np.array_equal(np.asarray(vg.to_vec()), vecs)
    assert vg.sinogram_shape() == (4, 40) and vg.det_spacing == 1.0
    lossy = FanGeometry.from_vec((32, 32), 40, vecs)
    assert not isinstance(lossy, FanVecGeometry)
    with pytest.raises(AttributeError):
        FanVecGeometry((32, 32), 40, vecs[:, :5])
