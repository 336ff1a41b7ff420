"""CPU tests of the FP64 oracle: known answers, symmetries, and its pin
against the golden vectors made by the reference's own CUDA operators."""
import numpy as np
import pytest

import oracle
from conftest import load_golden, max_abs, rel_l2
from curadon_gb300 import FanGeometry
from curadon_gb300.phantom import ellipses_2d, fan_config


def disc(n, r, cx=0.0, cy=0.0):
    c = np.arange(n) - n / 2 + 0.5
    Y, X = np.meshgrid(c, c, indexing="ij")
    return (((X - cx) ** 2 + (Y - cy) ** 2) <= r * r).astype(np.float32)


G0 = fan_config(64, 360, 91, 1.5, 256.0, 384.0)


def test_disc_central_chord():
    s = oracle.fwd2d(G0, disc(64, 20.0))
    # the central cell of an odd detector passes through the centre at every
    # angle: chord 40 up to the pixel staircase of the disc's edge
    assert s[0, 45] == pytest.approx(40.0, abs=1e-9)
    assert np.all(np.abs(s[:, 45] - 40.0) < 1.0)
    assert s[:, 45].mean() == pytest.approx(40.0, abs=0.2)


def test_disc_chord_profile():
    # a large disc: the ray at distance d from the centre has chord 2 sqrt(r^2-d^2)
    n, r = 128, 50.0
    g = fan_config(n, 8, 181, 1.0, 4000.0, 4000.0 + 1e-3)  # almost parallel rays
    s = oracle.fwd2d(g, disc(n, r))
    d = (np.arange(181) - 90) * 1.0
    chord = 2 * np.sqrt(np.clip(r * r - d * d, 0, None))
    inner = np.abs(d) < r - 3
    assert np.max(np.abs(s[0, inner] - chord[inner])) < 1.2


def test_rotation_symmetry():
    # a centred radial Gaussian is invariant under rotation: every view is
    # the same up to interpolation error
    c = np.arange(64) - 32 + 0.5
    Y, X = np.meshgrid(c, c, indexing="ij")
    blob = np.exp(-(X * X + Y * Y) / (2 * 8.0**2)).astype(np.float32)
    s = oracle.fwd2d(G0, blob)
    assert rel_l2(s, np.broadcast_to(s[0], s.shape)) < 2e-3


def test_quarter_turn_of_image_is_quarter_turn_of_views():
    ph = ellipses_2d(64, 3).numpy()
    g = fan_config(64, 4, 91, 1.5, 256.0, 384.0)
    s = oracle.fwd2d(g, ph)
    # view k+1 of the image equals view k of the image rotated by 90 degrees
    rot = np.ascontiguousarray(np.rot90(ph, k=1))
    s_rot = oracle.fwd2d(g, rot)
    assert min(rel_l2(s_rot[0], s[1]), rel_l2(s_rot[0], s[3])) < 1e-6


def test_impulse_backprojection_support():
    # backprojecting one detector cell of one view lights up a thin fan line
    g = fan_config(64, 1, 91, 1.5, 256.0, 384.0)
    sino = np.zeros((1, 91), np.float32)
    sino[0, 45] = 1.0
    vol = oracle.bwd2d(g, sino)
    # angle 0: source on +y, ray along -y through the centre column
    cols = np.nonzero(vol.sum(axis=0))[0]
    assert set(cols) <= {30, 31, 32, 33, 34}
    assert vol.min() >= 0


def test_vol_offset_shifts_sinogram():
    ph = ellipses_2d(64, 5).numpy()
    g = fan_config(64, 2, 91, 1.5, 1e5, 1e5 + 1e-3)  # parallel beam limit
    g.update(vol_offset=(0.0, 3.0))  # (y, x): image moved +3 in x
    s_off = oracle.fwd2d(g, ph)
    shifted = np.zeros_like(ph)
    shifted[:, 3:] = ph[:, :-3]
    g2 = dict(g, vol_offset=(0.0, 0.0))
    s_shift = oracle.fwd2d(g2, shifted)
    assert rel_l2(s_off, s_shift) < 5e-3


def test_backward_is_accumulating():
    ph = ellipses_2d(64, 0).numpy()
    s = oracle.fwd2d(G0, ph).astype(np.float32)
    v1 = oracle.bwd2d(G0, s)
    v2 = oracle.bwd2d(G0, s, vol0=np.ones((64, 64)))
    assert np.allclose(v2, v1 + 1.0)


def test_threads_do_not_change_results():
    ph = ellipses_2d(64, 0).numpy()
    a = oracle.fwd2d(G0, ph, nthreads=1)
    b = oracle.fwd2d(G0, ph, nthreads=7)
    assert np.array_equal(a, b)


# ----------------------------------------------------------- golden pins

@pytest.mark.parametrize("case", ["fan_cfg0", "fan_var"])
def test_oracle_matches_reference_fan(case):
    z, g = load_golden(case)
    for quant in (0, 1):
        s = oracle.fwd2d(g, z["volume"], quant=quant)
        assert rel_l2(s, z["sino_ref"]) < 1e-4, (quant, rel_l2(s, z["sino_ref"]))
        b = oracle.bwd2d(g, z["sino_ref"], quant=quant)
        assert rel_l2(b, z["bwd_ref"]) < 1e-4, (quant, rel_l2(b, z["bwd_ref"]))
    # texture-quantised weights must be at least as close as exact ones
    e0 = rel_l2(oracle.fwd2d(g, z["volume"], quant=0), z["sino_ref"])
    e1 = rel_l2(oracle.fwd2d(g, z["volume"], quant=1), z["sino_ref"])
    assert e1 <= e0 * 1.05


@pytest.mark.parametrize("case", ["fan_cfg0", "fan_var"])
def test_oracle_tables_match_reference(case):
    z, g = load_golden(case)
    src, u0, du = oracle.fan_tables(g)
    assert max_abs(src, z["sources"]) < 1e-3
    assert max_abs(u0, z["u_origins"]) < 1e-2
    assert max_abs(du, z["delta_us"]) < 1e-3


@pytest.mark.parametrize("case", ["cone_small", "cone_rot"])
def test_oracle_matches_reference_cone(case):
    z, g = load_golden(case)
    sref = z["sino_ref"]
    s = oracle.fwd3d(g, z["volume"], sino0=np.full(sref.shape, -7.0), quant=1)
    missed = sref == -7.0
    assert np.array_equal(missed, s == -7.0), "miss pattern differs"
    assert rel_l2(s[~missed], sref[~missed]) < 1e-3, rel_l2(s[~missed], sref[~missed])
    b = oracle.bwd3d(g, z["bwd_in"], vol0=np.ones(z["volume"].shape), quant=1)
    assert rel_l2(b, z["bwd_ref"]) < 1e-3, rel_l2(b, z["bwd_ref"])


def test_vector_oracle_matches_circular():
    """The vector-geometry oracle (direct ray / detector-line intersection)
    reproduces the circular oracle for vectors of a circular geometry."""
    g = fan_config(64, 90, 91, 1.5, 256, 384)
    geom = FanGeometry(**g)
    vecs = np.asarray(geom.to_vec())
    vecs[:, 4:] *= g["det_spacing"]  # u as the cell step
    ph = ellipses_2d(64, 3).numpy()
    a, b = oracle.fwd2d(g, ph), oracle.fwd2d_vec(g, vecs, ph)
    assert np.abs(a - b).max() < 1e-5 * np.abs(a).max()
    s = a.astype(np.float32)
    c, d = oracle.bwd2d(g, s), oracle.bwd2d_vec(g, vecs, s)
    assert np.abs(c - d).max() < 1e-5 * np.abs(c).max()


@pytest.mark.parametrize("reverse", [False, True])
def test_quarter_turn_of_views_turns_the_backprojection(reverse):
    """The identity the quarter-turn backprojection rests on, in the FP64
    restatement: with n views evenly over a full turn, the same row
    backprojected as view v + n/4 gives view v's image turned by 90 degrees
    about the image centre, pixel (x, y) going to (y, W - 1 - x) (the other
    way, (W - 1 - y, x), for reversed angles)."""
    g = dict(G0)
    if reverse:
        g["angles"] = np.ascontiguousarray(-G0["angles"])
    n = len(g["angles"])
    q = n // 4
    rng = np.random.default_rng(11)
    row = rng.uniform(0, 1, g["det_shape"]).astype(np.float32)
    for v in (0, 7, 100):
        s1 = np.zeros((n, g["det_shape"]), np.float32)
        s2 = np.zeros_like(s1)
        s1[v] = row
        s2[(v + q) % n] = row
        a = oracle.bwd2d(g, s1)          # (y, x)
        b = oracle.bwd2d(g, s2)
        W = a.shape[1]
        y, x = np.meshgrid(np.arange(W), np.arange(W), indexing="ij")
        if not reverse:
            turned = b[W - 1 - x, y]     # b at pixel (y, W - 1 - x)
        else:
            turned = b[x, W - 1 - y]     # b at pixel (W - 1 - y, x)
        assert rel_l2(turned, a) < 1e-6, (v, rel_l2(turned, a))
