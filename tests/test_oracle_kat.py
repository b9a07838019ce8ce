"""The oracle against the reference's own known-answer and property tests.

Each case restates a test of the reference (file:line cited) with the same
inputs and expected values; nothing here needs a GPU.
"""

import numpy as np
import pytest

import oracle

F32_EPS = np.float32(1.1920929e-07)


# clovers/src/spectrum.rs:74-101 -- exact f32 results of the spectral uplift
@pytest.mark.parametrize("xyz,expected", [((1.0, 1.0, 1.0), np.float32(1.000_000_7)),
                                          ((0.0, 0.0, 0.0), np.float32(0.0)),
                                          ((2.0, 2.0, 2.0), np.float32(2.000_001_4))])
def test_spectral_power_kat(xyz, expected):
    assert oracle.spectral_power(xyz, 600) == expected


# clovers/tests/spectrum.rs:5-27 -- every wavelength converts for black, grey and white
@pytest.mark.parametrize("grey", [0.0, 0.5, 1.0])
def test_spectral_power_all_wavelengths(grey):
    vals = [oracle.spectral_power((grey, grey, grey), lam) for lam in range(380, 780)]
    assert all(np.isfinite(vals))
    if grey > 0:
        assert min(vals) > 0


# clovers/tests/wavelength.rs:4-27
def test_rotate_wavelength_properties():
    for lam in range(380, 780):
        w = oracle.rotate_wavelength(lam)
        assert w[0] == lam
        s = sorted(w)
        d = s[1] - s[0]
        assert s[2] - s[1] == d and s[3] - s[2] == d
        assert all(380 <= x < 780 for x in w)


def test_wavelength_into_xyz_all():
    xyz = np.array([oracle.wavelength_into_xyz(lam) for lam in range(380, 780)])
    assert np.all(np.isfinite(xyz))
    # the CIE 1931 fit peaks: y near 555 nm, z near 445 nm
    assert 540 <= 380 + int(np.argmax(xyz[:, 1])) <= 570
    assert 430 <= 380 + int(np.argmax(xyz[:, 2])) <= 460


# clovers/src/interval.rs:69-99
def test_interval_kat():
    mn, mx, size, center = oracle.interval(0.0, 1.0)
    assert (mn, mx, size, center) == (0.0, 1.0, 1.0, 0.5)
    mn, mx, size, center = oracle.interval(-1.0, 1.0)
    assert size == 2.0 and center == 0.0
    mn, mx, _, _ = oracle.interval(1.0, -1.0)  # Interval::new orders its ends
    assert (mn, mx) == (-1.0, 1.0)


# clovers/src/aabb.rs:185-282
def test_aabb_kat():
    assert oracle.aabb_area([0, 1, 0, 1, 0, 1]) == 6.0
    assert oracle.aabb_area([0, 1, 0, 2, 0, 3]) == 22.0
    assert oracle.aabb_area([-1, 0, -2, 0, -3, 0]) == 22.0
    assert list(oracle.aabb_centroid([0, 1, 0, 1, 0, 1])) == [0.5, 0.5, 0.5]
    assert list(oracle.aabb_centroid([0, 0, 0, 0, 0, 0])) == [0.0, 0.0, 0.0]
    assert list(oracle.aabb_combine([0] * 6, [0] * 6)) == [0.0] * 6
    assert list(oracle.aabb_combine([0] * 6, [0, 1, 0, 1, 0, 1])) == [0, 1, 0, 1, 0, 1]
    assert list(oracle.aabb_combine([0, 1, 0, 1, 0, 1], [0, -1, 0, -1, 0, -1])) == [-1, 1, -1, 1, -1, 1]


RAY_POS = [0.01, 0.01, -1.0, 0.0, 0.0, 0.0, 1.0, 1.0]      # tmin/tmax = TIME_0/TIME_1 for the box test
RAY_NEG = [-0.01, -0.01, -1.0, 0.0, 0.0, 0.0, 1.0, 1.0]
INF = float("inf")


# clovers/src/objects/triangle.rs:262-416: four unit triangles
@pytest.mark.parametrize("u,v,ray,front", [
    ((1, 0, 0), (0, 1, 0), RAY_POS, False),
    ((0, 1, 0), (1, 0, 0), RAY_POS, True),
    ((-1, 0, 0), (0, -1, 0), RAY_NEG, False),
    ((0, -1, 0), (-1, 0, 0), RAY_NEG, True),
])
def test_triangle_kat(u, v, ray, front):
    hit_ray = list(ray)
    hit_ray[3], hit_ray[7] = -INF, INF  # the hit itself is tested over (-inf, inf)
    hit, rec, box = oracle.prim_hit(1, (0, 0, 0), u, v, hit_ray)
    lo = -1.0 if min(u + v) < 0 else 0.0
    eps = np.float32(0.0001)
    expected_box = np.array([lo, lo + 1, lo, lo + 1, -eps, eps], np.float32)
    assert np.array_equal(box, expected_box)
    assert oracle.aabb_hit(box, ray)
    assert hit
    assert rec[0] - 1.0 <= F32_EPS
    assert list(rec[1:4]) == [np.float32(ray[0]), np.float32(ray[1]), 0.0]
    assert list(rec[4:7]) == [0.0, 0.0, -1.0]
    assert bool(rec[9]) == front


def test_quad_and_sphere_basics():
    # a quad accepts t on the closed interval, a sphere only on the open one
    hit, rec, _ = oracle.prim_hit(2, (0, 0, 0), (1, 0, 0), (0, 1, 0), [0.5, 0.5, -1, 1.0, 0, 0, 1, 1.0])
    assert hit and rec[0] == 1.0
    hit, rec, _ = oracle.prim_hit(3, (0, 0, 0), (1, 0, 0), (0, 0, 0), [0, 0, -2, 1.0, 0, 0, 1, 1.0])
    assert not hit  # root at exactly t=1 is outside (1, 1)
    hit, rec, _ = oracle.prim_hit(3, (0, 0, 0), (1, 0, 0), (0, 0, 0), [0, 0, -2, 0.001, 0, 0, 1, 10.0])
    assert hit and rec[0] == 1.0 and bool(rec[9])


def test_srgb_roundtrip():
    for rgb in [(0.73, 0.73, 0.73), (0.65, 0.05, 0.05), (0.12, 0.45, 0.15), (1, 1, 1), (0, 0, 0)]:
        xyz = oracle.srgb_to_xyz_e(rgb)
        back = oracle.xyz_e_to_srgb8(xyz)[0]
        assert np.all(np.abs(back.astype(int) - np.round(np.array(rgb) * 255).astype(int)) <= 1)
    # sRGB white maps to the equal-energy white (1, 1, 1) up to rounding
    assert np.allclose(oracle.srgb_to_xyz_e((1, 1, 1)), [1, 1, 1], atol=2e-4)
