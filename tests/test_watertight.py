"""The optional watertight mode (CLV_OPT_WATERTIGHT; not the reference's
test): Woop et al. 2013 triangle tests and Ize 2013 conservative box tests.
On a closed mesh, rays from inside aimed exactly at vertices and edge points
never escape in watertight mode, while the reference's Triangle::hit lets a
share of them through; the GPU's watertight ray casts are checked bit-exact
against this oracle in test_gpu_raycast.py."""

import numpy as np
import pytest

import clovers_gb300 as cg
import oracle
from clovers_gb300 import scenes


def closed_mesh(rotate):
    tris = scenes.displaced_icosphere(24, amplitude=0.0)
    uv, inv = np.unique(tris.reshape(-1, 3), axis=0, return_inverse=True)
    v = uv
    if rotate:
        v = uv @ np.linalg.qr(np.random.default_rng(3).normal(size=(3, 3)))[0].T
    return v.astype(np.float32), inv.astype(np.uint32).reshape(-1, 3)


def edge_and_vertex_rays(v, f, origin, n=20000, seed=2):
    rng = np.random.default_rng(seed)
    e = rng.integers(0, len(f), n)
    s = rng.random(n).astype(np.float32)
    a, b = v[f[e, 0]], v[f[e, 1]]
    targets = np.concatenate([v, a + (b - a) * s[:, None]])
    d = targets - origin
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.zeros((len(d), 8), np.float32)
    rays[:, :3] = origin
    rays[:, 4:7] = d
    rays[:, 7] = 3.4e38
    return rays


@pytest.mark.parametrize("rotate", [False, True])
@pytest.mark.parametrize("origin", [(0.0, 0.0, 0.0), (0.1, -0.05, 0.2)])
def test_closed_mesh_does_not_leak(rotate, origin):
    v, f = closed_mesh(rotate)
    rays = edge_and_vertex_rays(v, f, np.array(origin, np.float32))
    ref_prim, _ = oracle.Scene.from_mesh(v, f).raycast(rays)
    wt_prim, wt_t = oracle.Scene.from_mesh(v, f).set_watertight().raycast(rays)
    leaks_ref = int((ref_prim == 0xFFFFFFFF).sum())
    print("rays %d: the reference's test misses %d, watertight %d" % (len(rays), leaks_ref,
                                                                       int((wt_prim == 0xFFFFFFFF).sum())))
    assert np.all(wt_prim != 0xFFFFFFFF)
    assert leaks_ref > 0  # the reference's test is not watertight
    r = float(np.linalg.norm(origin))
    assert np.all((wt_t > 0.98 - r) & (wt_t < 1.0 + r + 1e-4))  # the unit geodesic sphere around the origin


def test_watertight_agrees_with_reference_away_from_edges():
    # rays through triangle interiors: both tests hit the same triangle at nearly the same distance
    v, f = closed_mesh(True)
    rng = np.random.default_rng(5)
    e = rng.integers(0, len(f), 5000)
    w = rng.dirichlet([4, 4, 4], 5000).astype(np.float32)
    targets = (w[:, :1] * v[f[e, 0]] + w[:, 1:2] * v[f[e, 1]] + w[:, 2:] * v[f[e, 2]]).astype(np.float32)
    rays = np.zeros((5000, 8), np.float32)
    rays[:, 4:7] = targets / np.linalg.norm(targets, axis=1, keepdims=True)
    rays[:, 7] = 3.4e38
    p0, t0 = oracle.Scene.from_mesh(v, f).raycast(rays)
    p1, t1 = oracle.Scene.from_mesh(v, f).set_watertight().raycast(rays)
    assert np.array_equal(p0, p1)
    assert np.allclose(t0, t1, rtol=1e-5)


def test_scene_option_api():
    v, f = closed_mesh(False)
    s = cg.Scene.from_mesh(v, f)
    assert s.set_watertight(True) is s
    s.set_watertight(False)
    with pytest.raises(cg.ClvError):
        cg._lib.check(cg.lib().clv_scene_set_option(s._h, 99, 1))
    with pytest.raises(cg.ClvError):
        cg._lib.check(cg.lib().clv_scene_set_option(s._h, cg._lib.CLV_OPT_WATERTIGHT, 2))
