"""GPU closest-hit ray casts against the oracle: bit-exact hit ids and
distances, and identical traversal counts (BVHNode::hit calls and primitive
tests per ray), through the C ABI."""

import numpy as np
import pytest

import clovers_gb300 as cg
import oracle
from clovers_gb300 import scenes

pytestmark = pytest.mark.gpu


def _compare(dscene, oscene, rays):
    prim, t, nodes, tests = cg.raycast(dscene, rays, with_counts=True)
    oprim, ot, onodes, otests = oscene.raycast(rays, with_counts=True)
    assert np.array_equal(prim, oprim), "hit ids differ on %d rays" % int((prim != oprim).sum())
    hit = oprim != 0xFFFFFFFF
    assert np.array_equal(t[hit].view(np.uint32), ot[hit].view(np.uint32)), "hit distances differ"
    assert np.array_equal(nodes, onodes), "BVH node visit counts differ"
    assert np.array_equal(tests, otests), "primitive test counts differ"
    assert dscene.status() == 0
    return hit.mean()


@pytest.mark.parametrize("ntris,nrays", [(1, 4096), (2, 4096), (7, 4096), (4096, 65536), (65536, 262144)])
def test_triangle_soup_parity(ntris, nrays):
    v, i = scenes.triangle_soup(ntris, seed=5)
    rays = scenes.random_rays(nrays, seed=6)
    d = cg.Scene.from_mesh(v, i).upload()
    frac = _compare(d, oracle.Scene.from_mesh(v, i), rays)
    if ntris >= 4096:
        assert frac > 0.1


def test_full_depth_tree_parity():
    """The ray-cast workload's own tree: 2^20 random triangles (SAH, depth 29),
    2^20 of its random rays; ids, distance bits and traversal counts equal the
    oracle's on every ray."""
    v, i = scenes.triangle_soup(1 << 20, seed=2)
    rays = scenes.random_rays(1 << 20, seed=3)
    h = cg.Scene.from_mesh(v, i)
    assert h.info()["tree_depth"] >= 25
    frac = _compare(h.upload(), oracle.Scene.from_mesh(v, i), rays)
    assert frac > 0.5


def test_shared_edges_and_grid_rays():
    # a regular grid mesh: many rays hit edges and vertices shared by two or more triangles
    n = 64
    xs = np.linspace(0, 1, n + 1, dtype=np.float32)
    gx, gy = np.meshgrid(xs, xs)
    verts = np.stack([gx.ravel(), gy.ravel(), np.zeros(gx.size, np.float32)], 1).astype(np.float32)
    idx = []
    for r in range(n):
        for c in range(n):
            a = r * (n + 1) + c
            idx += [[a, a + 1, a + n + 1], [a + 1, a + n + 2, a + n + 1]]
    idx = np.array(idx, np.uint32)
    g = np.linspace(0, 1, 257, dtype=np.float32)
    ox, oy = np.meshgrid(g, g)
    rays = np.zeros((ox.size, 8), np.float32)
    rays[:, 0], rays[:, 1], rays[:, 2] = ox.ravel(), oy.ravel(), -1.0
    rays[:, 3], rays[:, 6], rays[:, 7] = 0.001, 1.0, np.float32(3.4e38)
    d = cg.Scene.from_mesh(verts, idx).upload()
    # the reference's plane-then-barycentric test is not watertight: rays through shared
    # edges can miss both triangles; the GPU must miss exactly the same ones
    assert _compare(d, oracle.Scene.from_mesh(verts, idx), rays) > 0.3


def test_axis_aligned_and_degenerate_rays():
    v, i = scenes.triangle_soup(2048, seed=8)
    rng = np.random.default_rng(9)
    rays = np.zeros((6 * 2048, 8), np.float32)
    rays[:, 0:3] = rng.random((rays.shape[0], 3))
    for k in range(6):  # +-x, +-y, +-z directions: zero components give inf/NaN slabs
        rays[k * 2048:(k + 1) * 2048, 4 + k // 2] = 1.0 if k % 2 == 0 else -1.0
    rays[:, 3], rays[:, 7] = 0.001, np.float32(3.4e38)
    d = cg.Scene.from_mesh(v, i).upload()
    _compare(d, oracle.Scene.from_mesh(v, i), rays)


def test_box_scene_parity(box_scene_path):
    w = h = 96
    d = cg.Scene.from_json(box_scene_path, w, h).upload()
    o = oracle.Scene.from_json(box_scene_path, w, h)
    cam = scenes.camera_rays(w, h, lambda pu, pv: o.camera_ray(pu, pv))
    rays = np.concatenate([cam, scenes.random_rays(20000, seed=4) * np.array([555] * 3 + [1] * 5, np.float32)])
    assert _compare(d, o, rays) > 0.5


def test_spheres_scene_parity(spheres_scene_path):
    w, h = 80, 45
    d = cg.Scene.from_json(spheres_scene_path, w, h).upload()
    o = oracle.Scene.from_json(spheres_scene_path, w, h)
    cam = scenes.camera_rays(w, h, lambda pu, pv: o.camera_ray(pu, pv))
    _compare(d, o, cam)


def test_empty_ray_batch():
    v, i = scenes.triangle_soup(16, seed=1)
    d = cg.Scene.from_mesh(v, i).upload()
    prim, t = cg.raycast(d, np.zeros((0, 8), np.float32))
    assert prim.size == 0 and t.size == 0


def test_fast_slab_division_is_ieee_division():
    import ctypes
    from clovers_gb300 import _lib
    bad = ctypes.c_uint64()
    _lib.check(_lib.lib().clv_selftest_division(1 << 28, 12345, ctypes.byref(bad)))
    assert bad.value == 0


def test_ply_mesh_scene_parity(tmp_path):
    # a PLY mesh (big-endian binary body) in a scene with lights and a floor, origins around the mesh
    rng = np.random.default_rng(12)
    n = 48
    xs, zs = np.meshgrid(np.linspace(-1, 1, n), np.linspace(-1, 1, n), indexing="ij")
    v = np.stack([xs, 0.3 * rng.random((n, n)), zs], -1).reshape(-1, 3).astype(np.float32)
    f = np.array([(i * n + j, (i + 1) * n + j, (i + 1) * n + j + 1) for i in range(n - 1) for j in range(n - 1)] +
                 [(i * n + j, (i + 1) * n + j + 1, i * n + j + 1) for i in range(n - 1) for j in range(n - 1)])
    ply = scenes.write_ply(str(tmp_path / "m.ply"), v, f, fmt="binary_big_endian")
    sc = scenes.dense_mesh_scene("unused.stl")
    for o in sc["objects"]:
        if o.get("kind") == "STL":
            o.update({"kind": "PLY", "path": ply, "scale": 2.0, "center": [0.0, 1.0, 0.0], "rotation": [5, 40, 0]})
    path = scenes.write_scene(sc, str(tmp_path / "s.json"))
    rays = scenes.random_rays(131072, seed=13)
    rays[:, :3] = rays[:, :3] * 6.0 - 3.0
    frac = _compare(cg.Scene.from_json(path, 64, 36).upload(), oracle.Scene.from_json(path, 64, 36), rays)
    assert frac > 0.2


@pytest.mark.parametrize("rotate", [False, True])
def test_watertight_mode_parity_and_no_leaks(rotate):
    # CLV_OPT_WATERTIGHT: the GPU's watertight triangle and conservative box tests against the oracle's
    tris = scenes.displaced_icosphere(24, amplitude=0.0)
    uv, inv = np.unique(tris.reshape(-1, 3), axis=0, return_inverse=True)
    v = uv @ np.linalg.qr(np.random.default_rng(3).normal(size=(3, 3)))[0].T if rotate else uv
    v = v.astype(np.float32)
    f = inv.astype(np.uint32).reshape(-1, 3)
    rng = np.random.default_rng(2)
    e = rng.integers(0, len(f), 200000)
    s = rng.random(200000).astype(np.float32)
    targets = np.concatenate([v, v[f[e, 0]] + (v[f[e, 1]] - v[f[e, 0]]) * s[:, None]])
    origin = np.array([0.1, -0.05, 0.2], np.float32)
    d = targets - origin
    rays = np.zeros((len(d), 8), np.float32)
    rays[:, :3] = origin
    rays[:, 4:7] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays[:, 7] = 3.4e38
    dscene = cg.Scene.from_mesh(v, f).set_watertight().upload()
    frac = _compare(dscene, oracle.Scene.from_mesh(v, f).set_watertight(), rays)
    assert frac == 1.0  # from inside a closed mesh every ray through an edge or a vertex hits
    # random rays through the whole mesh, default mode untouched by the option of another scene
    rays2 = scenes.random_rays(65536, seed=9)
    rays2[:, :3] = rays2[:, :3] * 3.0 - 1.5
    _compare(dscene, oracle.Scene.from_mesh(v, f).set_watertight(), rays2)
    _compare(cg.Scene.from_mesh(v, f).upload(), oracle.Scene.from_mesh(v, f), rays2)


def test_raycast_into_caller_arrays():
    """Repeated host-buffer casts can reuse their output arrays: the same ids
    and distances as fresh arrays; arrays of the wrong type or size are refused."""
    v, idx = scenes.triangle_soup(4096, seed=7)
    d = cg.Scene.from_mesh(v, idx).upload()
    rays = scenes.random_rays(20000, seed=8)
    prim, t = cg.raycast(d, rays)
    out = (np.full(len(rays), 7, np.uint32), np.full(len(rays), -1.0, np.float32))
    for _ in range(2):
        p2, t2 = cg.raycast(d, rays, out=out)
        assert p2 is out[0] and t2 is out[1]
        assert np.array_equal(p2, prim) and np.array_equal(t2, t)
    with pytest.raises(ValueError):
        cg.raycast(d, rays, out=(np.empty(len(rays), np.int64), np.empty(len(rays), np.float32)))
    with pytest.raises(ValueError):
        cg.raycast(d, rays, out=(np.empty(len(rays) - 1, np.uint32), np.empty(len(rays), np.float32)))


@pytest.mark.parametrize("which", ["box", "spheres"])
def test_lam_tree_parity(box_scene_path, spheres_scene_path, which):
    """Ray casts through longest-axis-midpoint trees (`--bvh lam`): ids,
    distances and visit counts equal the oracle's on its own LAM tree."""
    path = box_scene_path if which == "box" else spheres_scene_path
    w, h = 96, 72
    d = cg.Scene.from_json(path, w, h, bvh="lam").upload()
    o = oracle.Scene.from_json(path, w, h, bvh="lam")
    cam = scenes.camera_rays(w, h, lambda pu, pv: o.camera_ray(pu, pv))
    extra = scenes.random_rays(20000, seed=9)
    if which == "box":
        extra = extra * np.array([555] * 3 + [1] * 5, np.float32)
    assert _compare(d, o, np.concatenate([cam, extra])) > 0.3
