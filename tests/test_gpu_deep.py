"""BVHs deeper than the 64-entry local traversal stack.

The reference's BVHNode::hit recurses with no depth limit
(clovers/src/bvh/hitable_trait.rs:54,66), and its SAH build peels one object
per level when every centroid is the same (surface_area_heuristic.rs:56-73),
so identical triangles make a chain as deep as their count.  The GPU keeps 64
stack entries in local memory and spills deeper ones to a per-scene global
region sized from the tree depth.  Checked against the oracle on such trees:
ray casts bit-exact (ids, distance bits, traversal counts), same-seed renders,
pixel-exact debug images, a batch holding a deep scene, and the
no-allocation render's refusal of deep trees.
"""

import ctypes
import os

import numpy as np
import pytest

import clovers_gb300 as cg
import oracle
from clovers_gb300 import _lib, scenes

pytestmark = pytest.mark.gpu

COPIES = 150  # identical triangles: a peel chain of about this depth


def deep_mesh(copies=COPIES, soup=2000):
    tri = np.array([[0.3, 0.3, 0.5], [0.7, 0.35, 0.5], [0.4, 0.7, 0.55]], np.float32)
    v0, i0 = scenes.triangle_soup(soup, seed=11)
    v = np.concatenate([np.tile(tri, (copies, 1)), v0])
    i = np.concatenate([np.arange(3 * copies, dtype=np.uint32).reshape(copies, 3), i0 + 3 * copies])
    return v, i


def deep_box_scene(tmp_path):
    tri = np.array([[[150, 100, 250], [400, 120, 260], [250, 420, 300]]], np.float32)
    stl = scenes.write_binary_stl(str(tmp_path / "stack.stl"), np.repeat(tri, 120, axis=0))
    sc = scenes.enclosed_box()
    sc["objects"].append({"kind": "STL", "path": stl, "center": [0, 0, 0], "scale": 1.0, "rotation": [0, 0, 0],
                          "material": sc["objects"][0]["material"]})
    return scenes.write_scene(sc, str(tmp_path / "deep_box.json"))


def test_deep_chain_raycast_parity():
    v, i = deep_mesh()
    h = cg.Scene.from_mesh(v, i)
    o = oracle.Scene.from_mesh(v, i)
    depth = h.info()["tree_depth"]
    assert depth == o.tree_stats()["tree_depth"] and depth >= 100
    rays = scenes.random_rays(1 << 16, seed=12)
    rng = np.random.default_rng(13)  # rays aimed at the stacked triangles
    aim = np.zeros((1 << 14, 8), np.float32)
    aim[:, 0:3] = rng.uniform(0.35, 0.6, (aim.shape[0], 3)).astype(np.float32)
    aim[:, 2] = -1.0
    aim[:, 4:7] = [0.0, 0.0, 1.0]
    aim[:, 3], aim[:, 7] = 0.001, np.float32(3.4e38)
    rays = np.concatenate([rays, aim])
    d = h.upload()
    prim, t, nodes, tests = cg.raycast(d, rays, with_counts=True)
    oprim, ot, onodes, otests = o.raycast(rays, with_counts=True)
    assert np.array_equal(prim, oprim)
    hit = oprim != 0xFFFFFFFF
    assert np.array_equal(t[hit].view(np.uint32), ot[hit].view(np.uint32))
    assert np.array_equal(nodes, onodes) and np.array_equal(tests, otests)
    assert (oprim[-aim.shape[0]:] < COPIES).mean() > 0.3  # the chain is really traversed
    assert nodes.max() >= 100
    p2, t2 = cg.raycast(d, rays)  # the plain (non-counting) variant agrees
    assert np.array_equal(p2, prim) and np.array_equal(t2.view(np.uint32), t.view(np.uint32))
    assert d.status() == 0


def test_deep_scene_render_and_debug_match_oracle(tmp_path):
    path = deep_box_scene(tmp_path)
    w = h = 48
    hs = cg.Scene.from_json(path, w, h)
    assert hs.info()["tree_depth"] > 100
    d = hs.upload()
    o = oracle.Scene.from_json(path, w, h)
    stats = {}
    img = cg.draw(cg.GlobalOptions(quiet=True), cg.RenderOptions(width=w, height=h, samples=16, max_depth=8, seed=9),
                  d, stats=stats)
    assert stats["device_errors"] == 0
    ref = o.render(w, h, 16, 8, seed=9) / 16
    err = float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))
    assert err <= 1e-4, err
    for mode, name in ((1, "normal-map"), (2, "bvh-test-count")):
        film = cg.DeviceBuffer(w * h * 3 * 8).zero()
        opts = cg.render_opts(cg.RenderOptions(width=w, height=h, samples=1, max_depth=1, mode=name, seed=21))
        _lib.check(_lib.lib().clv_render_device(d.handle, ctypes.byref(opts), film.ptr, None))
        gpu = film.to_numpy(np.float64, (w * h, 3)).astype(np.float32)
        assert np.array_equal(gpu, o.render_debug(w, h, mode, 21)), name
    assert d.status() == 0


def test_batch_with_a_deep_scene_equals_single_renders(tmp_path, box_scene_path):
    w = h = 32
    deep = cg.Scene.from_json(deep_box_scene(tmp_path), w, h).upload()
    flat = cg.Scene.from_json(box_scene_path, w, h).upload()
    opts = [cg.render_opts(cg.RenderOptions(width=w, height=h, samples=8, max_depth=8, seed=s)) for s in (3, 4)]
    films = [cg.DeviceBuffer(w * h * 24).zero() for _ in range(2)]
    L = _lib.lib()
    handles = (ctypes.c_void_p * 2)(flat.handle.value, deep.handle.value)
    optarr = (_lib.RenderOptsC * 2)(*opts)
    ptrs = (ctypes.c_void_p * 2)(films[0].ptr, films[1].ptr)
    _lib.check(L.clv_render_batch(handles, optarr, ptrs, 2, None))
    for k, dsc in enumerate((flat, deep)):
        one = cg.DeviceBuffer(w * h * 24).zero()
        _lib.check(L.clv_render_device(dsc.handle, ctypes.byref(optarr[k]), one.ptr, None))
        a, b = films[k].to_numpy(np.float64, (w * h, 3)), one.to_numpy(np.float64, (w * h, 3))
        assert np.allclose(a, b, rtol=1e-9, atol=1e-12)
    assert flat.status() == 0 and deep.status() == 0


def test_no_allocation_render_refuses_deep_trees(tmp_path):
    w = h = 16
    d = cg.Scene.from_json(deep_box_scene(tmp_path), w, h).upload()
    film = cg.DeviceBuffer(w * h * 24).zero()
    opts = cg.render_opts(cg.RenderOptions(width=w, height=h, samples=1, max_depth=4))
    rc = _lib.lib().clv_render_device_noalloc(d.handle, ctypes.byref(opts), film.ptr, None)
    assert rc == _lib.CLV_E_INVALID
    assert b"levels" in _lib.lib().clv_last_error()
