"""PLY meshes (clovers/src/objects/ply.rs): every body format, coordinate
type and index type loads exactly the triangles of the STL of the same mesh
(same tree, bit-identical oracle ray casts), the product and the oracle build
the same tree, and malformed files are refused with a message.  The GPU ray
casts of a PLY scene are checked bit-exact in test_gpu_raycast.py.

The reference's own bunny (ply/bunny.binary.ply) is loaded when the
environment variable CLOVERS_REFERENCE names a checkout of the reference."""

import json
import os

import numpy as np
import pytest

import clovers_gb300 as cg
import oracle
from clovers_gb300 import scenes


def grid_mesh(n=24, seed=4):
    rng = np.random.default_rng(seed)
    xs, zs = np.meshgrid(np.linspace(-1, 1, n), np.linspace(-1, 1, n), indexing="ij")
    ys = 0.2 * rng.random((n, n))
    v = np.stack([xs, ys, zs], -1).reshape(-1, 3).astype(np.float32)
    f = []
    for i in range(n - 1):
        for j in range(n - 1):
            a, b, c, d = i * n + j, (i + 1) * n + j, (i + 1) * n + j + 1, i * n + j + 1
            f += [(a, b, c), (a, c, d)]
    return v, np.array(f, np.int64)


def mesh_scene(kind, path):
    sc = scenes.dense_mesh_scene("unused.stl")
    for o in sc["objects"]:
        if o.get("kind") == "STL":
            o.update({"kind": kind, "path": path, "scale": 2.5, "center": [0.3, 1.0, -0.2],
                      "rotation": [10.0, 200.0, 30.0]})
    return sc


def load_both(tmp_path, kind, mesh_file, w=64, h=36):
    path = scenes.write_scene(mesh_scene(kind, mesh_file), str(tmp_path / ("%s.json" % kind)))
    return cg.Scene.from_json(path, w, h), oracle.Scene.from_json(path, w, h)


@pytest.fixture(scope="module")
def stl_reference(tmp_path_factory):
    tmp = tmp_path_factory.mktemp("ply")
    v, f = grid_mesh()
    stl = scenes.write_binary_stl(str(tmp / "mesh.stl"), v[f])
    prod, orc = load_both(tmp, "STL", stl)
    rays = scenes.random_rays(4096, seed=8)
    rays[:, :3] = rays[:, :3] * 4.0 - 2.0  # origins around the mesh
    prim, t = orc.raycast(rays)
    return v, f, prod.info(), orc.tree_stats(), rays, prim, t


@pytest.mark.parametrize("fmt", ["binary_little_endian", "binary_big_endian", "ascii"])
@pytest.mark.parametrize("coord,index", [("float", "int"), ("double", "uint"), ("float", "ushort"),
                                         ("int", "short")])
def test_ply_loads_the_same_triangles_as_stl(tmp_path, stl_reference, fmt, coord, index):
    v, f, info_stl, stats_stl, rays, prim_stl, t_stl = stl_reference
    if coord == "int":
        v = np.round(v * 8.0)  # integer coordinates: compare against the STL of the same values
        stl = scenes.write_binary_stl(str(tmp_path / "int.stl"), v.astype(np.float32)[f])
        _, o_stl = load_both(tmp_path, "STL", stl)
        prim_stl, t_stl = o_stl.raycast(rays)
        stats_stl = o_stl.tree_stats()
    ply = scenes.write_ply(str(tmp_path / "mesh.ply"), v, f, fmt=fmt, coord_type=coord, index_type=index,
                           extra_vertex_props=2)
    prod, orc = load_both(tmp_path, "PLY", ply)
    info = prod.info()
    assert info["triangles"] == info_stl["triangles"] == len(f)
    st = orc.tree_stats()
    assert (info["nodes"], info["tree_depth"], info["mis_nodes"]) == (st["nodes"], st["tree_depth"], st["mis_nodes"])
    assert st == stats_stl
    prim, t = orc.raycast(rays)
    assert np.array_equal(prim, prim_stl) and np.array_equal(t, t_stl)


def test_signed_indices_use_their_absolute_value(tmp_path, stl_reference):
    v, f, _, stats_stl, rays, prim_stl, t_stl = stl_reference
    ply = scenes.write_ply(str(tmp_path / "neg.ply"), v, -f, index_type="int")
    _, orc = load_both(tmp_path, "PLY", ply)
    prim, t = orc.raycast(rays)
    assert np.array_equal(prim, prim_stl) and np.array_equal(t, t_stl)


@pytest.mark.parametrize("text,msg", [
    (b"plx\nformat ascii 1.0\nend_header\n", "PLY"),
    (b"ply\nformat ascii 1.0\nelement vertex 1\nproperty float x\nelement face 0\n"
     b"property list uchar int vertex_indices\nend_header\n0\n", "x, y, z"),
    (b"ply\nformat ascii 1.0\nelement vertex 3\nproperty float x\nproperty float y\nproperty float z\n"
     b"element face 1\nproperty list uchar int vertex_indices\nend_header\n0 0 0\n1 0 0\n0 1 0\n3 0 1 7\n",
     "out of range"),
    (b"ply\nformat ascii 1.0\nelement vertex 3\nproperty uchar x\nproperty float y\nproperty float z\n"
     b"element face 1\nproperty list uchar int vertex_indices\nend_header\n0 0 0\n1 0 0\n0 1 0\n3 0 1 2\n",
     "unsupported"),
    (b"ply\nformat binary_little_endian 1.0\nelement vertex 3\nproperty float x\nproperty float y\n"
     b"property float z\nelement face 1\nproperty list uchar int vertex_indices\nend_header\n\x00\x00", "ends early"),
])
def test_malformed_ply_is_refused(tmp_path, text, msg):
    p = tmp_path / "bad.ply"
    p.write_bytes(text)
    path = scenes.write_scene(mesh_scene("PLY", str(p)), str(tmp_path / "bad.json"))
    with pytest.raises(cg.ClvError) as e:
        cg.Scene.from_json(path, 64, 36)
    assert e.value.code == -2 and msg in str(e.value)


REFERENCE = os.environ.get("CLOVERS_REFERENCE", "")


@pytest.mark.skipif(not REFERENCE or not os.path.isdir(os.path.join(REFERENCE, "scenes")),
                    reason="CLOVERS_REFERENCE does not name a reference checkout")
def test_reference_bunny_loads():
    ref = REFERENCE
    text = open(os.path.join(ref, "scenes", "bunny.json")).read()
    info = cg.Scene.from_json_text(text, 400, 400, base_dir=ref).info()
    assert info["triangles"] == 69451  # ply/README.md: 69,451 faces
    assert 0 < info["tree_depth"] <= 64
