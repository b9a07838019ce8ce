"""The longest-axis-midpoint BVH builder (clovers/src/bvh/build/longest_axis_midpoint.rs,
the clovers-cli `--bvh lam` option): the product and the oracle build trees
of the same shape for both the main and the MIS (priority) tree on scenes of
every object kind, including ties of box minima (a row of equal spheres); the
GPU's ray casts through LAM trees are checked bit-exact in test_gpu_raycast.py."""

import os

import pytest

import clovers_gb300 as cg
import oracle
from clovers_gb300 import scenes


def _scenes(tmp):
    stl = scenes.write_binary_stl(os.path.join(tmp, "p.stl"), scenes.prism_triangles())
    row = scenes.enclosed_box()
    row["objects"] += [{"kind": "Sphere", "center": [100.0 + 50.0 * (k % 3), 50.0, 300.0], "radius": 20.0,
                        "material": "white wall"} for k in range(9)]  # equal minima along x in threes
    return {"box": scenes.enclosed_box(), "spheres": scenes.random_spheres(1), "sink": scenes.kitchen_sink(stl),
            "prism": scenes.dispersive_prism(stl), "ties": row}


@pytest.mark.parametrize("name", ["box", "spheres", "sink", "prism", "ties"])
def test_lam_tree_shape_matches_oracle(tmp_path, name):
    path = scenes.write_scene(_scenes(str(tmp_path))[name], str(tmp_path / (name + ".json")))
    info = cg.Scene.from_json(path, 64, 48, bvh="lam").info()
    st = oracle.Scene.from_json(path, 64, 48, bvh="lam").tree_stats()
    assert (info["nodes"], info["tree_depth"], info["mis_nodes"]) == (st["nodes"], st["tree_depth"], st["mis_nodes"])
    sah = oracle.Scene.from_json(path, 64, 48).tree_stats()
    assert st["tree_depth"] <= sah["tree_depth"]  # median splits: a balanced tree
