"""The intersect variant a scene needs (clv_scene_info.traversal_level) is
decided by the objects the BVH reaches: meshes and object lists given at the
top level are flattened into the tree and need only the primitive variant (0);
Translate / RotateY chains over Boxy need the inline chain variant (1); media
and lists nested inside a wrapper need the object interpreter (2).  Host-side
only (no GPU); the GPU tests render every level, also mixed in one batch."""

import clovers_gb300 as cg
from clovers_gb300 import scenes


def level(tmp_path, sc, name):
    path = scenes.write_scene(sc, str(tmp_path / (name + ".json")))
    return cg.Scene.from_json(path, 32, 32).info()["traversal_level"]


def test_reference_workloads(tmp_path):
    prism = scenes.write_binary_stl(str(tmp_path / "prism.stl"), scenes.prism_triangles())
    assert level(tmp_path, scenes.random_spheres(1), "spheres") == 0
    assert level(tmp_path, scenes.dispersive_prism(prism), "prism") == 0  # top-level STL: flattened
    assert level(tmp_path, scenes.enclosed_box(), "box") == 1  # Translate(RotateY(Boxy))
    assert level(tmp_path, scenes.kitchen_sink(prism), "sink") == 2  # media, nested list


def _scene(objects):
    sc = scenes.enclosed_box()
    sc["objects"] = [sc["objects"][5]] + objects  # keep the lamp (a priority object)
    return sc


def test_top_level_list_is_flattened(tmp_path):
    lst = {"kind": "ObjectList", "objects": [
        {"kind": "Sphere", "center": [100, 100, 100], "radius": 20, "material": "white wall"},
        {"kind": "Quad", "q": [0, 0, 0], "u": [50, 0, 0], "v": [0, 0, 50], "material": "white wall"}]}
    assert level(tmp_path, _scene([lst]), "toplist") == 0


def test_wrapped_list_needs_the_interpreter(tmp_path):
    lst = {"kind": "ObjectList", "objects": [
        {"kind": "Sphere", "center": [100, 100, 100], "radius": 20, "material": "white wall"}]}
    assert level(tmp_path, _scene([{"kind": "Translate", "offset": [1, 2, 3], "object": lst}]), "wrapped") == 2


def test_wrapped_mesh_needs_the_interpreter(tmp_path):
    prism = scenes.write_binary_stl(str(tmp_path / "prism.stl"), scenes.prism_triangles())
    mesh = {"kind": "STL", "path": prism, "center": [200, 100, 200], "scale": 50, "rotation": [0, 0, 0],
            "material": "white wall"}
    assert level(tmp_path, _scene([mesh]), "mesh") == 0
    assert level(tmp_path, _scene([{"kind": "RotateY", "angle": 10, "object": mesh}]), "rotmesh") == 2


def test_chain_and_medium(tmp_path):
    boxy = {"kind": "Boxy", "corner_0": [0, 0, 0], "corner_1": [10, 10, 10], "material": "white wall"}
    assert level(tmp_path, _scene([{"kind": "RotateY", "angle": 15, "object": boxy}]), "chain") == 1
    assert level(tmp_path, _scene([boxy]), "boxy") == 1
    smoke = {"kind": "ConstantMedium", "density": 0.1, "boundary": boxy,
             "texture": {"kind": "SolidColor", "color": [0.5, 0.5, 0.5]}}
    assert level(tmp_path, _scene([smoke]), "smoke") == 2
