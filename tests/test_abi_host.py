"""The C ABI library and its host-side logic (no GPU needed).

* every function declared in include/clovers_gpu.h is exported;
* scenes load on the host and the flattened BVH has the shape of the
  oracle's literal restatement of the reference's SAH build;
* errors are reported as status codes with a message, like the reference's
  panics / Result errors (render.rs:142-144, scenefile.rs:106-108).
"""

import ctypes
import json
import os
import re

import numpy as np
import pytest

import clovers_gb300 as cg
import oracle
from clovers_gb300 import _lib, scenes

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "clovers_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(clv_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) == set(_lib.SIGNATURES), "ctypes signatures out of sync with the header"
    assert b"sm_103a" in L.clv_version()


def test_box_scene_flattening(box_scene_path):
    s = cg.Scene.from_json(box_scene_path, 64, 64)
    info = s.info()
    assert info["objects"] == 9
    assert info["quads"] == 6 + 12 and info["spheres"] == 1
    o = oracle.Scene.from_json(box_scene_path, 64, 64)
    st = o.tree_stats()
    assert (info["nodes"], info["tree_depth"], info["mis_nodes"]) == (st["nodes"], st["tree_depth"], st["mis_nodes"])


def test_spheres_scene_flattening(spheres_scene_path):
    s = cg.Scene.from_json(spheres_scene_path, 40, 22)
    info = s.info()
    o = oracle.Scene.from_json(spheres_scene_path, 40, 22)
    assert info["objects"] == o.object_count() == 4 + 22 * 22
    st = o.tree_stats()
    assert (info["nodes"], info["tree_depth"], info["mis_nodes"]) == (st["nodes"], st["tree_depth"], st["mis_nodes"])


@pytest.mark.parametrize("n", [1, 2, 3, 1000, 20000])
def test_mesh_bvh_shape_matches_oracle(n):
    v, i = scenes.triangle_soup(n, seed=11)
    info = cg.Scene.from_mesh(v, i).info()
    st = oracle.Scene.from_mesh(v, i).tree_stats()
    assert (info["nodes"], info["tree_depth"]) == (st["nodes"], st["tree_depth"])


def test_degenerate_centroids_peel_chain():
    # identical centroids: find_best_split finds nothing and the builder peels one object per level
    tri = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    v = np.tile(tri, (40, 1))
    i = np.arange(120, dtype=np.uint32).reshape(40, 3)
    info = cg.Scene.from_mesh(v, i).info()
    st = oracle.Scene.from_mesh(v, i).tree_stats()
    assert (info["nodes"], info["tree_depth"]) == (st["nodes"], st["tree_depth"])
    assert info["tree_depth"] > 30


def _load_text(obj, w=16, h=16):
    return cg.Scene.from_json_text(json.dumps(obj), w, h)


def test_errors_are_status_codes(tmp_path):
    box = scenes.enclosed_box()
    with pytest.raises(cg.ClvError) as e:
        cg.Scene.from_json(str(tmp_path / "missing.json"), 8, 8)
    assert e.value.code == _lib.CLV_E_SCENE
    with pytest.raises(cg.ClvError) as e:
        cg.Scene.from_json_text("{ not json", 8, 8)
    assert e.value.code == _lib.CLV_E_SCENE and "JSON" in str(e.value)
    no_prio = json.loads(json.dumps(box))
    for o in no_prio["objects"]:
        o.pop("priority", None)
    with pytest.raises(cg.ClvError, match="priority"):
        _load_text(no_prio)
    assert cg.Scene.from_json_text(json.dumps(box), 8, 8, bvh="lam").info()["nodes"] > 0  # BvhAlgorithm::Lam
    with pytest.raises(ValueError):
        cg.Scene.from_json_text(json.dumps(box), 8, 8, bvh="median")
    bad_kind = json.loads(json.dumps(box))
    bad_kind["objects"][0]["kind"] = "Torus"
    with pytest.raises(cg.ClvError, match="Torus"):
        _load_text(bad_kind)
    prio_box = json.loads(json.dumps(box))
    prio_box["objects"][6]["priority"] = True  # Translate has no random(): the reference panics
    with pytest.raises(cg.ClvError, match="random"):
        _load_text(prio_box)


def test_unknown_material_name_falls_back_to_default():
    box = scenes.enclosed_box()
    box["objects"][0]["material"] = "no such material"
    info = _load_text(box).info()
    assert info["objects"] == 9


def test_png_and_exr_encoders(tmp_path):
    import struct
    import zlib
    from clovers_gb300 import imageio
    rgb = (np.arange(4 * 3 * 3) % 256).astype(np.uint8).reshape(12, 3)
    data = imageio.png_bytes(rgb, 4, 3, [("Software", "clovers")])
    assert data[:8] == b"\x89PNG\r\n\x1a\n"
    # decode IDAT and compare
    pos, idat = 8, b""
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        tag = data[pos + 4:pos + 8]
        if tag == b"IDAT":
            idat += data[pos + 8:pos + 8 + n]
        pos += 12 + n
    raw = np.frombuffer(zlib.decompress(idat), np.uint8).reshape(3, 13)
    assert np.array_equal(raw[:, 1:].reshape(12, 3), rgb)
    xyz = np.random.default_rng(0).random((12, 3)).astype(np.float32)
    ex = imageio.exr_bytes(xyz, 4, 3)
    assert ex[:4] == b"\x76\x2f\x31\x01" and b"chromaticities" in ex
    # last scanline holds B, G, R planes of the last image row
    last = np.frombuffer(ex[-4 * 12:], "<f4").reshape(3, 4)
    assert np.array_equal(last[2], xyz.reshape(3, 4, 3)[2, :, 0])


def test_png_metadata_as_the_reference_writes_it(tmp_path):
    """write.rs:54-73: a Comment tEXt chunk (scene, mode in its Rust name,
    resolution, samples and depth for path tracing, the duration in humantime's
    format, the thread count) followed by Software = clovers."""
    import struct
    import clovers_gb300 as cg
    from clovers_gb300 import imageio
    assert imageio.format_duration(0) == "0s"
    assert imageio.format_duration(1.23456789) == "1s 234ms 567us 890ns"
    assert imageio.format_duration(9420.001) == "2h 37m 1ms"
    assert imageio.format_duration(90061) == "1day 1h 1m 1s"
    assert imageio.format_duration(2 * 86400 + 0.5) == "2days 500ms"
    opts = cg.RenderOptions(input="scenes/cornell.json", width=4, height=3, samples=16, max_depth=8)
    path = str(tmp_path / "x.png")
    imageio.write_png(path, np.zeros((12, 3), np.uint8), 4, 3, opts, duration_s=1.5)
    data = open(path, "rb").read()
    texts, pos = [], 8
    while pos < len(data):
        n = struct.unpack(">I", data[pos:pos + 4])[0]
        if data[pos + 4:pos + 8] == b"tEXt":
            texts.append(data[pos + 8:pos + 8 + n].decode("latin-1"))
        pos += 12 + n
    import os
    assert texts == ["Comment\0Rendered with the clovers path tracing engine. Scene file scenes/cornell.json rendered "
                     "using the PathTracing rendering mode at 4x3 resolution, 16 samples per pixel, 8 max ray bounce "
                     "depth. Rendering finished in 1s 500ms, using %d threads." % (os.cpu_count() or 1),
                     "Software\0clovers"]
