"""The oracle's debug render modes (clovers-cli/src/draw_cpu.rs:148-207) on
known answers, without a GPU:

* normal map (normals.rs:11-37): the enclosed box's back wall faces the
  camera, so its face normal is (0, 0, -1); after the x/z flip that is
  (0, 0, 1), colour (0.5, 0.5, 1.0) exactly;
* BVH and primitive test counts (debug_visualizations.rs:18-35): every pixel
  is a grey level k / 255 or one of the ramp's colours for larger counts, and
  every ray enters the root node.
The GPU's debug images are compared with these in tests/test_gpu_render.py."""

import numpy as np
import pytest

import oracle
from clovers_gb300 import scenes


@pytest.fixture(scope="module")
def box(tmp_path_factory):
    path = scenes.write_scene(scenes.enclosed_box(), str(tmp_path_factory.mktemp("dbg") / "box.json"))
    return oracle.Scene.from_json(path, 64, 64)


def test_normal_map_back_wall(box):
    img = box.render_debug(64, 64, 1, seed=3)
    assert np.all((img >= 0) & (img <= 1))
    back = np.all(img == np.array([0.5, 0.5, 1.0], np.float32), axis=1)
    assert back.mean() > 0.1  # a good part of the view is the back wall


@pytest.mark.parametrize("mode", [2, 3])
def test_count_modes_are_ramp_values(box, mode):
    img = box.render_debug(64, 64, mode, seed=3)
    grey = (img[:, 0] == img[:, 1]) & (img[:, 1] == img[:, 2])
    k = np.round(img[:, 0] * 255.0)
    assert np.all(~grey | (np.abs(img[:, 0] - (k / 255.0).astype(np.float32)) == 0))
    ramp = np.array([[1.0, 1.0, 0.0], [1.0, 0.5, 0.0], [1.0, 0.0, 0.0]], np.float32)
    others = img[~grey]
    assert all(any(np.array_equal(p, r) for r in ramp) for p in others)
    nodes = np.round(box.render_debug(64, 64, 2, seed=3)[:, 0] * 255.0)
    assert np.all(nodes >= 1)  # every ray enters the root


def test_bad_mode_is_refused(box):
    with pytest.raises(RuntimeError):
        box.render_debug(8, 8, 4, seed=1)
