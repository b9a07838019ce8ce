import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def box_scene_path(tmp_path_factory):
    from clovers_gb300 import scenes
    return scenes.write_scene(scenes.enclosed_box(), str(tmp_path_factory.mktemp("scenes") / "box.json"))


@pytest.fixture(scope="session")
def spheres_scene_path(tmp_path_factory):
    from clovers_gb300 import scenes
    return scenes.write_scene(scenes.random_spheres(1), str(tmp_path_factory.mktemp("scenes") / "spheres.json"))
