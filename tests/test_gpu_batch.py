"""Multi-scene wavefront (clv_render_batch): rendering several scenes of
different sizes, sample counts and depths in one wavefront gives each scene
the film that its own render gives (same random streams; only the order of
the f64 film additions differs, relative tolerance 1e-9)."""

import numpy as np
import pytest

import clovers_gb300 as cg
from clovers_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_batch_matches_individual_renders(tmp_path):
    stl = scenes.write_binary_stl(str(tmp_path / "prism.stl"), scenes.prism_triangles())
    specs = [(scenes.enclosed_box(), 48, 40, 16, 12, 3),
             (scenes.random_spheres(1), 64, 36, 8, 50, 4),
             (scenes.kitchen_sink(stl), 40, 30, 24, 10, 5)]
    dev, opts = [], []
    for k, (sc, w, h, spp, depth, seed) in enumerate(specs):
        path = scenes.write_scene(sc, str(tmp_path / ("s%d.json" % k)))
        dev.append(cg.Scene.from_json(path, w, h).upload())
        opts.append(cg.RenderOptions(width=w, height=h, samples=spp, max_depth=depth, seed=seed))
    batched = cg.draw_batch(dev, opts)
    for d, o, img in zip(dev, opts, batched):
        single = cg.draw(cg.GlobalOptions(quiet=True), o, d)
        np.testing.assert_allclose(img, single, rtol=1e-6, atol=1e-9)
        assert d.status() == 0
