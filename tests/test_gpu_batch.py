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
    # a batch with a watertight scene runs the variants that choose the triangle test per scene
    path = scenes.write_scene(specs[2][0], str(tmp_path / "wt.json"))
    wt = cg.Scene.from_json(path, 40, 30).set_watertight().upload()
    wt_opts = cg.RenderOptions(width=40, height=30, samples=16, max_depth=10, seed=9)
    batched = cg.draw_batch(dev + [wt], opts + [wt_opts])
    for d, o, img in zip(dev + [wt], opts + [wt_opts], batched):
        single = cg.draw(cg.GlobalOptions(quiet=True), o, d)
        np.testing.assert_allclose(img, single, rtol=1e-6, atol=1e-9)
        assert d.status() == 0


def test_guided_batch_matches_guided_single_renders(tmp_path):
    """clv_render_batch_guided with one guide for every scene gives each scene the film that
    clv_render_guided gives it alone with the same guide (same random streams; each query's network
    output depends only on its own inputs, normalised to its own scene's box)."""
    specs = [(scenes.enclosed_box(), 40, 32, 16, 10, 7), (scenes.random_spheres(1), 48, 27, 8, 12, 8)]
    dev, opts = [], []
    for k, (sc, w, h, spp, depth, seed) in enumerate(specs):
        path = scenes.write_scene(sc, str(tmp_path / ("g%d.json" % k)))
        dev.append(cg.Scene.from_json(path, w, h).upload())
        opts.append(cg.RenderOptions(width=w, height=h, samples=spp, max_depth=depth, seed=seed))
    guide = cg.Guide(seed=5)
    for alpha in (0.0, 0.5):
        batched = cg.draw_batch(dev, opts, guide=guide, alpha=alpha)
        for d, o, img in zip(dev, opts, batched):
            film = cg.DeviceBuffer(o.width * o.height * 24).zero()
            cg.render_guided(d, o, guide, alpha, film)
            single = film.to_numpy(np.float64, (o.width * o.height, 3)) / o.samples
            np.testing.assert_allclose(img, single, rtol=1e-6, atol=1e-9)
            assert d.status() == 0
    assert guide.status() == 0


def test_batch_larger_than_one_wavefront(tmp_path):
    """A batch of more than 128 scenes (the size of the constant-memory scene tables) renders as
    consecutive wavefronts; every scene still gets its own render's film."""
    specs = [scenes.enclosed_box(), scenes.random_spheres(1), scenes.batch_scene(1, str(tmp_path))[0]]
    dev = []
    for k, sc in enumerate(specs):
        path = scenes.write_scene(sc, str(tmp_path / ("m%d.json" % k)))
        dev.append(cg.Scene.from_json(path, 16, 12).upload())
    ds, opts = [], []
    for k in range(131):
        ds.append(dev[k % 3])
        opts.append(cg.RenderOptions(width=16, height=12, samples=1 + k % 3, max_depth=4 + k % 5, seed=100 + k))
    batched = cg.draw_batch(ds, opts)
    assert len(batched) == 131
    for k in (0, 1, 2, 64, 127, 128, 129, 130):
        single = cg.draw(cg.GlobalOptions(quiet=True), opts[k], ds[k])
        np.testing.assert_allclose(batched[k], single, rtol=1e-6, atol=1e-9)
    assert all(d.status() == 0 for d in dev)
