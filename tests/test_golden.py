"""Convergence against the committed golden crops (oracle, 65,536 spp, seed 1;
tests/golden/make_golden.py).

relMSE = mean over crop pixels and XYZ channels of (I - R)^2 / (R^2 + 1e-2).
For an unbiased estimator it falls as 1/spp; the bounds below allow 1.7x the
expected value at the stated spp (measured: box 64 spp 4.6e-3, 256 spp 1.2e-3,
1024 spp 2.9e-4 for the oracle with another seed).
"""

import os
import sys
import tempfile

import numpy as np
import pytest

import clovers_gb300 as cg
import oracle

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import make_golden  # noqa: E402

EPS = 1e-2
# workload -> (spp used by the check, relMSE bound)
BOUNDS_CPU = {"box": (64, 8e-3)}
BOUNDS_GPU = {"box": (256, 2e-3), "prism": (1024, None), "spheres": (256, None)}


def relmse(img, ref):
    return float(np.mean((img - ref) ** 2 / (ref ** 2 + EPS)))


def golden(name):
    path = os.path.join(HERE, "golden", "%s_ref.npz" % name)
    if not os.path.exists(path):
        pytest.skip("golden crop %s not generated" % name)
    return np.load(path)


@pytest.mark.parametrize("name", sorted(make_golden.WORKLOADS))
def test_golden_file_is_well_formed(name):
    g = golden(name)
    x0, r0, x1, r1 = [int(v) for v in g["window"]]
    assert g["mean"].shape == ((r1 - r0) * (x1 - x0), 3)
    assert np.all(np.isfinite(g["mean"])) and g["mean"].mean() > 0
    assert int(g["spp"]) == 65536


def test_oracle_converges_to_golden_box():
    g = golden("box")
    spp, bound = BOUNDS_CPU["box"]
    w, h = [int(v) for v in g["size"]]
    with tempfile.TemporaryDirectory() as tmp:
        o = oracle.Scene.from_json(make_golden.scene_file("box", tmp), w, h)
        img = o.render(w, h, spp, int(g["depth"]), 5, window=tuple(int(v) for v in g["window"])) / spp
    err = relmse(img, g["mean"])
    assert 1e-4 < err < bound


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["box", "prism", "spheres"])
def test_gpu_converges_to_golden(name):
    g = golden(name)
    spp, bound = BOUNDS_GPU[name]
    w, h = [int(v) for v in g["size"]]
    x0, r0, x1, r1 = [int(v) for v in g["window"]]
    with tempfile.TemporaryDirectory() as tmp:
        d = cg.Scene.from_json(make_golden.scene_file(name, tmp), w, h).upload()
    img = cg.draw(cg.GlobalOptions(quiet=True), cg.RenderOptions(width=w, height=h, samples=spp,
                                                                 max_depth=int(g["depth"]), seed=4242), d)
    crop = img.reshape(h, w, 3)[r0:r1, x0:x1].reshape(-1, 3).astype(np.float64)
    err = relmse(crop, g["mean"])
    print("%s: relMSE %.3g at %d spp" % (name, err, spp))
    if bound is None:  # no calibrated bound yet: the mean must still agree within 2 % on each channel
        assert np.all(np.abs(crop.mean(0) - g["mean"].mean(0)) <= 0.02 * g["mean"].mean(0) + 1e-4)
    else:
        assert err < bound
