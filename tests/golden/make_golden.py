"""Regenerates the golden references in this directory.

Each file holds the oracle's mean XYZ(E), rendered in double precision (the
oracle's f64 build: the reference's algorithm with Float = f64) at 65,536
samples per pixel with seed 1, over two pixel sets of a workload image:

* ``mean``: a 64x64 crop (``window`` = x0, r0, x1, r1 in buffer coordinates);
* ``sub_mean``: a stratified subset of the whole image, the centre pixel of
  every ``stride`` x ``stride`` cell (``sub_pixels`` = buffer indices
  r * width + x).

These are the converged references that GPU renders are measured against
(relMSE, GPU time to relMSE <= 1e-3).  GPU renders use other seeds.

    python tests/golden/make_golden.py [name ...]     # names: box, prism, spheres, dense
"""

import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import oracle  # noqa: E402
from clovers_gb300 import scenes  # noqa: E402

SPP = 65536
SEED = 1
PRECISION = "f64"
# name -> (scene builder, width, height, max depth, crop window (x0, r0, x1, r1), subset stride)
WORKLOADS = {
    "box": ("enclosed_box", 512, 512, 16, (224, 192, 288, 256), 16),
    "prism": ("dispersive_prism", 1024, 1024, 16, (408, 568, 472, 632), 16),
    "spheres": ("random_spheres", 400, 225, 50, (168, 80, 232, 144), 16),
    "dense": ("dense_mesh_scene", 1920, 1080, 12, (928, 508, 992, 572), 32),
}


def scene_file(name, tmp):
    builder = WORKLOADS[name][0]
    if builder == "dispersive_prism":
        stl = scenes.write_binary_stl(os.path.join(tmp, "prism.stl"), scenes.prism_triangles())
        sc = scenes.dispersive_prism(stl)
    elif builder == "dense_mesh_scene":
        stl = scenes.write_binary_stl(os.path.join(tmp, "ico.stl"), scenes.displaced_icosphere(209))
        sc = scenes.dense_mesh_scene(stl)
    elif builder == "random_spheres":
        sc = scenes.random_spheres(1)
    else:
        sc = getattr(scenes, builder)()
    return scenes.write_scene(sc, os.path.join(tmp, name + ".json"))


def subset_pixels(width, height, stride):
    """Buffer indices of the centre pixel of every stride x stride cell of the image."""
    xs = np.arange(stride // 2, width, stride)
    rs = np.arange(stride // 2, height, stride)
    return (rs[:, None] * width + xs[None, :]).reshape(-1).astype(np.uint32)


def make(name):
    _, w, h, depth, win, stride = WORKLOADS[name]
    px = subset_pixels(w, h, stride)
    with tempfile.TemporaryDirectory() as tmp:
        o = oracle.Scene.from_json(scene_file(name, tmp), w, h, precision=PRECISION)
        t0 = time.time()
        crop = o.render(w, h, SPP, depth, SEED, window=win) / SPP
        sub = o.render_pixels(w, h, SPP, depth, SEED, px) / SPP
        el = time.time() - t0
    out = os.path.join(HERE, "%s_ref.npz" % name)
    np.savez_compressed(out, mean=crop, window=np.array(win), sub_mean=sub, sub_pixels=px, sub_stride=stride,
                        size=np.array([w, h]), spp=SPP, seed=SEED, depth=depth, builder=WORKLOADS[name][0],
                        precision=PRECISION)
    print("%s: %.1f s on %d threads, crop mean %s, subset mean %s -> %s" % (
        name, el, os.cpu_count(), crop.mean(0), sub.mean(0), out), flush=True)


if __name__ == "__main__":
    for n in (sys.argv[1:] or list(WORKLOADS)):
        make(n)
