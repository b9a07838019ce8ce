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

    python tests/golden/make_golden.py [name ...]     # names: box, prism, spheres, dense, batch

``batch_ref.npz`` holds the same kind of subset reference for four scenes of the
batched multi-scene workload (BATCH below).
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


# Scenes of the batched multi-scene workload (clovers_gb300.scenes.batch_scene(index)) with a golden
# reference over a stratified subset of their pixels: index -> subset stride.  Two without and two with
# constant-density media, of four material kinds.
BATCH = {3: 8, 23: 8, 31: 8, 40: 8}
BATCH_DEPTH = 16


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


def make_batch():
    """tests/golden/batch_ref.npz: per scene of BATCH its subset's pixel indices and means."""
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for k, stride in sorted(BATCH.items()):
            sc, w, h, _ = scenes.batch_scene(k, tmp)
            path = scenes.write_scene(sc, os.path.join(tmp, "batch_%02d.json" % k))
            o = oracle.Scene.from_json(path, w, h, precision=PRECISION)
            px = subset_pixels(w, h, stride)
            t0 = time.time()
            sub = o.render_pixels(w, h, SPP, BATCH_DEPTH, SEED, px) / SPP
            out["s%d_pixels" % k] = px
            out["s%d_mean" % k] = sub
            out["s%d_size" % k] = np.array([w, h])
            print("batch scene %d: %dx%d, %d pixels, %.1f s, mean %s" % (k, w, h, px.size, time.time() - t0,
                                                                        sub.mean(0)), flush=True)
    np.savez_compressed(os.path.join(HERE, "batch_ref.npz"), scenes=np.array(sorted(BATCH)), spp=SPP, seed=SEED,
                        depth=BATCH_DEPTH, precision=PRECISION, **out)


if __name__ == "__main__":
    for n in (sys.argv[1:] or list(WORKLOADS) + ["batch"]):
        make_batch() if n == "batch" else make(n)
