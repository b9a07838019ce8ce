"""Regenerates the golden reference crops in this directory.

Each file holds the oracle's (CPU restatement of the reference) mean XYZ(E)
over a 64x64 crop of a workload image, rendered at 65,536 samples per pixel
with seed 1: the converged reference that GPU renders are measured against
(relMSE, time to relMSE <= 1e-3).  GPU renders use other seeds.

    python tests/golden/make_golden.py [name ...]     # names: box, prism, spheres
"""

import json
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
# name -> (scene builder, width, height, max depth, crop window (x0, r0, x1, r1) in buffer coordinates)
WORKLOADS = {
    "box": ("enclosed_box", 512, 512, 16, (224, 192, 288, 256)),
    "prism": ("dispersive_prism", 1024, 1024, 16, (408, 568, 472, 632)),
    "spheres": ("random_spheres", 400, 225, 50, (168, 80, 232, 144)),
}


def scene_file(name, tmp):
    builder = WORKLOADS[name][0]
    if builder == "dispersive_prism":
        stl = scenes.write_binary_stl(os.path.join(tmp, "prism.stl"), scenes.prism_triangles())
        sc = scenes.dispersive_prism(stl)
    elif builder == "random_spheres":
        sc = scenes.random_spheres(1)
    else:
        sc = getattr(scenes, builder)()
    return scenes.write_scene(sc, os.path.join(tmp, name + ".json"))


def make(name):
    _, w, h, depth, win = WORKLOADS[name]
    with tempfile.TemporaryDirectory() as tmp:
        o = oracle.Scene.from_json(scene_file(name, tmp), w, h)
        t0 = time.time()
        total = o.render(w, h, SPP, depth, SEED, window=win)
        el = time.time() - t0
    mean = total / SPP
    out = os.path.join(HERE, "%s_ref.npz" % name)
    np.savez_compressed(out, mean=mean, window=np.array(win), size=np.array([w, h]), spp=SPP, seed=SEED,
                        depth=depth, builder=WORKLOADS[name][0])
    print("%s: %.1f s on %d threads, mean %s -> %s" % (name, el, os.cpu_count(), mean.mean(0), out), flush=True)


if __name__ == "__main__":
    for n in (sys.argv[1:] or list(WORKLOADS)):
        make(n)
