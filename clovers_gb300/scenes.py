"""Seeded synthetic workloads in the reference's own input formats.

* :func:`enclosed_box` -- a 555-unit box scene in the layout of the
  reference's ``scenes/cornell.json``: five diffuse walls (sRGB-encoded white
  0.73, red 0.65/0.05/0.05, green 0.12/0.45/0.15), a 130x105 area light of
  radiance XYZ(E) 15, two rotated boxes and an r=90 glass sphere.
* :func:`random_spheres` -- the random-sphere scene of the reference's
  ``scenes/one_weekend.js`` generator (ground sphere, 3 large spheres, a 22x22
  grid of r=0.2 spheres, 80/15/5 % Lambertian/metal/glass), static spheres.
* :func:`triangle_soup` / :func:`random_rays` -- independent random
  triangles in the unit cube and random rays, for closest-hit ray casts.
"""

import json

import numpy as np

CORNELL_CAMERA = {"look_from": [278, 278, -800], "look_at": [278, 278, 0], "up": [0, 1, 0], "vertical_fov": 40,
                  "aperture": 0, "focus_distance": 10}


def enclosed_box():
    """Scene dict of the enclosed-box workload (the 512x512, 256 spp, depth 16 render)."""
    quad = lambda q, u, v, m: {"kind": "Quad", "q": q, "u": u, "v": v, "material": m}
    objects = [
        quad([555, 0, 0], [0, 0, 555], [0, 555, 0], "green wall"),
        quad([0, 0, 555], [0, 0, -555], [0, 555, 0], "red wall"),
        quad([0, 0, 0], [555, 0, 0], [0, 0, 555], "white wall"),
        quad([0, 555, 0], [555, 0, 0], [0, 0, 555], "white wall"),
        quad([0, 0, 555], [555, 0, 0], [0, 555, 0], "white wall"),
        dict(quad([213, 554, 227], [130, 0, 0], [0, 0, 105], "lamp"), priority=True),
        {"kind": "Translate", "offset": [265, 0, 295],
         "object": {"kind": "RotateY", "angle": 15,
                    "object": {"kind": "Boxy", "corner_0": [0, 0, 0], "corner_1": [165, 330, 165],
                               "material": "white wall"}}},
        {"kind": "Translate", "offset": [130, 0, 65],
         "object": {"kind": "RotateY", "angle": -18,
                    "object": {"kind": "Boxy", "corner_0": [0, 0, 0], "corner_1": [165, 165, 165],
                               "material": "white wall"}}},
        {"kind": "Sphere", "priority": True, "center": [420, 90, 130], "radius": 90, "material": "glass"},
    ]
    materials = [
        {"name": "glass", "kind": "Dielectric", "refractive_index": 1.5, "color": [1, 1, 1]},
        {"name": "lamp", "kind": "DiffuseLight", "emit": {"kind": "SolidColor", "color": {"xyz_e": [15, 15, 15]}}},
        {"name": "green wall", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.12, 0.45, 0.15]}},
        {"name": "red wall", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.65, 0.05, 0.05]}},
        {"name": "white wall", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.73, 0.73, 0.73]}},
    ]
    return {"time_0": 0, "time_1": 1, "camera": CORNELL_CAMERA, "background_color": [0, 0, 0],
            "objects": objects, "materials": materials}


def random_spheres(seed=1):
    """Scene dict of the random-sphere workload (400x225, 64 spp, depth 50)."""
    rng = np.random.default_rng(seed)
    objects = [
        {"kind": "Sphere", "center": [0.0, -1000.0, 0.0], "radius": 1000.0, "material": "ground"},
        {"kind": "Sphere", "center": [0.0, 1.0, 0.0], "radius": 1.0, "material": "glass", "priority": True},
        {"kind": "Sphere", "center": [-4.0, 1.0, 0.0], "radius": 1.0, "material": "big diffuse"},
        {"kind": "Sphere", "center": [4.0, 1.0, 0.0], "radius": 1.0, "material": "big metal"},
    ]
    materials = [
        {"name": "ground", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.5, 0.5, 0.5]}},
        {"name": "glass", "kind": "Dielectric", "refractive_index": 1.5},
        {"name": "big diffuse", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.4, 0.2, 0.1]}},
        {"name": "big metal", "kind": "Metal", "albedo": {"kind": "SolidColor", "color": [0.7, 0.6, 0.5]},
         "fuzz": 0.0},
    ]
    for a in range(-11, 11):
        for b in range(-11, 11):
            choose = float(rng.random())
            center = [a + 0.9 * float(rng.random()), 0.2, b + 0.9 * float(rng.random())]
            name = "sphere %d_%d" % (a, b)
            if choose < 0.8:
                c = rng.random(3) * rng.random(3)
                materials.append({"name": name, "kind": "Lambertian",
                                  "albedo": {"kind": "SolidColor", "color": [float(x) for x in c]}})
            elif choose < 0.95:
                c = rng.random(3)
                materials.append({"name": name, "kind": "Metal",
                                  "albedo": {"kind": "SolidColor", "color": [float(x) for x in c]},
                                  "fuzz": float(rng.random() * 0.5)})
            else:
                name = "glass"
            objects.append({"kind": "Sphere", "center": center, "radius": 0.2, "material": name})
    camera = {"look_from": [13.0, 2.0, 3.0], "look_at": [0.0, 0.0, 0.0], "up": [0.0, 1.0, 0.0],
              "vertical_fov": 25.0, "aperture": 0.0, "focus_distance": 10.0}
    return {"time_0": 0, "time_1": 1, "camera": camera, "background_color": [0.7, 0.7, 0.9],
            "objects": objects, "materials": materials}


def write_scene(scene, path):
    with open(path, "w") as f:
        json.dump(scene, f)
    return path


def _unit_vectors(rng, n):
    v = rng.normal(size=(n, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v


def triangle_soup(n, seed=2):
    """n independent triangles: a ~ U[0,1]^3, b = a + e1, c = a + e2, |e_i| ~ U[0.001, 0.05].

    Returns (vertices (3n, 3) float32, indices (n, 3) uint32)."""
    rng = np.random.default_rng(seed)
    a = rng.random((n, 3))
    e1 = _unit_vectors(rng, n) * rng.uniform(0.001, 0.05, (n, 1))
    e2 = _unit_vectors(rng, n) * rng.uniform(0.001, 0.05, (n, 1))
    v = np.stack([a, a + e1, a + e2], axis=1).reshape(-1, 3).astype(np.float32)
    idx = np.arange(3 * n, dtype=np.uint32).reshape(n, 3)
    return v, idx


def random_rays(n, seed=3, tmin=0.001, tmax=3.4028234663852886e38):
    """n rays {ox,oy,oz,tmin,dx,dy,dz,tmax}: origins U[0,1]^3, directions uniform on the sphere."""
    rng = np.random.default_rng(seed)
    r = np.empty((n, 8), np.float32)
    r[:, 0:3] = rng.random((n, 3))
    d = _unit_vectors(rng, n).astype(np.float32)
    d /= np.sqrt((d.astype(np.float32) ** 2).sum(axis=1, keepdims=True)).astype(np.float32)
    r[:, 4:7] = d
    r[:, 3] = tmin
    r[:, 7] = np.float32(tmax)
    return r


def camera_rays(width, height, camera_fn):
    """Pinhole rays through pixel corners via camera_fn(pu, pv) -> (o3, d3)."""
    out = np.empty((width * height, 8), np.float32)
    k = 0
    for row in range(height):
        y = height - 1 - row
        for x in range(width):
            o = camera_fn(x / width, y / height)
            out[k, 0:3] = o[0:3]
            out[k, 4:7] = o[3:6]
            out[k, 3] = 0.001
            out[k, 7] = 3.4028234663852886e38
            k += 1
    return out


def write_binary_stl(path, triangles):
    """Binary STL of triangles (n, 3, 3) float32 (normals written as zero)."""
    import struct
    tris = np.asarray(triangles, np.float32).reshape(-1, 3, 3)
    with open(path, "wb") as f:
        f.write(b"\0" * 80 + struct.pack("<I", tris.shape[0]))
        rec = np.zeros((tris.shape[0], 50), np.uint8)
        body = np.concatenate([np.zeros((tris.shape[0], 3), np.float32), tris.reshape(-1, 9)], axis=1)
        rec[:, :48] = body.view(np.uint8).reshape(-1, 48)
        f.write(rec.tobytes())
    return path


def prism_triangles():
    """A triangular prism as 8 triangles (2 end caps, 3 rectangular sides split in two)."""
    a = np.array([[0, 0, 0], [1, 0, 0], [0.5, 0.866, 0]], np.float32)
    b = a + np.array([0, 0, 1], np.float32)
    tris = [a, b[::-1]]
    for i in range(3):
        j = (i + 1) % 3
        tris += [np.stack([a[i], a[j], b[j]]), np.stack([a[i], b[j], b[i]])]
    return np.stack(tris)


def kitchen_sink(stl_path):
    """Every object, material and texture kind on the render path in one small scene."""
    objects = [
        {"kind": "Quad", "q": [-10, 0, -10], "u": [20, 0, 0], "v": [0, 0, 20], "material": "surface checker floor"},
        {"kind": "Quad", "q": [-10, 0, -6], "u": [20, 0, 0], "v": [0, 10, 0], "material": "spatial checker wall"},
        {"kind": "Quad", "priority": True, "q": [-2, 7.99, -2], "u": [4, 0, 0], "v": [0, 0, 4], "material": "lamp d65"},
        {"kind": "Sphere", "priority": True, "center": [4, 6, -1], "radius": 0.5, "material": "cone lamp"},
        {"kind": "Triangle", "priority": True, "q": [-6, 5, 3], "u": [1.5, 0, 0], "v": [0, 1.5, 0],
         "material": {"kind": "DiffuseLight", "emit": {"kind": "IlluminantLedB3", "intensity": 3.0}}},
        {"kind": "Sphere", "center": [-3, 1, 0], "radius": 1, "material": "thin film"},
        {"kind": "Sphere", "center": [0, 1, -2], "radius": 1, "material": "cauchy glass"},
        {"kind": "Sphere", "center": [3, 1, 1], "radius": 1, "material": "sellmeier glass"},
        {"kind": "Sphere", "center": [0, 0.6, 2.5], "radius": 0.6, "material": "fuzzy metal"},
        {"kind": "MovingSphere", "center_0": [-1.5, 0.4, 3], "center_1": [-1.5, 0.9, 3], "radius": 0.4,
         "material": "tinted glass"},
        {"kind": "Translate", "offset": [1.5, 0, -4],
         "object": {"kind": "RotateY", "angle": 30,
                    "object": {"kind": "Boxy", "corner_0": [0, 0, 0], "corner_1": [1, 2, 1], "material": "lambert"}}},
        {"kind": "ConstantMedium", "density": 0.6,
         "boundary": {"kind": "Boxy", "corner_0": [-5, 0, -4], "corner_1": [-3.5, 1.5, -2.5]},
         "texture": {"kind": "SolidColor", "color": [0.9, 0.9, 0.7]}},
        {"kind": "ConstantMedium", "density": 0.3,
         "boundary": {"kind": "Sphere", "center": [5, 1, -3], "radius": 0.9},
         "texture": {"kind": "IlluminantD50", "intensity": 0.8}},
        {"kind": "Translate", "offset": [0, 3, 4],
         "object": {"kind": "ObjectList", "objects": [
             {"kind": "Quad", "q": [-1, 0, 0], "u": [1, 0, 0], "v": [0, 1, 0], "material": "lambert"},
             {"kind": "Quad", "q": [0, 0, 0], "u": [1, 0, 0], "v": [0, 1, 0], "material": "lambert"}]}},
        {"kind": "ObjectList", "objects": [
            {"kind": "Sphere", "center": [-4, 3, -4], "radius": 0.3, "material": "lambert"},
            {"kind": "Triangle", "q": [2, 3, -5], "u": [1, 0, 0], "v": [0, 1, 0], "material": "lambert"}]},
        {"kind": "STL", "path": stl_path, "center": [-1, 2.5, -4], "scale": 1.2, "rotation": [0, 20, -30],
         "material": "sellmeier glass"},
    ]
    materials = [
        {"name": "surface checker floor", "kind": "Lambertian",
         "albedo": {"kind": "SurfaceChecker", "even": [0.8, 0.8, 0.8], "odd": {"hex": "#335577"}, "density": 8}},
        {"name": "spatial checker wall", "kind": "Lambertian",
         "albedo": {"kind": "SpatialChecker", "even": {"srgb": [0.9, 0.4, 0.2]}, "odd": {"lin_srgb": [0.1, 0.2, 0.6]},
                    "density": 2}},
        {"name": "lamp d65", "kind": "DiffuseLight", "emit": {"kind": "IlluminantD65", "intensity": 4.0}},
        {"name": "cone lamp", "kind": "ConeLight", "spread": 40.0,
         "emit": {"kind": "SolidColor", "color": {"xyz_e": [30, 25, 20]}}},
        {"name": "thin film", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.7, 0.7, 0.7]},
         "thin_film": {"refractive_index": 1.33, "thickness": 420.0}},
        {"name": "cauchy glass", "kind": "Dispersive", "cauchy_a": 1.728, "cauchy_b": 0.01342},
        {"name": "sellmeier glass", "kind": "Dispersive", "sellmeier_b": [1.0396, 0.2318, 1.0105],
         "sellmeier_c": [0.0060, 0.0200, 103.56]},
        {"name": "fuzzy metal", "kind": "Metal", "albedo": {"kind": "SolidColor", "color": {"xyz_d65": [0.6, 0.6, 0.5]}},
         "fuzz": 0.3},
        {"name": "tinted glass", "kind": "Dielectric", "refractive_index": 1.45, "color": [0.9, 1.0, 0.8]},
        {"name": "lambert", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.5, 0.6, 0.4]}},
    ]
    camera = {"look_from": [0.0, 4.0, 14.0], "look_at": [0.0, 1.5, 0.0], "up": [0.0, 1.0, 0.0],
              "vertical_fov": 40.0, "aperture": 0.1, "focus_distance": 13.0}
    return {"time_0": 0, "time_1": 1, "camera": camera, "background_color": [0.05, 0.06, 0.1],
            "objects": objects, "materials": materials}
