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


def write_ply(path, vertices, faces, fmt="binary_little_endian", coord_type="float", index_type="int",
              extra_vertex_props=0):
    """PLY mesh in the layout of the reference's ply/ files: vertex x, y, z (+ extra
    float properties, written as zero), face list uchar <index_type> vertex_indices.
    fmt: ascii, binary_little_endian or binary_big_endian."""
    v = np.asarray(vertices, np.float64).reshape(-1, 3)
    f = np.asarray(faces, np.int64).reshape(-1, 3)
    ctype = {"float": "f4", "double": "f8", "int": "i4", "uint": "u4"}[coord_type]
    itype = {"int": "i4", "uint": "u4", "short": "i2", "ushort": "u2", "uchar": "u1"}[index_type]
    head = ["ply", "format %s 1.0" % fmt, "comment clovers_gb300 test mesh", "element vertex %d" % len(v)]
    head += ["property %s %s" % (coord_type, c) for c in "xyz"]
    head += ["property float extra%d" % k for k in range(extra_vertex_props)]
    head += ["element face %d" % len(f), "property list uchar %s vertex_indices" % index_type, "end_header"]
    with open(path, "wb") as out:
        out.write(("\n".join(head) + "\n").encode())
        if fmt == "ascii":
            lines = []
            for row in v:
                vals = [repr(float(np.float32(x))) if coord_type == "float" else
                        (repr(float(x)) if coord_type == "double" else str(int(x))) for x in row]
                lines.append(" ".join(vals + ["0"] * extra_vertex_props))
            lines += ["3 %d %d %d" % tuple(r) for r in f]
            out.write(("\n".join(lines) + "\n").encode())
            return path
        e = "<" if fmt == "binary_little_endian" else ">"
        vt = np.dtype([(c, e + ctype) for c in "xyz"] + [("extra%d" % k, e + "f4") for k in range(extra_vertex_props)])
        va = np.zeros(len(v), vt)
        for k, c in enumerate("xyz"):
            va[c] = v[:, k]
        out.write(va.tobytes())
        ft = np.dtype([("n", "u1"), ("i", e + itype, (3,))])
        fa = np.zeros(len(f), ft)
        fa["n"] = 3
        fa["i"] = f
        out.write(fa.tobytes())
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


def dispersive_prism(stl_path):
    """Dispersive-caustics workload: a Sellmeier-glass triangular prism (8 triangles), an r=0.3 glass
    sphere, two 0.2x0.2 lights of radiance XYZ(E) 50 and a grey 0.5 floor (1024x1024, up to 4096 spp)."""
    glass = {"name": "sellmeier glass", "kind": "Dispersive", "sellmeier_b": [1.0396, 0.2318, 1.0105],
             "sellmeier_c": [0.0060, 0.0200, 103.56]}
    lamp = {"name": "lamp", "kind": "DiffuseLight", "emit": {"kind": "SolidColor", "color": {"xyz_e": [50, 50, 50]}}}
    floor = {"name": "floor", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.5, 0.5, 0.5]}}
    objects = [
        {"kind": "Quad", "q": [-5, 0, -5], "u": [10, 0, 0], "v": [0, 0, 10], "material": "floor"},
        {"kind": "STL", "path": stl_path, "center": [-0.35, 0.35, -0.25], "scale": 0.7, "rotation": [90, 0, 15],
         "material": "sellmeier glass", "priority": True},
        {"kind": "Sphere", "priority": True, "center": [0.75, 0.3, 0.1], "radius": 0.3, "material": "sellmeier glass"},
        {"kind": "Quad", "priority": True, "q": [-0.6, 2.0, -0.1], "u": [0.2, 0, 0], "v": [0, 0, 0.2],
         "material": "lamp"},
        {"kind": "Quad", "priority": True, "q": [0.9, 1.6, 0.5], "u": [0.2, 0, 0], "v": [0, 0, 0.2], "material": "lamp"},
    ]
    camera = {"look_from": [0.0, 2.2, 3.2], "look_at": [0.1, 0.2, 0.0], "up": [0.0, 1.0, 0.0],
              "vertical_fov": 40.0, "aperture": 0.0, "focus_distance": 3.5}
    return {"time_0": 0, "time_1": 1, "camera": camera, "background_color": [0, 0, 0],
            "objects": objects, "materials": [glass, lamp, floor]}


def _hash_noise(p, seed):
    """Value noise in [-1, 1] on the integer lattice, trilinearly interpolated with smoothstep weights."""
    i = np.floor(p).astype(np.int64)
    f = p - i
    w = f * f * (3.0 - 2.0 * f)

    def h(ix, iy, iz):
        x = (ix * 73856093) ^ (iy * 19349663) ^ (iz * 83492791) ^ (seed * 2654435761)
        x = (x ^ (x >> 13)) * 1274126177
        x = x ^ (x >> 16)
        return (x & 0xFFFF).astype(np.float64) / 32767.5 - 1.0

    out = 0.0
    for dx in (0, 1):
        for dy in (0, 1):
            for dz in (0, 1):
                wx = w[:, 0] if dx else 1 - w[:, 0]
                wy = w[:, 1] if dy else 1 - w[:, 1]
                wz = w[:, 2] if dz else 1 - w[:, 2]
                out = out + wx * wy * wz * h(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz)
    return out


def fbm(p, seed, octaves=5):
    total, amp, freq = 0.0, 0.5, 2.0
    for _ in range(octaves):
        total = total + amp * _hash_noise(p * freq, seed)
        amp *= 0.5
        freq *= 2.0
    return total


def displaced_icosphere(frequency, seed=3, amplitude=0.15):
    """Geodesic sphere: each icosahedron face split into frequency^2 triangles (20 f^2 in total),
    vertices pushed radially by amplitude * fbm(p).  Returns triangles (n, 3, 3) float32."""
    t = (1.0 + 5 ** 0.5) / 2.0
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
                  [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], np.float64)
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    F = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6],
         [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10],
         [8, 6, 7], [9, 8, 1]]
    n = frequency
    ii, jj = np.meshgrid(np.arange(n + 1), np.arange(n + 1), indexing="ij")
    mask = ii + jj <= n
    bi, bj = ii[mask], jj[mask]
    index = -np.ones((n + 1, n + 1), np.int64)
    index[bi, bj] = np.arange(bi.size)
    up = []
    for i in range(n):
        for j in range(n - i):
            up.append((index[i, j], index[i + 1, j], index[i, j + 1]))
            if i + j + 1 < n:
                up.append((index[i + 1, j], index[i + 1, j + 1], index[i, j + 1]))
    up = np.array(up, np.int64)
    tris = []
    for a, b, c in F:
        pa, pb, pc = V[a], V[b], V[c]
        pts = (pa[None, :] * ((n - bi - bj) / n)[:, None] + pb[None, :] * (bi / n)[:, None] +
               pc[None, :] * (bj / n)[:, None])
        pts /= np.linalg.norm(pts, axis=1, keepdims=True)
        tris.append(pts[up])
    tris = np.concatenate(tris)  # (20 n^2, 3, 3), unit sphere
    flat = tris.reshape(-1, 3)
    r = 1.0 + amplitude * fbm(flat * 2.0, seed)
    return (flat * r[:, None]).reshape(-1, 3, 3).astype(np.float32)


def dense_mesh_scene(stl_path, seed=3):
    """Dense-mesh workload: a displaced geodesic sphere (frequency 209: 873,620 triangles, the nearest
    geodesic count to 871k) in a thin-film material (IOR 1.33, thickness U[300,600] nm), a grey 0.5
    floor and two rectangular lights (1920x1080, 1024 spp, depth 12)."""
    rng = np.random.default_rng(seed)
    thickness = float(rng.uniform(300.0, 600.0))
    mats = [
        {"name": "iridescent", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.8, 0.8, 0.8]},
         "thin_film": {"refractive_index": 1.33, "thickness": thickness}},
        {"name": "floor", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.5, 0.5, 0.5]}},
        {"name": "lamp", "kind": "DiffuseLight", "emit": {"kind": "SolidColor", "color": {"xyz_e": [8, 8, 8]}}},
    ]
    objects = [
        {"kind": "Quad", "q": [-20, -1.2, -20], "u": [40, 0, 0], "v": [0, 0, 40], "material": "floor"},
        {"kind": "STL", "path": stl_path, "center": [0, 0, 0], "scale": 1.0, "rotation": [0, 0, 0],
         "material": "iridescent"},
        {"kind": "Quad", "priority": True, "q": [-3, 4, -1], "u": [2, 0, 0], "v": [0, 0, 2], "material": "lamp"},
        {"kind": "Quad", "priority": True, "q": [2, 3, 1], "u": [0, 0, 1.5], "v": [1.5, 0.5, 0], "material": "lamp"},
    ]
    camera = {"look_from": [0.0, 1.0, 4.5], "look_at": [0.0, 0.0, 0.0], "up": [0.0, 1.0, 0.0],
              "vertical_fov": 40.0, "aperture": 0.0, "focus_distance": 4.5}
    return {"time_0": 0, "time_1": 1, "camera": camera, "background_color": [0.02, 0.02, 0.03],
            "objects": objects, "materials": mats}


def batch_scene(index, stl_dir):
    """Scene `index` (0..63, seed 100 + index) of the batched multi-scene workload: a displaced geodesic
    sphere of 1k-200k triangles (log-uniform; frequency f gives 20 f^2 triangles), 0-3 constant-density
    smoke boxes (density U[0.01, 0.2]), a Lambertian / dielectric / thin-film sphere material, a grey floor
    and one area light.  Returns (scene dict, width, height, spp)."""
    import os
    rng = np.random.default_rng(100 + index)
    ntri = float(np.exp(rng.uniform(np.log(1000.0), np.log(200000.0))))
    freq = max(7, int(round((ntri / 20.0) ** 0.5)))
    stl = write_binary_stl(os.path.join(stl_dir, "batch_%02d.stl" % index),
                           displaced_icosphere(freq, seed=100 + index, amplitude=0.15))
    kind = int(rng.integers(0, 3))
    if kind == 0:
        mat = {"name": "body", "kind": "Lambertian",
               "albedo": {"kind": "SolidColor", "color": [float(x) for x in rng.uniform(0.2, 0.9, 3)]}}
    elif kind == 1:
        mat = {"name": "body", "kind": "Dielectric", "refractive_index": float(rng.uniform(1.3, 1.7))}
    else:
        mat = {"name": "body", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.8, 0.8, 0.8]},
               "thin_film": {"refractive_index": 1.33, "thickness": float(rng.uniform(300.0, 600.0))}}
    objects = [
        {"kind": "Quad", "q": [-10, -1.2, -10], "u": [20, 0, 0], "v": [0, 0, 20], "material": "floor"},
        {"kind": "STL", "path": stl, "center": [0, 0, 0], "scale": 1.0, "rotation": [0, 0, 0], "material": "body"},
        {"kind": "Quad", "priority": True, "q": [-1.5, 3.5, -1.5], "u": [3, 0, 0], "v": [0, 0, 3], "material": "lamp"},
    ]
    for k in range(int(rng.integers(0, 4))):
        c = rng.uniform(-2.5, 2.5, 3)
        c[1] = rng.uniform(-1.0, 0.5)
        s = rng.uniform(0.4, 1.0, 3)
        objects.append({"kind": "ConstantMedium", "density": float(rng.uniform(0.01, 0.2)),
                        "boundary": {"kind": "Boxy", "corner_0": [float(x) for x in c],
                                     "corner_1": [float(x) for x in c + s]},
                        "texture": {"kind": "SolidColor", "color": [0.9, 0.9, 0.9]}})
    materials = [mat,
                 {"name": "floor", "kind": "Lambertian", "albedo": {"kind": "SolidColor", "color": [0.5, 0.5, 0.5]}},
                 {"name": "lamp", "kind": "DiffuseLight", "emit": {"kind": "SolidColor", "color": {"xyz_e": [6, 6, 6]}}}]
    camera = {"look_from": [0.0, 1.0, 4.5], "look_at": [0.0, 0.0, 0.0], "up": [0.0, 1.0, 0.0],
              "vertical_fov": 45.0, "aperture": 0.0, "focus_distance": 4.5}
    side = int(2 ** rng.uniform(7, 10)) // 8 * 8
    spp = int(2 ** int(rng.integers(4, 10)))
    return ({"time_0": 0, "time_1": 1, "camera": camera, "background_color": [0.05, 0.05, 0.08],
             "objects": objects, "materials": materials}, side, side, spp)
