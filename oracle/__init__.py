"""CPU oracle of the clovers render path -- TEST INFRASTRUCTURE ONLY.

A ctypes wrapper over ``oracle.cpp`` (a C++ restatement of the reference's
Rust algorithm).  Only the test suite, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of ``bench.py`` may use it, and only as the checker or the
CPU baseline -- never as the product path.
"""

import ctypes
import os
import subprocess
import threading

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
LIB64 = os.path.join(HERE, "_build", "liboracle64.so")  # the same algorithm in double precision
_CSRC = os.path.join(HERE, "..", "clovers_gb300", "csrc")
_SRC = [os.path.join(HERE, "oracle.cpp"), os.path.join(HERE, "guide.cpp"), os.path.join(HERE, "Makefile"),
        os.path.join(_CSRC, "json.hpp"), os.path.join(_CSRC, "spectral_tables.h"), os.path.join(_CSRC, "clv_log.h")]
_L = None
_L64 = None
_LOCK = threading.Lock()


def build(force=False):
    stale = force or any(not os.path.exists(x) for x in (LIB, LIB64)) or any(
        os.path.getmtime(s) > min(os.path.getmtime(LIB), os.path.getmtime(LIB64)) for s in _SRC)
    if stale:
        p = subprocess.run(["make", "-C", HERE, "-B" if force else "all"], stdout=subprocess.PIPE,
                           stderr=subprocess.STDOUT, text=True)
        if p.returncode != 0:
            raise RuntimeError("oracle build failed:\n" + p.stdout)
    return LIB


_SIG = {
    "orc_last_error": ("c_char_p", []),
    "orc_spectral_power": ("i32", ["f32", "f32", "f32", "i32", "pf32"]),
    "orc_wavelength_into_xyz": (None, ["i32", "vp"]),
    "orc_rotate_wavelength": (None, ["i32", "vp"]),
    "orc_srgb_to_xyz_e": (None, ["vp", "vp"]),
    "orc_xyz_e_to_srgb8": (None, ["vp", "u64", "vp"]),
    "orc_aabb_area": ("f32", ["vp"]),
    "orc_aabb_centroid": (None, ["vp", "vp"]),
    "orc_aabb_combine": (None, ["vp", "vp", "vp"]),
    "orc_aabb_hit": ("i32", ["vp", "vp"]),
    "orc_interval": (None, ["f32", "f32", "vp"]),
    "orc_prim_hit": ("i32", ["i32", "vp", "vp", "vp", "vp", "vp", "vp"]),
    "orc_scene_load_json": ("vp", ["c_char_p", "u32", "u32"]),
    "orc_scene_load_json_bvh": ("vp", ["c_char_p", "u32", "u32", "i32"]),
    "orc_scene_from_mesh": ("vp", ["vp", "u32", "vp", "u32"]),
    "orc_scene_free": (None, ["vp"]),
    "orc_scene_set_watertight": (None, ["vp", "i32"]),
    "orc_scene_object_count": ("u64", ["vp"]),
    "orc_scene_tree_stats": (None, ["vp", "vp"]),
    "orc_camera_ray": (None, ["vp", "f32", "f32", "f32", "f32", "vp"]),
    "orc_scene_background_xyz": (None, ["vp", "vp"]),
    "orc_raycast": ("i32", ["vp", "vp", "u64", "vp", "vp", "vp", "vp", "i32"]),
    "orc_render": ("i32", ["vp", "u32", "u32", "u32", "u32", "u64", "u32", "u32", "u32", "u32", "u32", "vp", "i32"]),
    "orc_render_pixels": ("i32", ["vp", "u32", "u32", "u32", "u32", "u64", "vp", "u64", "u32", "vp", "i32"]),
    "orc_render_debug": ("i32", ["vp", "u32", "u32", "u32", "u64", "u32", "vp", "i32"]),
    "orc_trace_sample": ("i32", ["vp", "u32", "u32", "u32", "u32", "u32", "u32", "u64", "vp", "vp", "vp"]),
    "orc_log_f32": (None, ["vp", "u64", "vp"]),
    "orc_guide_forward": (None, ["vp", "vp", "u64", "i32", "vp"]),
    "orc_guide_gradient": ("f64", ["vp", "vp", "u64", "i32", "vp"]),
    "orc_guide_pdf": ("f64", ["vp", "vp"]),
    "orc_guide_sample": (None, ["vp", "f32", "f32", "f32", "vp"]),
}
_CT = {"vp": ctypes.c_void_p, "u32": ctypes.c_uint32, "u64": ctypes.c_uint64, "i32": ctypes.c_int,
       "f32": ctypes.c_float, "f64": ctypes.c_double, "c_char_p": ctypes.c_char_p,
       "pf32": ctypes.POINTER(ctypes.c_float), None: None}


def _load(path):
    L = ctypes.CDLL(path)
    for name, (res, args) in _SIG.items():
        fn = getattr(L, name, None)
        if fn is None:  # the f64 build leaves out the guide
            continue
        fn.restype = _CT[res]
        fn.argtypes = [_CT[a] for a in args]
    return L


def lib():
    """The f32 oracle (the reference's precision): parity checks and the CPU baseline."""
    global _L
    with _LOCK:
        if _L is None:
            build()
            _L = _load(LIB)
        return _L


def lib64():
    """The same algorithm with Float = f64: image-quality references."""
    global _L64
    with _LOCK:
        if _L64 is None:
            build()
            _L64 = _load(LIB64)
        return _L64


def _err():
    return lib().orc_last_error().decode()


def _buf(a):
    return a.ctypes.data


def spectral_power(xyz, lam):
    out = ctypes.c_float()
    if lib().orc_spectral_power(float(xyz[0]), float(xyz[1]), float(xyz[2]), int(lam), ctypes.byref(out)) != 0:
        raise ValueError(_err())
    return np.float32(out.value)


def wavelength_into_xyz(lam):
    o = np.zeros(3, np.float32)
    lib().orc_wavelength_into_xyz(int(lam), _buf(o))
    return o


def rotate_wavelength(hero):
    o = np.zeros(4, np.int32)
    lib().orc_rotate_wavelength(int(hero), _buf(o))
    return o


def srgb_to_xyz_e(rgb):
    i = np.asarray(rgb, np.float32)
    o = np.zeros(3, np.float32)
    lib().orc_srgb_to_xyz_e(_buf(i), _buf(o))
    return o


def xyz_e_to_srgb8(xyz):
    x = np.ascontiguousarray(xyz, np.float32).reshape(-1, 3)
    o = np.zeros_like(x, dtype=np.uint8)
    lib().orc_xyz_e_to_srgb8(_buf(x), x.shape[0], _buf(o))
    return o


def aabb_area(box):
    b = np.asarray(box, np.float32)
    return np.float32(lib().orc_aabb_area(_buf(b)))


def aabb_centroid(box):
    b = np.asarray(box, np.float32)
    o = np.zeros(3, np.float32)
    lib().orc_aabb_centroid(_buf(b), _buf(o))
    return o


def aabb_combine(a, b):
    x, y = np.asarray(a, np.float32), np.asarray(b, np.float32)
    o = np.zeros(6, np.float32)
    lib().orc_aabb_combine(_buf(x), _buf(y), _buf(o))
    return o


def aabb_hit(box, ray):
    b, r = np.asarray(box, np.float32), np.asarray(ray, np.float32)
    return bool(lib().orc_aabb_hit(_buf(b), _buf(r)))


def interval(a, b):
    o = np.zeros(4, np.float32)
    lib().orc_interval(float(a), float(b), _buf(o))
    return o  # min, max, size, center


def prim_hit(kind, q, u, v, ray):
    """kind 1 triangle, 2 quad, 3 sphere (q = center, u[0] = radius).  -> (hit, record[10], box[6])"""
    qa, ua, va = (np.asarray(x, np.float32) for x in (q, u, v))
    r = np.asarray(ray, np.float32)
    rec = np.zeros(10, np.float32)
    box = np.zeros(6, np.float32)
    h = lib().orc_prim_hit(kind, _buf(qa), _buf(ua), _buf(va), _buf(r), _buf(rec), _buf(box))
    return bool(h), rec, box


def log_f32(x):
    """ln through the render path's own logarithm (clovers_gb300/csrc/clv_log.h), as f32."""
    a = np.ascontiguousarray(x, np.float32).reshape(-1)
    y = np.empty_like(a)
    lib().orc_log_f32(_buf(a), a.size, _buf(y))
    return y


class Scene:
    """A scene of the oracle.  precision "f32" is the reference's arithmetic (parity checks, the CPU
    baseline); "f64" runs the same algorithm in double precision (image-quality references)."""

    def __init__(self, handle, L=None):
        self._L = L or lib()
        if not handle:
            raise ValueError(self._L.orc_last_error().decode())
        self.h = ctypes.c_void_p(handle)

    @staticmethod
    def _lib_for(precision):
        if precision not in ("f32", "f64"):
            raise ValueError("precision must be f32 or f64")
        return lib() if precision == "f32" else lib64()

    def _error(self):
        return self._L.orc_last_error().decode()

    @classmethod
    def from_json(cls, path, width, height, bvh="sah", precision="f32"):
        if bvh not in ("sah", "lam"):
            raise ValueError("unknown BVH algorithm %r" % bvh)
        L = cls._lib_for(precision)
        return cls(L.orc_scene_load_json_bvh(os.fsencode(path), width, height, 0 if bvh == "lam" else 1), L)

    @classmethod
    def from_mesh(cls, verts, idx, precision="f32"):
        v = np.ascontiguousarray(verts, np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(idx, np.uint32).reshape(-1, 3)
        L = cls._lib_for(precision)
        return cls(L.orc_scene_from_mesh(_buf(v), v.shape[0], _buf(i), i.shape[0]), L)

    def __del__(self):
        try:
            if self.h and self.h.value:
                self._L.orc_scene_free(self.h)
        except Exception:
            pass

    def set_watertight(self, on=True):
        """Watertight triangle test on every triangle (no counterpart in the reference)."""
        self._L.orc_scene_set_watertight(self.h, 1 if on else 0)
        return self

    def object_count(self):
        return self._L.orc_scene_object_count(self.h)

    def tree_stats(self):
        o = np.zeros(3, np.uint64)
        self._L.orc_scene_tree_stats(self.h, _buf(o))
        return {"nodes": int(o[0]), "tree_depth": int(o[1]), "mis_nodes": int(o[2])}

    def camera_ray(self, pu, pv, lx=0.0, ly=0.0):
        o = np.zeros(6, np.float32)
        self._L.orc_camera_ray(self.h, pu, pv, lx, ly, _buf(o))
        return o

    def background_xyz(self):
        o = np.zeros(3, np.float32)
        self._L.orc_scene_background_xyz(self.h, _buf(o))
        return o

    def raycast(self, rays, threads=None, with_counts=False):
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = r.shape[0]
        prim = np.empty(n, np.uint32)
        t = np.empty(n, np.float32)
        nodes = np.empty(n, np.uint32) if with_counts else None
        tests = np.empty(n, np.uint32) if with_counts else None
        self._L.orc_raycast(self.h, _buf(r), n, _buf(prim), _buf(t), _buf(nodes) if with_counts else None,
                            _buf(tests) if with_counts else None, threads or os.cpu_count() or 1)
        return (prim, t, nodes, tests) if with_counts else (prim, t)

    def render(self, width, height, spp, max_depth, seed, window=None, sample_offset=0, threads=None):
        """Per-pixel SUM of film deposits (f64), window = (x0, r0, x1, r1) in buffer coordinates."""
        x0, r0, x1, r1 = window or (0, 0, width, height)
        out = np.zeros(((r1 - r0) * (x1 - x0), 3), np.float64)
        rc = self._L.orc_render(self.h, width, height, spp, max_depth, seed, x0, r0, x1, r1, sample_offset,
                                _buf(out), threads or os.cpu_count() or 1)
        if rc != 0:
            raise RuntimeError(self._error())
        return out

    def render_pixels(self, width, height, spp, max_depth, seed, pixels, sample_offset=0, threads=None):
        """Per-pixel SUM of film deposits (f64) for buffer pixels r * width + x (any order)."""
        px = np.ascontiguousarray(pixels, np.uint32).reshape(-1)
        out = np.zeros((px.size, 3), np.float64)
        rc = self._L.orc_render_pixels(self.h, width, height, spp, max_depth, seed, _buf(px), px.size, sample_offset,
                                       _buf(out), threads or os.cpu_count() or 1)
        if rc != 0:
            raise RuntimeError(self._error())
        return out

    def render_debug(self, width, height, mode, seed, sample_offset=0, threads=None):
        """Debug render modes (1 normal map, 2 BVH test count, 3 primitive test count): (h*w, 3) linear sRGB."""
        out = np.zeros((width * height, 3), np.float32)
        rc = self._L.orc_render_debug(self.h, width, height, mode, seed, sample_offset, _buf(out),
                                      threads or os.cpu_count() or 1)
        if rc != 0:
            raise RuntimeError(self._error())
        return out

    def trace_sample(self, width, height, x, r, sample, max_depth, seed):
        p = np.zeros(4, np.float32)
        w = np.zeros(4, np.int32)
        ray = np.zeros(6, np.float32)
        if self._L.orc_trace_sample(self.h, width, height, x, r, sample, max_depth, seed, _buf(p), _buf(w),
                                    _buf(ray)) != 0:
            raise RuntimeError(self._error())
        return p, w, ray


# ---- path guide (specification restated in oracle/guide.cpp) ----------------
GUIDE_PARAMS = 22016
GUIDE_OUTPUTS = 40


def guide_forward(params, queries, bf16=True):
    """Raw network outputs (n, 40) for queries (n, 8) = normalised inputs u0..u6, 0."""
    p = np.ascontiguousarray(params, np.float32).reshape(GUIDE_PARAMS)
    q = np.ascontiguousarray(queries, np.float32).reshape(-1, 8)
    out = np.empty((q.shape[0], GUIDE_OUTPUTS), np.float32)
    lib().orc_guide_forward(p.ctypes.data, q.ctypes.data, q.shape[0], 1 if bf16 else 0, out.ctypes.data)
    return out


def guide_gradient(params, records, bf16=True):
    """(gradient sums (22016,) float64, loss sum) of -f log q(w) over records (n, 12)."""
    p = np.ascontiguousarray(params, np.float32).reshape(GUIDE_PARAMS)
    r = np.ascontiguousarray(records, np.float32).reshape(-1, 12)
    g = np.empty(GUIDE_PARAMS, np.float64)
    loss = lib().orc_guide_gradient(p.ctypes.data, r.ctypes.data, r.shape[0], 1 if bf16 else 0, g.ctypes.data)
    return g, loss


def guide_pdf(out40, w):
    o = np.ascontiguousarray(out40, np.float32).reshape(GUIDE_OUTPUTS)
    d = np.ascontiguousarray(w, np.float32).reshape(3)
    return lib().orc_guide_pdf(o.ctypes.data, d.ctypes.data)


def guide_sample(out40, u0, u1, u2):
    o = np.ascontiguousarray(out40, np.float32).reshape(GUIDE_OUTPUTS)
    w = np.empty(3, np.float32)
    lib().orc_guide_sample(o.ctypes.data, u0, u1, u2, w.ctypes.data)
    return w
