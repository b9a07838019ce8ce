"""ctypes binding of ``include/clovers_gpu.h`` (libclovers_gb300.so).

The library is built in-tree (``clovers_gb300/_build``).  Importing this
module never falls back to anything else: if the shared library is missing
or cannot be loaded, :func:`lib` raises.
"""

import ctypes
import os
import threading

from . import build as _build

c_u32, c_u64, c_i32, c_f32, c_f64 = ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int, ctypes.c_float, ctypes.c_double
P = ctypes.POINTER

CLV_OK, CLV_E_INVALID, CLV_E_SCENE, CLV_E_CUDA, CLV_E_DEVICE = 0, -1, -2, -3, -4
CLV_BVH_LAM, CLV_BVH_SAH = 0, 1
CLV_OPT_WATERTIGHT = 1
MODES = {"path-tracing": 0, "normal-map": 1, "bvh-test-count": 2, "primitive-test-count": 3}


class RenderOptsC(ctypes.Structure):
    _fields_ = [("width", c_u32), ("height", c_u32), ("samples", c_u32), ("max_depth", c_u32),
                ("mode", c_u32), ("sampler", c_u32), ("seed", c_u64), ("sample_offset", c_u32),
                ("path_slots", c_u32)]


class SceneInfoC(ctypes.Structure):
    _fields_ = [("objects", c_u64), ("nodes", c_u32), ("triangles", c_u32), ("quads", c_u32),
                ("spheres", c_u32), ("compound", c_u32), ("materials", c_u32), ("tree_depth", c_u32),
                ("mis_nodes", c_u32), ("width", c_u32), ("height", c_u32), ("traversal_level", c_u32)]


class StatsC(ctypes.Structure):
    _fields_ = [("gpu_ms", c_f64), ("samples", c_u64), ("device_errors", c_u32), ("kernel_launches", c_u32)]


class GuideOptsC(ctypes.Structure):
    _fields_ = [("record_capacity", c_u32), ("learning_rate", c_f32), ("seed", c_u64)]


class TuneResultC(ctypes.Structure):
    _fields_ = [("path_slots", c_u32), ("shade_blocks_per_sm", c_u32), ("warp_appends", c_u32),
                ("diffuse_blocks_per_sm", c_u32), ("ms", c_f32)]


class RenderProfileC(ctypes.Structure):
    _fields_ = [("ms_init", c_f64), ("ms_intersect", c_f64), ("ms_shade", c_f64), ("intersect_launches", c_u64),
                ("shade_launches", c_u64), ("paths", c_u64), ("path_segments", c_u64), ("node_visits", c_u64),
                ("prim_tests", c_u64), ("path_slots", c_u64)]


# name -> (restype, argtypes); mirrors include/clovers_gpu.h
SIGNATURES = {
    "clv_scene_load_json": (c_i32, [ctypes.c_char_p, c_u32, c_u32, c_i32, P(ctypes.c_void_p)]),
    "clv_scene_load_json_text": (c_i32, [ctypes.c_char_p, ctypes.c_char_p, c_u32, c_u32, c_i32,
                                         P(ctypes.c_void_p)]),
    "clv_scene_from_mesh": (c_i32, [ctypes.c_void_p, c_u32, ctypes.c_void_p, c_u32, P(ctypes.c_void_p)]),
    "clv_scene_info_get": (c_i32, [ctypes.c_void_p, P(SceneInfoC)]),
    "clv_scene_set_option": (c_i32, [ctypes.c_void_p, c_u32, c_u32]),
    "clv_scene_free": (None, [ctypes.c_void_p]),
    "clv_scene_upload": (c_i32, [ctypes.c_void_p, P(ctypes.c_void_p)]),
    "clv_device_scene_free": (None, [ctypes.c_void_p]),
    "clv_render": (c_i32, [ctypes.c_void_p, P(RenderOptsC), ctypes.c_void_p, P(StatsC)]),
    "clv_render_device": (c_i32, [ctypes.c_void_p, P(RenderOptsC), ctypes.c_void_p, ctypes.c_void_p]),
    "clv_render_batch": (c_i32, [ctypes.c_void_p, P(RenderOptsC), ctypes.c_void_p, c_u32, ctypes.c_void_p]),
    "clv_render_device_noalloc": (c_i32, [ctypes.c_void_p, P(RenderOptsC), ctypes.c_void_p, ctypes.c_void_p]),
    "clv_autotune": (c_i32, [ctypes.c_void_p, P(RenderOptsC), ctypes.c_void_p, c_u32, P(c_u32), ctypes.c_void_p]),
    "clv_device_scene_set_shape": (c_i32, [ctypes.c_void_p, c_u32, c_u32, c_u32, c_u32]),
    "clv_resolve_device": (c_i32, [ctypes.c_void_p, c_u32, c_u32, c_u32, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p]),
    "clv_resolve_srgb": (c_i32, [ctypes.c_void_p, c_u32, c_u32, ctypes.c_void_p]),
    "clv_raycast": (c_i32, [ctypes.c_void_p, ctypes.c_void_p, c_u64, ctypes.c_void_p, ctypes.c_void_p,
                            ctypes.c_void_p, ctypes.c_void_p]),
    "clv_raycast_device": (c_i32, [ctypes.c_void_p, ctypes.c_void_p, c_u64, ctypes.c_void_p, ctypes.c_void_p,
                                   ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "clv_device_status": (c_i32, [ctypes.c_void_p, P(c_u32)]),
    "clv_selftest_division": (c_i32, [c_u64, c_u64, P(c_u64)]),
    "clv_selftest_log": (c_i32, [ctypes.c_void_p, ctypes.c_void_p, c_u64, P(c_f64), P(c_u64)]),
    "clv_kernel_launches": (c_u64, []),
    "clv_device_alloc": (c_i32, [c_u64, P(ctypes.c_void_p)]),
    "clv_device_free": (None, [ctypes.c_void_p]),
    "clv_memcpy": (c_i32, [ctypes.c_void_p, ctypes.c_void_p, c_u64]),
    "clv_memset": (c_i32, [ctypes.c_void_p, ctypes.c_int, c_u64]),
    "clv_render_profile_run": (c_i32, [ctypes.c_void_p, P(RenderOptsC), ctypes.c_void_p, ctypes.c_void_p,
                                       P(RenderProfileC)]),
    "clv_guide_create": (c_i32, [P(GuideOptsC), P(ctypes.c_void_p)]),
    "clv_guide_free": (None, [ctypes.c_void_p]),
    "clv_guide_get_params": (c_i32, [ctypes.c_void_p, ctypes.c_void_p]),
    "clv_guide_set_params": (c_i32, [ctypes.c_void_p, ctypes.c_void_p]),
    "clv_render_guided": (c_i32, [ctypes.c_void_p, P(RenderOptsC), ctypes.c_void_p, c_f32, ctypes.c_void_p,
                                  ctypes.c_void_p]),
    "clv_render_batch_guided": (c_i32, [ctypes.c_void_p, P(RenderOptsC), ctypes.c_void_p, c_u32, ctypes.c_void_p,
                                        c_f32, ctypes.c_void_p]),
    "clv_guide_train": (c_i32, [ctypes.c_void_p, c_u32, c_u32, P(c_f64), ctypes.c_void_p]),
    "clv_guide_record_count": (c_i32, [ctypes.c_void_p, P(c_u64)]),
    "clv_guide_get_records": (c_i32, [ctypes.c_void_p, ctypes.c_void_p, c_u64]),
    "clv_guide_forward": (c_i32, [ctypes.c_void_p, ctypes.c_void_p, c_u64, ctypes.c_void_p]),
    "clv_guide_gradient": (c_i32, [ctypes.c_void_p, ctypes.c_void_p, c_u64, ctypes.c_void_p, P(c_f64)]),
    "clv_guide_status": (c_i32, [ctypes.c_void_p, P(c_u32)]),
    "clv_guide_selftest_mma": (c_i32, [c_u32, c_u32, c_u64, ctypes.c_void_p, P(c_f32)]),
    "clv_guide_selftest_timeout": (c_i32, [c_u64, P(c_u32), P(c_u32)]),
    "clv_last_error": (ctypes.c_char_p, []),
    "clv_version": (ctypes.c_char_p, []),
}

_LIB = None
_LOCK = threading.Lock()


def library_path():
    return _build.LIB


def lib(build_if_missing=True):
    """The loaded library.  Builds it when missing (nvcc required); raises otherwise."""
    global _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = library_path()
        if not os.path.exists(path):
            if not build_if_missing:
                raise RuntimeError("libclovers_gb300.so is not built (run clovers_gb300/build.py)")
            _build.build()
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
        return L


class ClvError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("clovers_gb300 error %d: %s" % (code, msg))
        self.code = code


def check(rc):
    if rc != CLV_OK:
        msg = lib().clv_last_error()
        raise ClvError(rc, msg.decode("utf-8", "replace") if msg else "")
    return rc
