"""clovers_gb300 -- the clovers render hot path on GB300 (sm_103a).

A drop-in for the reference's render path (clovers-cli's ``draw_cpu::draw``
and the scene it renders).  The names and argument meanings below mirror the
reference:

* :class:`GlobalOptions`, :class:`RenderOptions` -- clovers-cli/src/lib.rs:17-25,
  clovers-cli/src/render.rs:16-49 (same fields, same defaults);
* :func:`initialize` -- clovers-cli/src/json_scene.rs:12-27;
* :func:`draw` -- clovers-cli/src/draw_cpu.rs:26-98, returning the
  ``Vec<Xyz<E>>`` pixel buffer as a ``(height*width, 3)`` float32 array, row 0
  at the top of the image;
* :func:`render` -- clovers-cli/src/render.rs:81-183 (load, draw, write).

All computation runs in ``libclovers_gb300.so`` (CUDA kernels for sm_103a);
there is no CPU fallback.
"""

import ctypes
import dataclasses
import os
from typing import List, Optional

import numpy as np

from . import _lib
from ._lib import ClvError, check, lib

__all__ = ["GlobalOptions", "RenderOptions", "Scene", "DeviceScene", "initialize", "draw", "draw_batch", "render",
           "raycast", "resolve_srgb", "ClvError", "DeviceBuffer", "Guide", "draw_guided", "render_guided"]


@dataclasses.dataclass
class GlobalOptions:
    """clovers-cli/src/lib.rs:17-25"""
    debug: bool = False
    quiet: bool = False


@dataclasses.dataclass
class RenderOptions:
    """clovers-cli/src/render.rs:16-49, same defaults; ``seed`` selects the random streams."""
    input: str = ""
    output: Optional[str] = None
    width: int = 1024
    height: int = 1024
    samples: int = 64
    max_depth: int = 64
    mode: str = "path-tracing"
    sampler: str = "random"
    bvh: str = "sah"
    formats: List[str] = dataclasses.field(default_factory=lambda: ["png"])
    seed: int = 0


def _bvh_code(bvh):
    if bvh == "sah":
        return _lib.CLV_BVH_SAH
    if bvh == "lam":
        return _lib.CLV_BVH_LAM
    raise ValueError("unknown BVH algorithm %r" % bvh)


class Scene:
    """A scene flattened on the host (clovers::scenes::Scene equivalent)."""

    def __init__(self, handle):
        self._h = ctypes.c_void_p(handle)

    @classmethod
    def from_json(cls, path, width, height, bvh="sah"):
        out = ctypes.c_void_p()
        check(lib().clv_scene_load_json(os.fsencode(path), width, height, _bvh_code(bvh), ctypes.byref(out)))
        return cls(out.value)

    @classmethod
    def from_json_text(cls, text, width, height, base_dir=".", bvh="sah"):
        out = ctypes.c_void_p()
        check(lib().clv_scene_load_json_text(text.encode(), os.fsencode(base_dir), width, height, _bvh_code(bvh),
                                             ctypes.byref(out)))
        return cls(out.value)

    @classmethod
    def from_mesh(cls, vertices, indices):
        v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 3)
        i = np.ascontiguousarray(indices, dtype=np.uint32).reshape(-1, 3)
        out = ctypes.c_void_p()
        check(lib().clv_scene_from_mesh(v.ctypes.data, v.shape[0], i.ctypes.data, i.shape[0], ctypes.byref(out)))
        return cls(out.value)

    def set_watertight(self, on=True):
        """Watertight triangle test (CLV_OPT_WATERTIGHT) for the next upload."""
        check(lib().clv_scene_set_option(self._h, _lib.CLV_OPT_WATERTIGHT, 1 if on else 0))
        return self

    def info(self):
        inf = _lib.SceneInfoC()
        check(lib().clv_scene_info_get(self._h, ctypes.byref(inf)))
        return {f: getattr(inf, f) for f, _ in _lib.SceneInfoC._fields_}

    def upload(self):
        return DeviceScene(self)

    def close(self):
        if self._h and self._h.value:
            lib().clv_scene_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceScene:
    """A scene resident in GPU memory."""

    def __init__(self, scene):
        out = ctypes.c_void_p()
        check(lib().clv_scene_upload(scene._h, ctypes.byref(out)))
        self._h = out
        self.info = scene.info()

    @property
    def handle(self):
        return self._h

    def close(self):
        if self._h and self._h.value:
            lib().clv_device_scene_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def status(self):
        f = ctypes.c_uint32()
        check(lib().clv_device_status(self._h, ctypes.byref(f)))
        return f.value

    def set_shape(self, path_slots=0, shade_blocks_per_sm=0, warp_appends=0, diffuse_blocks_per_sm=0):
        """clv_device_scene_set_shape: the wavefront shape of later renders (0 = built-in defaults)."""
        check(lib().clv_device_scene_set_shape(self._h, path_slots, shade_blocks_per_sm, warp_appends,
                                               diffuse_blocks_per_sm))

    def autotune(self, render_options, stream=None):
        """clv_autotune on a short render: the chosen shape is kept for later
        renders of this scene; returns [(path_slots, shade_blocks_per_sm, warp_appends,
        diffuse_blocks_per_sm, ms)]."""
        o = render_opts(render_options)
        res = (_lib.TuneResultC * 64)()
        n = ctypes.c_uint32()
        check(lib().clv_autotune(self._h, ctypes.byref(o), res, 64, ctypes.byref(n), stream))
        return [(r.path_slots, r.shade_blocks_per_sm, r.warp_appends, r.diffuse_blocks_per_sm, r.ms)
                for r in res[:n.value]]


def render_opts(opts: RenderOptions, sample_offset=0, path_slots=0):
    if opts.sampler != "random":
        raise ClvError(_lib.CLV_E_INVALID, "only the random sampler is supported")
    if opts.mode not in _lib.MODES:
        raise ValueError("unknown render mode %r" % opts.mode)
    return _lib.RenderOptsC(opts.width, opts.height, opts.samples, opts.max_depth, _lib.MODES[opts.mode], 0,
                            opts.seed, sample_offset, path_slots)


def initialize(path, bvh, width, height):
    """json_scene::initialize: load + flatten + upload; returns a DeviceScene."""
    return Scene.from_json(path, width, height, bvh).upload()


def draw(global_options: GlobalOptions, render_options: RenderOptions, scene: DeviceScene, sampler=None,
         stats=None):
    """draw_cpu::draw: the (height*width, 3) float32 XYZ(E) pixel buffer, row 0 at the top."""
    del global_options, sampler
    o = render_opts(render_options)
    out = np.empty((render_options.height * render_options.width, 3), dtype=np.float32)
    st = _lib.StatsC()
    check(lib().clv_render(scene.handle, ctypes.byref(o), out.ctypes.data, ctypes.byref(st)))
    if stats is not None:
        stats.update(gpu_ms=st.gpu_ms, samples=st.samples, device_errors=st.device_errors,
                     kernel_launches=st.kernel_launches)
    return out


class DeviceBuffer:
    """Device memory owned by the library's allocator (films, ray buffers)."""

    def __init__(self, nbytes):
        p = ctypes.c_void_p()
        check(lib().clv_device_alloc(nbytes, ctypes.byref(p)))
        self.ptr, self.nbytes = p, nbytes

    def zero(self):
        check(lib().clv_memset(self.ptr, 0, self.nbytes))
        return self

    def to_numpy(self, dtype, shape):
        out = np.empty(shape, dtype)
        check(lib().clv_memcpy(out.ctypes.data, self.ptr, out.nbytes))
        return out

    def __del__(self):
        try:
            if self.ptr:
                lib().clv_device_free(self.ptr)
        except Exception:
            pass


def draw_batch(scenes, options, stats=None, guide=None, alpha=0.5):
    """Renders several scenes in one wavefront (clv_render_batch, or clv_render_batch_guided with a
    guide): a list of (h*w, 3) XYZ(E) means."""
    n = len(scenes)
    if n == 0 or n != len(options):
        raise ValueError("one RenderOptions per scene")
    opts = (_lib.RenderOptsC * n)(*[render_opts(o) for o in options])
    films = [DeviceBuffer(o.width * o.height * 3 * 8).zero() for o in options]
    handles = (ctypes.c_void_p * n)(*[s.handle.value for s in scenes])
    ptrs = (ctypes.c_void_p * n)(*[f.ptr.value for f in films])
    if guide is None:
        check(lib().clv_render_batch(handles, opts, ptrs, n, None))
    else:
        check(lib().clv_render_batch_guided(handles, opts, ptrs, n, guide.handle, alpha, None))
    out = []
    for f, o in zip(films, options):
        out.append((f.to_numpy(np.float64, (o.width * o.height, 3)) / o.samples).astype(np.float32))
    return out


GUIDE_PARAMS = 22016
GUIDE_OUTPUTS = 40


class Guide:
    """The learned path guide (clv_guide_*): an MLP that maps a Lambertian path
    vertex to an 8-lobe von Mises-Fisher mixture over incident directions,
    trained online on the records of guided renders.  No counterpart in the
    reference."""

    def __init__(self, record_capacity=0, learning_rate=0.0, seed=0):
        o = _lib.GuideOptsC(record_capacity, learning_rate, seed)
        h = ctypes.c_void_p()
        check(lib().clv_guide_create(ctypes.byref(o), ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def params(self):
        p = np.empty(GUIDE_PARAMS, np.float32)
        check(lib().clv_guide_get_params(self._h, p.ctypes.data))
        return p

    def set_params(self, p):
        a = np.ascontiguousarray(p, np.float32).reshape(GUIDE_PARAMS)
        check(lib().clv_guide_set_params(self._h, a.ctypes.data))

    def forward(self, queries):
        """Raw outputs (n, 40) for normalised inputs (n, 8) = u0..u6, 0."""
        q = np.ascontiguousarray(queries, np.float32).reshape(-1, 8)
        out = np.empty((q.shape[0], GUIDE_OUTPUTS), np.float32)
        check(lib().clv_guide_forward(self._h, q.ctypes.data, q.shape[0], out.ctypes.data))
        return out

    def gradient(self, records):
        """(gradient sums (22016,), loss sum) of -f log q(w) over records (n, 12)."""
        r = np.ascontiguousarray(records, np.float32).reshape(-1, 12)
        g = np.empty(GUIDE_PARAMS, np.float32)
        loss = ctypes.c_double()
        check(lib().clv_guide_gradient(self._h, r.ctypes.data, r.shape[0], g.ctypes.data, ctypes.byref(loss)))
        return g, loss.value

    def train(self, steps, batch=0, stream=None):
        """Adam steps on the records of the last guided render; returns their mean loss."""
        loss = ctypes.c_double()
        check(lib().clv_guide_train(self._h, steps, batch, ctypes.byref(loss), stream))
        return loss.value

    def records(self):
        """Training records (n, 12) of the last guided render: u0..u6, 0, w.xyz, f."""
        n = ctypes.c_uint64()
        check(lib().clv_guide_record_count(self._h, ctypes.byref(n)))
        out = np.empty((n.value, 12), np.float32)
        check(lib().clv_guide_get_records(self._h, out.ctypes.data, n.value))
        return out

    def status(self):
        f = ctypes.c_uint32()
        check(lib().clv_guide_status(self._h, ctypes.byref(f)))
        return f.value

    def close(self):
        if self._h and self._h.value:
            lib().clv_guide_free(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def render_guided(scene: DeviceScene, render_options: RenderOptions, guide: Guide, alpha, film: "DeviceBuffer",
                  sample_offset=0, stream=None):
    """One guided render pass adding its film sums into `film` (clv_render_guided)."""
    o = render_opts(render_options, sample_offset=sample_offset)
    check(lib().clv_render_guided(scene.handle, ctypes.byref(o), guide.handle, alpha, film.ptr, stream))


def draw_guided(global_options: GlobalOptions, render_options: RenderOptions, scene: DeviceScene, guide=None,
                alpha=0.5, train_passes=32, pass_spp=4, train_steps=64, train_batch=32768, chunk_spp=32):
    """draw() with online path guiding: `train_passes` passes of `pass_spp`
    samples per pixel (the first with alpha 0, the reference's estimator), each
    followed by `train_steps` Adam steps on its records, then passes of
    `chunk_spp` with the trained guide.  Every pass adds to the image (all are
    unbiased).  Returns the (height*width, 3) float32 XYZ(E) means, like draw()."""
    del global_options
    guide = guide or Guide()
    w, h, spp = render_options.width, render_options.height, render_options.samples
    film = DeviceBuffer(w * h * 3 * 8).zero()
    done, k = 0, 0
    while done < spp:
        training = k < train_passes
        n = min(pass_spp if training else chunk_spp, spp - done)
        opts = dataclasses.replace(render_options, samples=n)
        render_guided(scene, opts, guide, 0.0 if k == 0 else alpha, film, sample_offset=done)
        if training and train_steps:
            guide.train(train_steps, train_batch)
        done += n
        k += 1
    return (film.to_numpy(np.float64, (w * h, 3)) / spp).astype(np.float32)


def raycast(scene: DeviceScene, rays, with_counts=False, out=None):
    """Closest hits of rays (n, 8) = {ox,oy,oz,tmin,dx,dy,dz,tmax}: (prim_id u32, t f32[, nodes, tests]).
    `out` = (prim, t): arrays of n u32 / f32 to fill instead of new ones (repeated casts reuse them)."""
    r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 8)
    n = r.shape[0]
    if out is not None:
        prim, t = out
        if prim.dtype != np.uint32 or t.dtype != np.float32 or prim.size != n or t.size != n or \
                not (prim.flags.c_contiguous and t.flags.c_contiguous):
            raise ValueError("out must be contiguous u32 and f32 arrays of one entry per ray")
    else:
        prim = np.empty(n, np.uint32)
        t = np.empty(n, np.float32)
    nodes = np.empty(n, np.uint32) if with_counts else None
    tests = np.empty(n, np.uint32) if with_counts else None
    check(lib().clv_raycast(scene.handle, r.ctypes.data, n, prim.ctypes.data, t.ctypes.data,
                            nodes.ctypes.data if with_counts else None, tests.ctypes.data if with_counts else None))
    return (prim, t, nodes, tests) if with_counts else (prim, t)


def resolve_srgb(xyz, width, height):
    """write.rs:39-44 colour conversion: XYZ(E) means -> sRGB u8, (height*width, 3)."""
    x = np.ascontiguousarray(xyz, dtype=np.float32).reshape(-1, 3)
    out = np.empty((width * height, 3), np.uint8)
    check(lib().clv_resolve_srgb(x.ctypes.data, width, height, out.ctypes.data))
    return out


def render(global_options: GlobalOptions, render_options: RenderOptions):
    """render.rs:81-183: load the scene, draw, write the requested formats."""
    from .imageio import format_duration, write_png, write_exr
    import time

    o = render_options
    if not global_options.quiet:  # render.rs:112-125
        print("clovers \U0001F340 path tracing renderer")
        print()
        print("%dx%d resolution" % (o.width, o.height))
        if o.mode == "normal-map":
            print("rendering a normalmap")
        else:
            print("%d samples per pixel" % o.samples)
            print("using the %s sampler" % o.sampler)
            print("%d max bounce depth" % o.max_depth)
        print()
    if o.sampler == "blue":
        if o.samples not in (1, 2, 4, 8, 16, 32, 64, 128, 256):  # render.rs:127-129
            raise ClvError(_lib.CLV_E_INVALID, "the blue sampler only supports the following sample-per-pixel "
                                               "counts: [1, 2, 4, 8, 16, 32, 64, 128, 256]")
        raise ClvError(_lib.CLV_E_INVALID, "the blue-noise sampler is not available in this build (its "
                                           "precomputed tables are not part of it); use --sampler random")
    if not render_options.input.endswith(".json"):
        raise ClvError(_lib.CLV_E_INVALID, "Unknown file type")
    scene = initialize(render_options.input, render_options.bvh, render_options.width, render_options.height)
    t0 = time.perf_counter()
    pixels = draw(global_options, render_options, scene)
    duration = time.perf_counter() - t0
    if not global_options.quiet:
        print("Finished render in %s" % format_duration(duration))
    written = []
    for fmt in render_options.formats:
        target = (render_options.output or os.path.join("renders", str(int(time.time())))) + "." + fmt
        os.makedirs(os.path.dirname(target) or ".", exist_ok=True)
        if fmt == "png":
            rgb = resolve_srgb(pixels, render_options.width, render_options.height)
            write_png(target, rgb, render_options.width, render_options.height, render_options, duration)
        elif fmt == "exr":
            write_exr(target, pixels, render_options.width, render_options.height)
        else:
            raise ValueError("unknown format %r" % fmt)
        written.append(target)
        print("Image saved to: %s" % target)  # printed in quiet mode too (render.rs:179)
    return written
