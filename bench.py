"""Benchmark of the clovers render hot path on GB300.

Workload (one step): the enclosed-box scene (a 555-unit box in the layout of
the reference's cornell.json: five diffuse walls, a 130x105 area light, two
rotated boxes, a glass sphere) rendered at 512x512, 256 samples per pixel,
max depth 16, by the wavefront path tracer: 67,108,864 samples per step.
Metric: Msamples/s = width*height*spp / GPU seconds (whole job over all ranks).

Also reported: the closest-hit ray-cast workload of the same configuration
(2^24 seeded random rays against an SAH BVH over 2^20 random triangles),
as traversal Grays/s with its HBM roofline.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

`--impl reference` times the reference's algorithm on the host cores instead:
the reference (Rust) cannot be built here, so its CPU restatement (oracle/)
runs the same workload, row-parallel over all host threads like the
reference's rayon loop, on a bounded sample of samples per pixel.
"""

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

W_IMG, H_IMG, SPP, DEPTH = 512, 512, 256, 16
RAYS, TRIS = 1 << 24, 1 << 20
SEED = 1


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes from the committed ncu summary (profiles/traffic.txt), if present."""
    out = {}
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    if os.path.exists(path):
        for line in open(path):
            line = line.strip()
            if line and not line.startswith("#") and "=" in line:
                k, v = line.split("=", 1)
                try:
                    out[k.strip()] = float(v)
                except ValueError:
                    pass
    return out


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    FIELDS = ["clocks.sm", "clocks.max.sm", "clocks_event_reasons.active", "clocks_event_reasons.hw_slowdown",
              "clocks_event_reasons.hw_thermal_slowdown", "clocks_event_reasons.sw_thermal_slowdown",
              "clocks_event_reasons.sw_power_cap"]

    def __init__(self, gpu_index):
        self.gpu_index = gpu_index
        self.proc = None
        self.tmp = None

    def __enter__(self):
        try:
            self.tmp = tempfile.NamedTemporaryFile("w+", delete=False, suffix=".csv")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu_index), "--query-gpu=" + ",".join(self.FIELDS),
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.tmp, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.tmp is None:
            return None
        try:
            self.tmp.flush()
            rows = [l.strip().split(", ") for l in open(self.tmp.name) if l.strip()]
            os.unlink(self.tmp.name)
        except Exception:
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            if len(r) < 7:
                continue
            try:
                sm.append(float(r[0]))
                mx.append(float(r[1]))
            except ValueError:
                continue
            for n, v in zip(names, r[3:7]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if args.impl != "reference" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def all_max(world, value):
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def box_scene_file():
    from clovers_gb300 import scenes
    path = os.path.join(tempfile.gettempdir(), "clovers_bench_box_%d.json" % os.getpid())
    scenes.write_scene(scenes.enclosed_box(), path)
    return path


def run_reference(args, world, rank):
    """The reference algorithm (CPU restatement) on the host cores, same workload, bounded sample."""
    if rank != 0:
        return
    import oracle
    threads = os.cpu_count() or 1
    path = box_scene_file()
    sc = oracle.Scene.from_json(path, W_IMG, H_IMG)
    spp_sample = args.cpu_spp
    for i in range(args.warmup):
        sc.render(W_IMG, H_IMG, 1, DEPTH, SEED, window=(0, 0, W_IMG, 16), threads=threads)
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        sc.render(W_IMG, H_IMG, spp_sample, DEPTH, SEED, sample_offset=k * spp_sample, threads=threads)
        times.append(time.perf_counter() - t0)
    samples = W_IMG * H_IMG * spp_sample
    value = samples * len(times) / sum(times) / 1e6
    sample = "%dx%d image at %d spp per step (of the workload's %d spp)" % (W_IMG, H_IMG, spp_sample, SPP)
    rows, spp1 = 16, 16  # one core, beside the all-threads figure: a band of the image
    t0 = time.perf_counter()
    sc.render(W_IMG, H_IMG, spp1, DEPTH, SEED, window=(0, H_IMG // 2, W_IMG, H_IMG // 2 + rows), threads=1)
    el1 = time.perf_counter() - t0
    one_core = {"value": round(W_IMG * rows * spp1 / el1 / 1e6, 4), "unit": "Msamples/s",
                "sample": "%d middle rows of %d pixels at %d spp (%.2f s)" % (rows, W_IMG, spp1, el1)}
    line = {
        "impl": "reference", "metric": "Msamples/s", "value": round(value, 4), "unit": "Msamples/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * sum(times) / len(times), 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded enclosed-box scene)",
        "config": {"workload": "enclosed box %dx%d, %d spp, depth %d" % (W_IMG, H_IMG, SPP, DEPTH), "sample": sample,
                   "parallelism": "host threads"},
        "cpu_baseline": {"value": round(value, 4), "unit": "Msamples/s", "cores": threads, "kind": "port",
                         "sample": sample, "one_core": one_core},
        "e2e": {"value": round(value, 4), "unit": "Msamples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is Rust and cannot be built here (no rustc/cargo); its algorithm runs as the "
                "C++ restatement in oracle/, row-parallel over all host threads",
    }
    print(json.dumps(line), flush=True)
    os.unlink(path)


def cpu_baseline_render(path, spp_sample):
    import oracle
    threads = os.cpu_count() or 1
    sc = oracle.Scene.from_json(path, W_IMG, H_IMG)
    sc.render(W_IMG, H_IMG, 1, DEPTH, SEED, window=(0, 0, W_IMG, 8), threads=threads)  # warm-up
    t0 = time.perf_counter()
    sc.render(W_IMG, H_IMG, spp_sample, DEPTH, SEED, threads=threads)
    el = time.perf_counter() - t0
    rows, spp1 = 16, 16  # one core: a band of the image
    t0 = time.perf_counter()
    sc.render(W_IMG, H_IMG, spp1, DEPTH, SEED, window=(0, H_IMG // 2, W_IMG, H_IMG // 2 + rows), threads=1)
    el1 = time.perf_counter() - t0
    return {"value": round(W_IMG * H_IMG * spp_sample / el / 1e6, 4), "unit": "Msamples/s", "cores": threads,
            "kind": "port", "sample": "%dx%d at %d spp (%.2f s)" % (W_IMG, H_IMG, spp_sample, el),
            "one_core": {"value": round(W_IMG * rows * spp1 / el1 / 1e6, 4), "unit": "Msamples/s",
                         "sample": "%d middle rows of %d pixels at %d spp (%.2f s)" % (rows, W_IMG, spp1, el1)}}


CONFIGS = {
    # name: (scene builder, width, height, spp, depth, description)
    "c1": ("random_spheres", 400, 225, 64, 50, "random spheres 400x225, 64 spp, depth 50"),
    "c3": ("dense_mesh_scene", 1920, 1080, 1024, 12,
           "displaced geodesic sphere (873,620 triangles), thin film, 1920x1080, 1024 spp, depth 12"),
    "c4": ("dispersive_prism", 1024, 1024, 256, 16, "dispersive prism + sphere, 1024x1024, depth 16 (plain)"),
    "box": ("enclosed_box", 512, 512, 256, 16, "enclosed box 512x512, 256 spp, depth 16"),
}
GOLDEN = {"c4": "prism", "box": "box", "c1": "spheres", "c3": "dense"}


def config_scene_file(builder, tmp):
    from clovers_gb300 import scenes
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
    return scenes.write_scene(sc, os.path.join(tmp, builder + ".json"))


def run_batch(args):
    """64 scenes of uneven size in one wavefront (clv_render_batch) vs the same renders one by one."""
    import torch
    import clovers_gb300 as cg
    from clovers_gb300 import _lib, scenes
    L = _lib.lib()
    sp = torch.cuda.current_stream().cuda_stream
    tmp = tempfile.mkdtemp()
    dev, opts, films, samples, tris = [], [], [], 0, 0
    t0 = time.perf_counter()
    for k in range(args.batch_scenes):
        sc, w, h, spp = scenes.batch_scene(k, tmp)
        path = scenes.write_scene(sc, os.path.join(tmp, "batch_%02d.json" % k))
        hs = cg.Scene.from_json(path, w, h)
        tris += hs.info()["triangles"]
        dev.append(hs.upload())
        opts.append(cg.render_opts(cg.RenderOptions(width=w, height=h, samples=spp, max_depth=DEPTH, seed=100 + k)))
        films.append(torch.zeros(w * h * 3, dtype=torch.float64, device="cuda"))
        samples += w * h * spp
    load_s = time.perf_counter() - t0
    n = len(dev)
    handles = (ctypes.c_void_p * n)(*[d.handle.value for d in dev])
    optarr = (_lib.RenderOptsC * n)(*opts)
    batch_opts = (_lib.RenderOptsC * n)(*opts)
    batch_opts[0].path_slots = args.batch_slots  # the batch's paths in flight (0: clv_render_batch's default)
    for k in range(n):
        optarr[k].path_slots = args.single_slots  # the one-by-one renders' paths in flight (0: their defaults)
    ptrs = (ctypes.c_void_p * n)(*[f.data_ptr() for f in films])

    def timed(fn):
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        return e0.elapsed_time(e1)

    def batched():
        _lib.check(L.clv_render_batch(handles, batch_opts, ptrs, n, sp))

    def one_by_one():
        for k in range(n):
            _lib.check(L.clv_render_device(dev[k].handle, ctypes.byref(optarr[k]), films[k].data_ptr(), sp))

    for _ in range(args.warmup):
        batched()
    t_batch = min(timed(batched) for _ in range(args.steps))
    t_seq = min(timed(one_by_one) for _ in range(args.steps))
    line = {"metric": "Msamples/s", "value": round(samples / (t_batch / 1e3) / 1e6, 3), "unit": "Msamples/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_batch, 3),
            "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeds 100..%d)" % (99 + n),
            "config": {"workload": "%d scenes in one wavefront: displaced geodesic spheres 1k-200k triangles, "
                                   "0-3 smoke boxes, 128^2-1024^2, 16-512 spp, depth %d" % (n, DEPTH),
                       "samples_per_step": samples, "triangles": tris, "scene_load_s": round(load_s, 2),
                       "batch_path_slots": args.batch_slots or "default", "single_path_slots":
                       args.single_slots or "default"},
            "one_by_one": {"ms": round(t_seq, 3), "value": round(samples / (t_seq / 1e3) / 1e6, 3)}}
    line["small_scenes"] = batch_small(args, L, sp, tmp, n, timed)
    conv = None if args.no_convergence else batch_convergence(args, dev, tmp)
    if conv:
        line["time_to_relmse"] = conv
    print(json.dumps(line), flush=True)


def batch_small(args, L, sp, tmp, n, timed, side=128, spp=16):
    """The same scenes at side x side pixels and spp samples per pixel: renders too small to fill the GPU
    alone (side^2 * spp work items against about 1.2 M path slots), batched vs one by one."""
    import torch
    import clovers_gb300 as cg
    from clovers_gb300 import _lib
    dev, opts, films = [], [], []
    for k in range(n):
        dev.append(cg.Scene.from_json(os.path.join(tmp, "batch_%02d.json" % k), side, side).upload())
        opts.append(cg.render_opts(cg.RenderOptions(width=side, height=side, samples=spp, max_depth=DEPTH,
                                                    seed=100 + k)))
        films.append(torch.zeros(side * side * 3, dtype=torch.float64, device="cuda"))
    handles = (ctypes.c_void_p * n)(*[d.handle.value for d in dev])
    optarr = (_lib.RenderOptsC * n)(*opts)
    ptrs = (ctypes.c_void_p * n)(*[f.data_ptr() for f in films])

    def batched():
        _lib.check(L.clv_render_batch(handles, optarr, ptrs, n, sp))

    def one_by_one():
        for k in range(n):
            _lib.check(L.clv_render_device(dev[k].handle, ctypes.byref(optarr[k]), films[k].data_ptr(), sp))

    for _ in range(args.warmup):
        batched()
        one_by_one()
    t_batch = min(timed(batched) for _ in range(args.steps))
    t_seq = min(timed(one_by_one) for _ in range(args.steps))
    samples = n * side * side * spp
    return {"workload": "the same %d scenes at %dx%d, %d spp" % (n, side, side, spp), "samples_per_step": samples,
            "batched": {"ms": round(t_batch, 3), "value": round(samples / (t_batch / 1e3) / 1e6, 3)},
            "one_by_one": {"ms": round(t_seq, 3), "value": round(samples / (t_seq / 1e3) / 1e6, 3)}}


def batch_convergence(args, dev, tmp):
    """GPU time to relMSE <= 1e-3 per scene for the batch scenes with a golden reference
    (tests/golden/batch_ref.npz: the oracle in double precision, 65,536 spp, a stratified pixel subset):
    progressive passes of --chunk-spp, (a) the scenes rendered together by clv_render_batch (a scene leaves
    the batch once it has converged), (b) each scene alone by clv_render_device, (c) each scene alone with
    the online-trained guide (clv_render_guided)."""
    import torch
    import clovers_gb300 as cg
    from clovers_gb300 import _lib
    gpath = os.path.join(ROOT, "tests", "golden", "batch_ref.npz")
    if not os.path.exists(gpath):
        return None
    g = np.load(gpath)
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    ids = [int(k) for k in g["scenes"]]
    size = {k: tuple(int(v) for v in g["s%d_size" % k]) for k in ids}
    films = {k: torch.zeros(size[k][0] * size[k][1] * 3, dtype=torch.float64, device="cuda") for k in ids}
    sets = {k: (torch.as_tensor(g["s%d_pixels" % k].astype(np.int64), device="cuda"), g["s%d_mean" % k]) for k in ids}
    chunk, target = args.chunk_spp, 1e-3

    def relmse(k, total_spp):
        w, h = size[k]
        img = (films[k].view(h * w, 3)[sets[k][0]] / total_spp).cpu().numpy()
        ref = sets[k][1]
        return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))

    def opts(k, offset, seed):
        w, h = size[k]
        o = cg.render_opts(cg.RenderOptions(width=w, height=h, samples=chunk, max_depth=DEPTH, seed=seed))
        o.sample_offset = offset
        return o

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    max_pass = max(1, args.max_spp // chunk)
    seed = SEED + 3000
    # (a) together
    for f in films.values():
        f.zero_()
    todo, t, res_batch, npass = list(ids), 0.0, {}, 0
    while todo and npass < max_pass:
        n = len(todo)
        handles = (ctypes.c_void_p * n)(*[dev[k].handle.value for k in todo])
        optarr = (_lib.RenderOptsC * n)(*[opts(k, npass * chunk, seed + k) for k in todo])
        ptrs = (ctypes.c_void_p * n)(*[films[k].data_ptr() for k in todo])
        t += timed(lambda: _lib.check(L.clv_render_batch(handles, optarr, ptrs, n, sp)))
        npass += 1
        for k in list(todo):
            e = relmse(k, npass * chunk)
            if e <= target:
                res_batch[k] = {"gpu_ms": round(t, 2), "spp": npass * chunk, "relmse": e}
                todo.remove(k)
    for k in todo:
        res_batch[k] = {"gpu_ms": None, "spp": npass * chunk, "reached": False}
    t_batch_all = t
    # (a') together, guided: one guide for all scenes, trained online on their records
    res_gbatch, t_gbatch_all = {}, None
    if args.guided:
        for f in films.values():
            f.zero_()
        guide = cg.Guide(seed=args.guide_seed if args.guide_seed is not None else 7, learning_rate=args.guide_lr)
        todo, t, npass, total = list(ids), 0.0, 0, 0
        while todo and total < args.max_spp:
            training = npass < args.guide_passes
            nspp = args.guide_pass_spp if training else chunk
            n = len(todo)
            handles = (ctypes.c_void_p * n)(*[dev[k].handle.value for k in todo])
            ol = []
            for k in todo:
                w, h = size[k]
                o = cg.render_opts(cg.RenderOptions(width=w, height=h, samples=nspp, max_depth=DEPTH, seed=seed + k))
                o.sample_offset = total
                ol.append(o)
            optarr = (_lib.RenderOptsC * n)(*ol)
            ptrs = (ctypes.c_void_p * n)(*[films[k].data_ptr() for k in todo])
            alpha = 0.0 if npass == 0 else args.guide_alpha

            def gstep():
                _lib.check(L.clv_render_batch_guided(handles, optarr, ptrs, n, guide.handle, alpha, sp))
                if training:
                    _lib.check(L.clv_guide_train(guide.handle, args.guide_steps, args.guide_batch, None, sp))
            t += timed(gstep)
            npass += 1
            total += nspp
            for k in list(todo):
                e = relmse(k, total)
                if e <= target:
                    res_gbatch[k] = {"gpu_ms": round(t, 2), "spp": total, "relmse": e}
                    todo.remove(k)
        for k in todo:
            res_gbatch[k] = {"gpu_ms": None, "spp": total, "reached": False}
        t_gbatch_all = t
    # (b) alone, plain; (c) alone, guided
    res_alone, res_guided = {}, {}
    for k in ids:
        films[k].zero_()
        t, npass, e = 0.0, 0, None
        while npass < max_pass:
            o = opts(k, npass * chunk, seed + k)
            t += timed(lambda: _lib.check(L.clv_render_device(dev[k].handle, ctypes.byref(o), films[k].data_ptr(),
                                                              sp)))
            npass += 1
            e = relmse(k, npass * chunk)
            if e <= target:
                break
        res_alone[k] = {"gpu_ms": round(t, 2), "spp": npass * chunk, "relmse": e, "reached": e <= target}
        if args.guided:
            films[k].zero_()
            guide = cg.Guide(seed=args.guide_seed if args.guide_seed is not None else 7, learning_rate=args.guide_lr)
            t, npass, total, e = 0.0, 0, 0, None
            while total < args.max_spp:
                training = npass < args.guide_passes
                nspp = args.guide_pass_spp if training else chunk
                w, h = size[k]
                o = cg.render_opts(cg.RenderOptions(width=w, height=h, samples=nspp, max_depth=DEPTH, seed=seed + k))
                o.sample_offset = total
                alpha = 0.0 if npass == 0 else args.guide_alpha

                def step():
                    _lib.check(L.clv_render_guided(dev[k].handle, ctypes.byref(o), guide.handle, alpha,
                                                   films[k].data_ptr(), sp))
                    if training:
                        _lib.check(L.clv_guide_train(guide.handle, args.guide_steps, args.guide_batch, None, sp))
                t += timed(step)
                npass += 1
                total += nspp
                e = relmse(k, total)
                if e <= target:
                    break
            res_guided[k] = {"gpu_ms": round(t, 2), "spp": total, "relmse": e, "reached": e <= target}
    out = {"target": target, "reference": "oracle (f64), 65536 spp, stratified pixel subsets (tests/golden/batch_ref.npz)",
           "pass_spp": chunk, "scenes": ids, "batched": {str(k): v for k, v in res_batch.items()},
           "batched_total_ms": round(t_batch_all, 2), "alone": {str(k): v for k, v in res_alone.items()},
           "alone_total_ms": round(sum(v["gpu_ms"] for v in res_alone.values()), 2)}
    if res_guided:
        out["guided_alone"] = {str(k): v for k, v in res_guided.items()}
        out["guided_alone_total_ms"] = round(sum(v["gpu_ms"] for v in res_guided.values()), 2)
    if res_gbatch:
        out["guided_batched"] = {str(k): v for k, v in res_gbatch.items()}
        out["guided_batched_total_ms"] = round(t_gbatch_all, 2)
        out["guided_estimator"] = ("alpha %.2f of Lambertian bounces from one vMF-mixture MLP shared by the scenes "
                                   "(positions normalised to each scene's box); %d training passes of %d spp, %d "
                                   "Adam steps of %d records after each" % (args.guide_alpha, args.guide_passes,
                                                                            args.guide_pass_spp, args.guide_steps,
                                                                            args.guide_batch))
    return out


def run_config(args):
    """One workload of the configuration list: Msamples/s, and for workloads with a golden
    oracle crop (tests/golden), the GPU time until the crop's relMSE reaches 1e-3."""
    import torch
    import clovers_gb300 as cg
    from clovers_gb300 import _lib
    builder, w, h, spp, depth, desc = CONFIGS[args.config]
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    tmp = tempfile.mkdtemp()
    path = config_scene_file(builder, tmp)
    t0 = time.perf_counter()
    host = cg.Scene.from_json(path, w, h)
    build_s = time.perf_counter() - t0
    d = host.upload()
    film = torch.zeros(w * h * 3, dtype=torch.float64, device="cuda")
    tune = None
    if not args.no_autotune:
        # wavefront shape search before any timing, on the workload's own samples per pixel where that is
        # at most 2^27 samples per candidate (a shorter render is mostly wavefront tail and favours small
        # shapes), else on 2^27 samples' worth
        t0 = time.perf_counter()
        tune_spp = max(1, min(spp, (1 << 27) // (w * h)))
        res = d.autotune(cg.RenderOptions(width=w, height=h, samples=tune_spp, max_depth=depth, seed=SEED + 7),
                         stream=sp)
        best = min(res, key=lambda r: r[4])
        tune = {"path_slots": best[0], "shade_blocks_per_sm": best[1], "warp_appends": best[2],
                "diffuse_blocks_per_sm": best[3], "candidates": len(res), "tuning_spp": tune_spp,
                "tuning_s": round(time.perf_counter() - t0, 3)}

    def render(n_spp, offset, seed=SEED):
        o = cg.render_opts(cg.RenderOptions(width=w, height=h, samples=n_spp, max_depth=depth, seed=seed))
        o.sample_offset = offset
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _lib.check(L.clv_render_device(d.handle, ctypes.byref(o), film.data_ptr(), sp))
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    for k in range(args.warmup):
        film.zero_()
        render(max(1, spp // 16), 10**7 + k * spp)
    ms = []
    for k in range(0 if args.guided_only else args.steps):
        film.zero_()
        ms.append(render(spp, k * spp))
    ms_step = sum(ms) / len(ms) if ms else float("nan")
    line = {"metric": "Msamples/s", "value": round(w * h * spp / (ms_step / 1e3) / 1e6, 3) if ms else None,
            "unit": "Msamples/s",
            "n_gpus": 1, "steps": len(ms), "warmup": args.warmup, "ms_per_step": round(ms_step, 3) if ms else None,
            "higher_is_better": True, "dtype": "f32", "data": "synthetic (seeded generator, reference scene format)",
            "config": {"workload": desc, "scene_load_and_bvh_s": round(build_s, 3), "objects": host.info()["objects"],
                       "autotune": tune}}
    gold = GOLDEN.get(args.config)
    if gold:
        plain, guided = time_to_relmse(args, gold, d, w, h, depth, film, stream, render, args.guided)
        if plain:
            line["time_to_relmse"] = plain
        if guided:
            line["time_to_relmse_guided"] = guided
    print(json.dumps(line), flush=True)


def golden_sets(gold, w, h):
    """The golden references of a workload (tests/golden/<gold>_ref.npz: the oracle in double precision at
    65,536 spp): {set name: (buffer pixel indices, reference means)} for the 64x64 crop and the
    stratified whole-image subset, and a description."""
    gpath = os.path.join(ROOT, "tests", "golden", "%s_ref.npz" % gold)
    if not os.path.exists(gpath):
        return None, None
    g = np.load(gpath)
    x0, r0, x1, r1 = [int(v) for v in g["window"]]
    rr, xx = np.meshgrid(np.arange(r0, r1), np.arange(x0, x1), indexing="ij")
    sets = {"crop": ((rr * w + xx).reshape(-1), g["mean"])}
    if "sub_mean" in g.files:
        sets["subset"] = (g["sub_pixels"].astype(np.int64), g["sub_mean"])
    where = "oracle (%s), %d spp: crop %s of %dx%d, subset = centre pixel of every %dx%d cell (%d pixels); " \
            "tests/golden/%s_ref.npz" % (str(g["precision"]) if "precision" in g.files else "f32", int(g["spp"]),
                                         [x0, r0, x1, r1], w, h, int(g["sub_stride"]) if "sub_stride" in g.files else 0,
                                         int(g["sub_stride"]) if "sub_stride" in g.files else 0,
                                         len(sets["subset"][0]) if "subset" in sets else 0, gold)
    return sets, where


def progressive(render_pass, film, sets, w, h, max_spp, target=1e-3):
    """Adds passes (render_pass(total_spp) -> (spp added, GPU ms)) to the film until the relMSE of every
    golden set is <= target; returns per set the GPU time and spp at which it first got there."""
    import torch
    idx = {k: torch.as_tensor(v[0], device=film.device) for k, v in sets.items()}
    total_ms, total_spp = 0.0, 0
    first, last = {}, {}
    while total_spp < max_spp and len(first) < len(sets):
        n, ms = render_pass(total_spp)
        total_ms += ms
        total_spp += n
        f = film.view(h * w, 3)
        for k, (_, ref) in sets.items():
            img = (f[idx[k]] / total_spp).cpu().numpy()
            last[k] = float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))
            if k not in first and last[k] <= target:
                first[k] = (total_ms, total_spp)
    out = {}
    for k in sets:
        out[k] = {"reached": k in first, "gpu_ms": round(first[k][0], 2) if k in first else round(total_ms, 2),
                  "spp": first[k][1] if k in first else total_spp, "relmse_last": last.get(k)}
    return out, total_ms


def time_to_relmse(args, gold, d, w, h, depth, film, stream, render, guided):
    """GPU time until the relMSE against the golden references (crop and whole-image subset) reaches 1e-3:
    progressive passes of --chunk-spp with the plain estimator, and (guided) with the online-trained guide."""
    sets, where = golden_sets(gold, w, h)
    if sets is None:
        return None, None
    film.zero_()

    def plain_pass(total_spp):
        return args.chunk_spp, render(args.chunk_spp, total_spp, seed=SEED + 1000)

    res, _ = ({}, 0) if getattr(args, "guided_only", False) else progressive(plain_pass, film, sets, w, h,
                                                                               args.max_spp)
    crop = res.get("crop", {})
    plain = {"target": 1e-3, "reached": crop.get("reached", False), "gpu_ms": crop.get("gpu_ms"),
             "spp": crop.get("spp"), "relmse": crop.get("relmse_last"), "sets": res, "reference": where,
             "epsilon": 1e-2, "estimator": "plain (BSDF + light mixture MIS)"}
    gres = None
    if guided:  # one guided run per guide seed; the run of median GPU time stands for all
        seeds = [args.guide_seed] if args.guide_seed is not None else [int(x) for x in args.guide_seeds.split(",")]
        runs = []
        for sd in seeds:
            r = run_guided(args, d, w, h, depth, film, stream, sets, where, sd)
            r["guide_seed"] = sd
            runs.append(r)
        runs.sort(key=lambda r: r["gpu_ms"] if r["reached"] else float("inf"))
        gres = dict(runs[(len(runs) - 1) // 2])
        gres["runs"] = [{"guide_seed": r["guide_seed"], "gpu_ms": r["gpu_ms"], "spp": r["spp"], "reached": r["reached"],
                         "subset_gpu_ms": r["sets"].get("subset", {}).get("gpu_ms")}
                        for r in sorted(runs, key=lambda r: r["guide_seed"])]
        gres["statistic"] = "median of %d guide seeds (the time to the target varies with the seed)" % len(runs)
        if plain["gpu_ms"]:
            gres["vs_plain_time"] = round(gres["gpu_ms"] / plain["gpu_ms"], 4)
        if "subset" in res and res["subset"]["reached"]:
            sub = sorted(r["sets"]["subset"]["gpu_ms"] for r in runs if r["sets"].get("subset", {}).get("reached"))
            if sub:
                gres["subset_median_gpu_ms"] = sub[(len(sub) - 1) // 2]
                gres["subset_vs_plain_time"] = round(gres["subset_median_gpu_ms"] / res["subset"]["gpu_ms"], 4)
    return plain, gres


def guided_vs_plain(args):
    """The dispersive-caustic workload (prism + sphere, 1024x1024, depth 16):
    GPU time to relMSE 1e-3 of the golden crop, plain and guided."""
    import torch
    import clovers_gb300 as cg
    from clovers_gb300 import _lib
    builder, w, h, _, depth, desc = CONFIGS["c4"]
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    tmp = tempfile.mkdtemp()
    d = cg.Scene.from_json(config_scene_file(builder, tmp), w, h).upload()
    film = torch.zeros(w * h * 3, dtype=torch.float64, device="cuda")

    def render(n_spp, offset, seed=SEED):
        o = cg.render_opts(cg.RenderOptions(width=w, height=h, samples=n_spp, max_depth=depth, seed=seed))
        o.sample_offset = offset
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        _lib.check(L.clv_render_device(d.handle, ctypes.byref(o), film.data_ptr(), stream.cuda_stream))
        e1.record(stream)
        e1.synchronize()
        return e0.elapsed_time(e1)

    render(16, 10**7)  # warm-up
    plain, guided = time_to_relmse(args, "prism", d, w, h, depth, film, stream, render, True)
    return {"workload": "dispersive prism + glass sphere, 1024x1024, depth 16 (C4)", "plain": plain,
            "guided": guided, "guided_vs_plain_time": guided["vs_plain_time"] if guided else None}


def run_guided(args, d, w, h, depth, film, stream, sets, where, guide_seed):
    """Progressive guided render until the relMSE of every golden set reaches 1e-3: training
    passes of --guide-pass-spp samples per pixel (the first with alpha 0), each followed by
    --guide-steps Adam steps on its records, then passes of --chunk-spp with the trained guide.
    Every pass adds to the film (all are unbiased); the GPU time includes rendering and training."""
    import torch
    import clovers_gb300 as cg
    from clovers_gb300 import _lib
    L = _lib.lib()
    sp = stream.cuda_stream
    guide = cg.Guide(seed=guide_seed, learning_rate=args.guide_lr)
    film.zero_()
    state = {"k": 0, "train_ms": 0.0}

    def guided_pass(total_spp):
        k = state["k"]
        training = k < args.guide_passes
        n = args.guide_pass_spp if training else args.chunk_spp
        alpha = 0.0 if k == 0 else args.guide_alpha
        o = cg.render_opts(cg.RenderOptions(width=w, height=h, samples=n, max_depth=depth, seed=SEED + 2000))
        o.sample_offset = total_spp
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record(stream)
        _lib.check(L.clv_render_guided(d.handle, ctypes.byref(o), guide.handle, alpha, film.data_ptr(), sp))
        e1.record(stream)
        if training:
            _lib.check(L.clv_guide_train(guide.handle, args.guide_steps, args.guide_batch, None, sp))
        e2.record(stream)
        e2.synchronize()
        state["k"] = k + 1
        state["train_ms"] += e1.elapsed_time(e2)
        return n, e0.elapsed_time(e2)

    res, _ = progressive(guided_pass, film, sets, w, h, args.max_spp)
    if guide.status():
        raise RuntimeError("guide kernels reported an error")
    crop = res["crop"]
    return {"target": 1e-3, "reached": crop["reached"], "gpu_ms": crop["gpu_ms"],
            "train_ms": round(state["train_ms"], 2), "spp": crop["spp"], "relmse": crop["relmse_last"],
            "sets": res, "reference": where,
            "estimator": "guided: alpha %.2f of Lambertian bounces from the vMF-mixture MLP (one-sample MIS with "
                         "the plain mixture); %d training passes of %d spp, %d Adam steps of %d records each" % (
                             args.guide_alpha, args.guide_passes, args.guide_pass_spp, args.guide_steps,
                             args.guide_batch)}


def main():
    global W_IMG, H_IMG, SPP, RAYS, TRIS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-spp", type=int, default=16, help="samples per pixel of each reference-arm step")
    ap.add_argument("--cpu-baseline-spp", type=int, default=64, help="samples per pixel of the CPU baseline leg")
    ap.add_argument("--no-traversal", action="store_true", help="skip the ray-cast section")
    ap.add_argument("--no-render", action="store_true", help="skip the render section (ray casts only)")
    ap.add_argument("--size", type=int, default=W_IMG, help="image width = height (reduced cases for profiling)")
    ap.add_argument("--spp", type=int, default=SPP, help="samples per pixel (reduced cases for profiling)")
    ap.add_argument("--rays", type=int, default=RAYS, help="ray count of the ray-cast section")
    ap.add_argument("--tris", type=int, default=TRIS, help="triangle count of the ray-cast section")
    ap.add_argument("--config", choices=sorted(CONFIGS), help="measure another workload of the configuration list")
    ap.add_argument("--chunk-spp", type=int, default=32, help="samples per pixel per progressive pass (relMSE)")
    ap.add_argument("--max-spp", type=int, default=8192, help="cap of the progressive relMSE measurement")
    ap.add_argument("--batch", action="store_true", help="measure the batched multi-scene workload")
    ap.add_argument("--batch-scenes", type=int, default=64)
    ap.add_argument("--batch-slots", type=int, default=0,
                    help="paths in flight of the batched render (0: clv_render_batch's default)")
    ap.add_argument("--single-slots", type=int, default=0,
                    help="paths in flight of each one-by-one render (0: clv_render_device's default)")
    ap.add_argument("--no-convergence", action="store_true",
                    help="with --batch: skip the per-scene time to relMSE 1e-3 (launch lists of the timed renders)")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline legs")
    ap.add_argument("--no-parity", action="store_true",
                    help="skip the check of every timed ray cast against the oracle (untimed, about 40 s of CPU)")
    ap.add_argument("--guided", action="store_true", help="with --config: also the guided time to relMSE 1e-3")
    ap.add_argument("--no-guided", action="store_true", help="skip the guided-vs-plain section of the default run")
    ap.add_argument("--no-autotune", action="store_true", help="skip the wavefront shape search before the timed render")
    ap.add_argument("--guided-only", action="store_true",
                    help="with --config --guided: only the guided passes (short case for profiling)")
    ap.add_argument("--guide-alpha", type=float, default=0.5)
    ap.add_argument("--guide-passes", type=int, default=32)
    ap.add_argument("--guide-pass-spp", type=int, default=4)
    ap.add_argument("--guide-steps", type=int, default=64)
    ap.add_argument("--guide-batch", type=int, default=32768)
    ap.add_argument("--guide-lr", type=float, default=5e-3)
    ap.add_argument("--guide-seed", type=int, default=None, help="one guided run with this guide seed")
    ap.add_argument("--guide-seeds", default="7,8,9,10,11", help="guide seeds of the guided runs (median reported)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    W_IMG = H_IMG = args.size
    SPP, RAYS, TRIS = args.spp, args.rays, args.tris
    if args.config:
        run_config(args)
        return
    if args.batch:
        run_batch(args)
        return
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
        return

    import torch
    import clovers_gb300 as cg
    from clovers_gb300 import _lib, scenes
    from clovers_gb300.distributed import reduce_film

    torch.cuda.set_device(local)
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    sp = stream.cuda_stream
    hbm_peak, peak_kind = measured_peaks()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2

    path = box_scene_file()
    gpu_index = os.environ.get("CUDA_VISIBLE_DEVICES", str(local)).split(",")[local if world > 1 else 0]
    traffic = ncu_traffic()
    if args.no_render:
        line = {"metric": "Grays/s", "unit": "Grays/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "higher_is_better": True, "config": {"workload": "ray casts only"}}
    else:
        # ---------------------------------------------------------------- render
        host_scene = cg.Scene.from_json(path, W_IMG, H_IMG)
        dscene = host_scene.upload()
        npix = W_IMG * H_IMG
        film = torch.zeros(npix * 3, dtype=torch.float64, device="cuda")

        def opts_for(step):
            o = cg.render_opts(cg.RenderOptions(width=W_IMG, height=H_IMG, samples=SPP, max_depth=DEPTH, seed=SEED))
            o.sample_offset = (rank * 1000003 + step) * SPP  # weak scaling: every rank renders its own samples
            return o

        tune = None
        if not args.no_autotune:  # one-time shape search on a shorter render of the same scene, before the timed region
            t0 = time.perf_counter()
            res = dscene.autotune(cg.RenderOptions(width=W_IMG, height=H_IMG, samples=max(1, SPP // 4),
                                                   max_depth=DEPTH, seed=SEED + 7), stream=sp)
            best = min(res, key=lambda r: r[4])
            tune = {"path_slots": best[0], "shade_blocks_per_sm": best[1], "warp_appends": best[2],
                    "diffuse_blocks_per_sm": best[3], "candidates": len(res),
                    "tuning_s": round(time.perf_counter() - t0, 3)}
        for w in range(args.warmup):
            film.zero_()
            _lib.check(L.clv_render_device(dscene.handle, ctypes.byref(opts_for(10**6 + w)), film.data_ptr(), sp))
        torch.cuda.synchronize()
        launches0 = L.clv_kernel_launches()
        step_ms = []
        barrier(world)
        torch.cuda.synchronize()
        with ClockSampler(gpu_index) as clocks:
            wall0 = time.perf_counter()
            for k in range(args.steps):
                film.zero_()
                flush.zero_()  # L2 flush between timed steps
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                _lib.check(L.clv_render_device(dscene.handle, ctypes.byref(opts_for(k)), film.data_ptr(), sp))
                if world > 1:  # one image of all ranks' samples: the film sum (clovers_gb300.distributed)
                    reduce_film(film)
                e1.record(stream)
                e1.synchronize()
                step_ms.append(e0.elapsed_time(e1))
            torch.cuda.synchronize()
            wall = time.perf_counter() - wall0
        barrier(world)
        launches = L.clv_kernel_launches() - launches0
        ms_step = all_max(world, sum(step_ms) / len(step_ms))
        samples_step = npix * SPP
        value = world * samples_step / (ms_step / 1e3) / 1e6

        # e2e: through the host-buffer C ABI (scene upload + render + image download), every step
        xyz = np.empty((npix, 3), np.float32)
        host_opts = opts_for(0)
        if tune:  # a fresh upload each step: carry the tuned pool size over
            host_opts.path_slots = tune["path_slots"]
        e2e_times = []
        st = _lib.StatsC()
        h2d = 0
        for k in range(args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            d2 = host_scene.upload()
            host_opts.sample_offset = (rank * 1000003 + 5000 + k) * SPP
            _lib.check(L.clv_render(d2.handle, ctypes.byref(host_opts), xyz.ctypes.data, ctypes.byref(st)))
            e2e_times.append(time.perf_counter() - t0)
            d2.close()
        info = host_scene.info()
        # bytes the upload copies (nodes, records, materials, spectral tables, illuminants, CMF)
        h2d = (info["nodes"] * 64 + info["triangles"] * 64 + info["quads"] * 64 + info["spheres"] * 16 +
               info["compound"] * 64 + info["materials"] * 112 + 38 * 400 * 4 + 400 * 12)
        e2e_s = all_max(world, sum(e2e_times) / len(e2e_times))
        e2e_value = world * samples_step / e2e_s / 1e6

        # profiling pass (untimed): per-kernel device time and traversal counts for the roofline
        prof = _lib.RenderProfileC()
        film.zero_()
        _lib.check(L.clv_render_profile_run(dscene.handle, ctypes.byref(opts_for(777)), film.data_ptr(), sp,
                                            ctypes.byref(prof)))
        torch.cuda.synchronize()
        segs = prof.path_segments
        # algorithmic bytes per closest-hit query (one per bounce of a live path):
        #   intersect: reads meta + origin + direction (48 B), writes the hit (16 B) and a queue entry (4 B),
        #              and fetches one 64-B node per BVHNode::hit call and one 64-B record per primitive test;
        #   shade (specular/diffuse/finish): reads the queue entry (4 B), path state + hit (88 B) and writes
        #              the next state (64 B) per query; per sample 80 B read at the end, 24 B of film and
        #              72 B for the regenerated path.
        isect_bytes = segs * (48 + 16 + 4) + 64 * (prof.node_visits + prof.prim_tests)
        shade_bytes = segs * (4 + 88 + 64) + prof.paths * (80 + 24 + 72)
        kernels = {"wf_intersect": (prof.ms_intersect, isect_bytes, prof.intersect_launches),
                   "wf_shade": (prof.ms_shade, shade_bytes, prof.shade_launches)}
        dom = max(kernels, key=lambda k: kernels[k][0])
        d_ms, d_bytes, d_launches = kernels[dom]
        # captured per-launch DRAM bytes, scaled to this render's path-slot count (one slot per query)
        dom_traffic = traffic.get(dom + ".bytes_per_launch")
        if dom_traffic is not None and traffic.get(dom + ".slots"):
            slots = tune["path_slots"] if tune else torch.cuda.get_device_properties(0).multi_processor_count * 8192
            dom_traffic = round(dom_traffic * slots / traffic[dom + ".slots"])
        achieved = d_bytes / (d_ms / 1e3) / 1e9
        roofline = {"kernel": dom, "bound": "hbm", "achieved": round(achieved, 1), "peak": hbm_peak, "unit": "GB/s",
                    "frac": round(achieved / hbm_peak, 4), "peak_kind": peak_kind,
                    "traffic": dom_traffic,
                    "algorithmic_bytes_per_launch": round(d_bytes / max(1, d_launches)),
                    "kernel_ms_per_step": {k: round(v[0], 3) for k, v in kernels.items()},
                    "path_segments": segs, "node_visits": prof.node_visits, "prim_tests": prof.prim_tests}

        line = {
            "metric": "Msamples/s", "value": round(value, 3), "unit": "Msamples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_step, 3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded enclosed-box scene in the reference's scene format)",
            "config": {"workload": "enclosed box %dx%d, %d spp, depth %d (wavefront engine)" % (W_IMG, H_IMG, SPP, DEPTH),
                       "samples_per_step": samples_step, "l2": "flushed between steps (256 MiB write)",
                       "parallelism": "sample ranges per GPU + film sum" if world > 1 else "single GPU",
                       "wall_s_timed_loop": round(wall, 3),
                       "autotune": tune},
            "e2e": {"value": round(e2e_value, 3), "unit": "Msamples/s", "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(npix * 3 * 4)},
            "gpu_launches": int(launches),
            "roofline": roofline,
            "clocks": clocks.summary(),
        }

    # ------------------------------------------------------------- ray casts
    if not args.no_traversal:
        v, idx = scenes.triangle_soup(TRIS, seed=2)
        mesh = cg.Scene.from_mesh(v, idx)
        dm = mesh.upload()
        rays_h = scenes.random_rays(RAYS, seed=3)
        rays = torch.from_numpy(rays_h).cuda()
        prim = torch.empty(RAYS, dtype=torch.int32, device="cuda")
        tt = torch.empty(RAYS, dtype=torch.float32, device="cuda")
        for _ in range(args.warmup):
            _lib.check(L.clv_raycast_device(dm.handle, rays.data_ptr(), RAYS, prim.data_ptr(), tt.data_ptr(),
                                            None, None, sp))
        ms = []
        torch.cuda.synchronize()
        for _ in range(args.steps):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            _lib.check(L.clv_raycast_device(dm.handle, rays.data_ptr(), RAYS, prim.data_ptr(), tt.data_ptr(),
                                            None, None, sp))
            e1.record(stream)
            e1.synchronize()
            ms.append(e0.elapsed_time(e1))
        r_ms = all_max(world, sum(ms) / len(ms))
        nodes = torch.empty(RAYS, dtype=torch.int32, device="cuda")
        tests = torch.empty(RAYS, dtype=torch.int32, device="cuda")
        _lib.check(L.clv_raycast_device(dm.handle, rays.data_ptr(), RAYS, prim.data_ptr(), tt.data_ptr(),
                                        nodes.data_ptr(), tests.data_ptr(), sp))
        torch.cuda.synchronize()
        nv = int(nodes.sum(dtype=torch.int64).item())
        pt = int(tests.sum(dtype=torch.int64).item())
        rbytes = RAYS * (32 + 8) + 64 * (nv + pt)
        r_ach = rbytes / (r_ms / 1e3) / 1e9
        # e2e ray casts: host rays in, host ids/distances out (host output arrays reused, as a caller
        # casting batch after batch would; one untimed call first, like the device-side warm-up)
        out_h = (np.empty(RAYS, np.uint32), np.empty(RAYS, np.float32))
        cg.raycast(dm, rays_h, out=out_h)
        r_e2e_all = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            cg.raycast(dm, rays_h, out=out_h)
            r_e2e_all.append(time.perf_counter() - t0)
        r_e2e = all_max(world, sum(r_e2e_all) / len(r_e2e_all) * 1e3) / 1e3
        trav = {"workload": "%d random rays vs %d random triangles (SAH BVH, closest hit)" % (RAYS, TRIS),
                "metric": "Grays/s", "value": round(RAYS / (r_ms / 1e3) / 1e9, 4), "ms_per_step": round(r_ms, 3),
                "e2e": {"value": round(RAYS / r_e2e / 1e9, 4), "unit": "Grays/s", "h2d_bytes_per_step": RAYS * 32,
                        "d2h_bytes_per_step": RAYS * 8},
                "nodes_per_ray": round(nv / RAYS, 2), "prims_per_ray": round(pt / RAYS, 2),
                "roofline": {"kernel": "raycast_persist_kernel", "bound": "hbm", "achieved": round(r_ach, 1),
                             "peak": hbm_peak, "unit": "GB/s", "frac": round(r_ach / hbm_peak, 4),
                             "traffic": traffic.get("raycast_persist_kernel.bytes_per_launch"),
                             "algorithmic_bytes_per_launch": int(rbytes)}}
        if rank == 0 and world == 1 and (not args.no_cpu or not args.no_parity):
            import oracle
            t0 = time.perf_counter()
            om = oracle.Scene.from_mesh(v, idx)  # the oracle builds its own SAH tree over the same triangles
            build_s = time.perf_counter() - t0
            threads = os.cpu_count() or 1
            if not args.no_cpu:
                n_cpu = 1 << 17
                t0 = time.perf_counter()
                om.raycast(rays_h[:n_cpu], threads=threads)
                el = time.perf_counter() - t0
                n1 = 1 << 13
                t0 = time.perf_counter()
                om.raycast(rays_h[:n1], threads=1)
                el1 = time.perf_counter() - t0
                trav["cpu_baseline"] = {"value": round(n_cpu / el / 1e9, 6), "unit": "Grays/s", "cores": threads,
                                        "kind": "port", "sample": "first %d of the 2^24 rays (%.2f s)" % (n_cpu, el),
                                        "one_core": {"value": round(n1 / el1 / 1e9, 7), "unit": "Grays/s",
                                                     "sample": "first %d rays (%.2f s)" % (n1, el1)}}
            if not args.no_parity:
                # every ray of the timed workload against the oracle: hit ids and distance bits
                gp = prim.cpu().numpy().view(np.uint32)
                gt = tt.cpu().numpy()
                t0 = time.perf_counter()
                op, ot = om.raycast(rays_h, threads=threads)
                cast_s = time.perf_counter() - t0
                hit = op != 0xFFFFFFFF
                same_id = gp == op
                both = hit & same_id
                ulp = np.abs(gt[both].view(np.int32).astype(np.int64) - ot[both].view(np.int32).astype(np.int64))
                trav["parity"] = {"rays_checked": int(RAYS), "id_mismatches": int((~same_id).sum()),
                                  "t_mismatches": int((ulp != 0).sum()), "max_t_ulp": int(ulp.max()) if ulp.size else 0,
                                  "hits": int(hit.sum()),
                                  "oracle": "CPU restatement of BVHNode::hit / Triangle::hit over its own SAH build "
                                            "(%.1f s build, %.1f s cast on %d threads)" % (build_s, cast_s, threads)}
        line["traversal"] = trav
        if args.no_render:
            line.update(value=trav["value"], ms_per_step=trav["ms_per_step"])

    if rank == 0 and world == 1 and not args.no_guided and not args.no_render:
        line["time_to_relmse"] = guided_vs_plain(args)
    if rank == 0 and world == 1 and not args.no_cpu and not args.no_render:
        line["cpu_baseline"] = cpu_baseline_render(path, args.cpu_baseline_spp)
    if rank == 0:
        print(json.dumps(line), flush=True)
    os.unlink(path)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
