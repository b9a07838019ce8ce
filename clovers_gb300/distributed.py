"""One render sharded over the ranks of a torch.distributed group (one process
per GPU), and the one exchange the render path has: the sum of the f64 films.

Every (pixel, sample) of the reference's render (clovers-cli/src/draw_cpu.rs:
53-145) is independent, and its random stream depends only on (seed, pixel,
sample index), so rank r renders the sample indices [offset_r, offset_r +
count_r) of the image into its own film and the films of all ranks add up to
the film of the whole render.  shard_samples() splits the sample indices,
reduce_film() sums the films (all_reduce, NCCL between GPUs, gloo between CPU
ranks), draw_distributed() is draw() over a group.  Without an initialised
process group everything runs as one rank.
"""

import ctypes

from ._lib import check, lib


def _world(group=None):
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return 1, 0
    return dist.get_world_size(group), dist.get_rank(group)


def shard_samples(spp, world, rank):
    """(first sample index, number of samples) of `rank` out of `world` for an
    spp-sample render: contiguous ranges, sizes differing by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("rank %d outside a group of %d" % (rank, world))
    base, extra = divmod(int(spp), int(world))
    count = base + (1 if rank < extra else 0)
    return rank * base + min(rank, extra), count


def reduce_film(film, group=None):
    """Sums a film (torch float64 tensor, device or host) over the group, in place."""
    import torch.distributed as dist
    if _world(group)[0] > 1:
        dist.all_reduce(film, op=dist.ReduceOp.SUM, group=group)
    return film


def draw_distributed(global_options, render_options, scene, group=None, sample_offset=0):
    """draw() with the samples split over the group's ranks (each rank on its
    current CUDA device); every rank returns the (height*width, 3) float32
    XYZ(E) means of the whole render."""
    import torch
    del global_options
    world, rank = _world(group)
    first, count = shard_samples(render_options.samples, world, rank)
    w, h = render_options.width, render_options.height
    film = torch.zeros(w * h * 3, dtype=torch.float64, device="cuda")
    if count:
        from . import render_opts
        o = render_opts(render_options, sample_offset=sample_offset + first)
        o.samples = count
        stream = torch.cuda.current_stream().cuda_stream
        check(lib().clv_render_device(scene.handle, ctypes.byref(o), ctypes.c_void_p(film.data_ptr()),
                                      ctypes.c_void_p(stream)))
    reduce_film(film, group)
    return (film / render_options.samples).to(torch.float32).cpu().numpy().reshape(-1, 3)


__all__ = ["shard_samples", "reduce_film", "draw_distributed"]
