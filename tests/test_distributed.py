"""Sample-range sharding and the film sum across ranks (clovers_gb300.distributed),
with real process groups on CPU (gloo, world size 2 and 3): each rank renders its
share of the samples with the oracle, reduce_film adds the films, and the sum
equals the film of one process rendering every sample (same random streams)."""

import os
import socket
import tempfile

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle
from clovers_gb300 import scenes
from clovers_gb300.distributed import reduce_film, shard_samples

W, H, SPP, DEPTH, SEED = 16, 16, 7, 8, 11


def test_shard_samples_cover_every_sample_once():
    for spp in (1, 2, 7, 64, 1000):
        for world in (1, 2, 3, 8):
            ranges = [shard_samples(spp, world, r) for r in range(world)]
            covered = [s for first, n in ranges for s in range(first, first + n)]
            assert covered == list(range(spp))
            assert max(n for _, n in ranges) - min(n for _, n in ranges) <= 1
    with pytest.raises(ValueError):
        shard_samples(8, 2, 2)


def _rank(rank, world, port, path, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    first, count = shard_samples(SPP, world, rank)
    o = oracle.Scene.from_json(path, W, H)
    film = np.zeros((W * H, 3))
    if count:
        # oracle.render renders samples [sample_offset, sample_offset + spp)
        film = o.render(W, H, count, DEPTH, SEED, sample_offset=first, threads=1)
    t = torch.from_numpy(film.reshape(-1).copy())
    reduce_film(t)
    if rank == 0:
        np.save(out, t.numpy())
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [2, 3])
def test_film_sum_over_ranks_equals_one_render(world, box_scene_path):
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "film.npy")
        mp.start_processes(_rank, args=(world, _free_port(), box_scene_path, out), nprocs=world, join=True,
                           start_method="spawn")
        summed = np.load(out).reshape(-1, 3)
    whole = oracle.Scene.from_json(box_scene_path, W, H).render(W, H, SPP, DEPTH, SEED, threads=1)
    assert np.allclose(summed, whole, rtol=1e-12, atol=1e-12)
    assert whole.sum() > 0
