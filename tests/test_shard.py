"""Replica sharding on CPU (gloo, world size 2): a render split by sample
range over two ranks and summed equals the single render; a job list is
covered exactly once.  The per-rank renders use the CPU oracle, so the
test needs no GPU; it checks the sharding and exchange logic the GPU
replicas use."""
import os
import socket

import numpy as np
import pytest

from raytracer_gb300 import shard


def test_sample_range_covers_every_sample_once():
    for spp in (1, 5, 64, 127):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                b, c = shard.sample_range(spp, r, world)
                seen.extend(range(b, b + c))
            assert seen == list(range(spp))
    with pytest.raises(ValueError):
        shard.sample_range(4, 2, 2)


def test_partition_jobs_balances_and_covers():
    costs = [5.0, 1.0, 1.0, 3.0, 2.0, 8.0, 1.0]
    parts = shard.partition_jobs(costs, 3)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(costs)))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) - min(loads) <= max(costs)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, spp, out_dir):
    import torch
    import torch.distributed as dist
    import oracle_lib as O
    from raytracer_gb300 import scenes
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    scene = scenes.cornell_box(16, 12)
    b, c = shard.sample_range(spp, rank, world)
    o = O.OracleScene(scene)
    film = torch.from_numpy(o.render(c, seed=3, sample_begin=b, threads=1))
    shard.reduce_films(film)
    if rank == 0:
        np.save(os.path.join(out_dir, "sum.npy"), film.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sample_split_matches_single_render(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import oracle_lib as O
    from raytracer_gb300 import scenes
    spp = 6
    mp.start_processes(_worker, args=(2, _free_port(), spp, str(tmp_path)), nprocs=2, start_method="spawn")
    summed = np.load(tmp_path / "sum.npy")
    full = O.OracleScene(scenes.cornell_box(16, 12)).render(spp, seed=3, threads=1)
    assert np.array_equal(summed[..., 3], full[..., 3])
    np.testing.assert_allclose(summed[..., :3], full[..., :3], rtol=1e-5, atol=1e-6)
