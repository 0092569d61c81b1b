"""Image-parallel sharding: partition properties on one process, and a two-rank gloo
run on CPU (ranks shard, 'image' their share with a stand-in, gather to rank 0)."""
import os
import socket

import numpy as np
import pytest

from emsim_gb300 import shard


def test_partition_covers_and_balances():
    rng = np.random.default_rng(0)
    costs = [shard.image_cost(int(s), n, n) for s, n in zip(rng.integers(20, 80, 50), rng.choice([256, 512], 50))]
    for world in (1, 2, 3, 8):
        parts = shard.partition(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(costs)))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)  # LPT bound
        assert parts == shard.partition(costs, world)  # deterministic
    assert shard.partition([], 4) == [[], [], [], []]
    with pytest.raises(ValueError):
        shard.partition([1.0], 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n_items, result_path):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    costs = [float(1 + (i * 7) % 5) for i in range(n_items)]
    mine = shard.my_share(costs, rank, world)
    local = {i: np.full((4, 4), i, dtype=np.float32) + rank * 0 for i in mine}  # stand-in for images
    out = shard.gather_to_root(local, n_items, rank, world)
    if rank == 0:
        np.save(result_path, np.stack(out))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_gather(tmp_path):
    import torch.multiprocessing as mp
    n_items = 11
    path = str(tmp_path / "gathered.npy")
    mp.start_processes(_worker, args=(2, _free_port(), n_items, path), nprocs=2, start_method="spawn", join=True)
    got = np.load(path)
    assert got.shape == (n_items, 4, 4)
    for i in range(n_items):
        assert (got[i] == i).all()
