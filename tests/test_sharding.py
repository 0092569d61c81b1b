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


def _mols(n):
    from emsim_gb300 import atoms
    rng = np.random.default_rng(3)
    out = []
    for i in range(n):
        extent = 10.0 + 7.0 * (i % 5)  # z extents 10..38 A: 5..19 slices of 2 A
        xyz = (rng.random((50, 3)) * np.array([extent, 20.0, 20.0])).astype(np.float32)
        out.append(atoms.AtomList(np.full(50, 6), xyz, label=f"m{i}"))
    return out


def _pipe_worker(rank, world, port, n_items, out_dir):
    """A real Pipe on a gloo rank: its cost estimate, the partition and the gather run as
    in production; only the device imaging (run_batch) is a stand-in that returns each
    molecule's index as its image."""
    import json

    import torch.distributed as dist

    from emsim_gb300 import pipe, tem
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mols = _mols(n_items)
    rois = [32 if i % 3 else 64 for i in range(n_items)]
    got = []

    def fake_run_batch(self, batch, defocus=None, to_host=False, rois=None):
        assert to_host
        got.extend(int(m.label[1:]) for m in batch)
        return [np.full((r, r), float(m.label[1:]), np.float32) for m, r in zip(batch, rois)]

    pipe.Pipe.run_batch = fake_run_batch
    p = pipe.Pipe(tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3),
                  resolution=1.0, slice_thickness=2.0, roi=64, add_water=False)
    imgs = p.run_sharded(mols, rois=rois)
    with open(os.path.join(out_dir, f"share{rank}.json"), "w") as f:
        json.dump({"share": got, "costs": p.shard_costs(mols, rois), "none": imgs is None}, f)
    if rank == 0:
        np.save(os.path.join(out_dir, "images.npy"), np.array([im.mean() for im in imgs]))
        np.save(os.path.join(out_dir, "sides.npy"), np.array([im.shape[0] for im in imgs]))
    dist.barrier()
    dist.destroy_process_group()


def test_pipe_run_sharded_two_gloo_ranks(tmp_path):
    """Pipe.run_sharded over two gloo ranks: each rank images exactly its cost-balanced
    share (shard.partition of Pipe.shard_costs), and rank 0 receives every image in input
    order; the other rank gets None."""
    import json

    import torch.multiprocessing as mp
    n_items = 13
    mp.start_processes(_pipe_worker, args=(2, _free_port(), n_items, str(tmp_path)), nprocs=2,
                       start_method="spawn", join=True)
    r0 = json.load(open(tmp_path / "share0.json"))
    r1 = json.load(open(tmp_path / "share1.json"))
    parts = shard.partition(r0["costs"], 2)
    assert r0["costs"] == r1["costs"]
    assert sorted(r0["share"]) == parts[0] and sorted(r1["share"]) == parts[1]
    assert sorted(r0["share"] + r1["share"]) == list(range(n_items))
    assert not r0["none"] and r1["none"]
    np.testing.assert_array_equal(np.load(tmp_path / "images.npy"), np.arange(n_items, dtype=np.float32))
    np.testing.assert_array_equal(np.load(tmp_path / "sides.npy"), [32 if i % 3 else 64 for i in range(n_items)])
    # the estimate follows the slice count: 5, 9, 12, 16, 19 slices of 2 A at equal roi
    c = r0["costs"]
    assert c[3] > c[0] and c[4] > c[1]


def test_emsim_round_robin_shards():
    """EMSim(shard=(rank, world)): every rank images the molecules i % world == rank of the
    same source, in order, and the ranks together image every molecule once."""
    from emsim_gb300.simulator import EMSim

    class FakePipe:
        def run(self, mol):
            return np.full(2, float(mol.label[1:]), np.float32)

    mols = _mols(10)
    seen = []
    for rank in range(3):
        got = []
        EMSim(FakePipe(), iter(mols), lambda img, label: got.append(label), shard=(rank, 3)).run()
        assert got == [f"m{i}" for i in range(rank, 10, 3)]
        seen += got
    assert sorted(seen, key=lambda s: int(s[1:])) == [f"m{i}" for i in range(10)]
    with pytest.raises(ValueError):
        EMSim(FakePipe(), iter(mols), print, shard=(2, 2))
