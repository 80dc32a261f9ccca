"""Multi-process host logic on CPU (gloo, world_size 2): the slowest-rank
reduction bench.py uses under torchrun, and the split of a batch of systems
across ranks.  No GPU involved."""
import importlib
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from conftest import PKG_NAME, ROOT


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_dir):
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        batch = importlib.import_module(PKG_NAME + ".batch")
        ic = importlib.import_module(PKG_NAME + ".ic")
        slowest = bench.max_over_ranks(10.0 + rank, dist, torch.device("cpu"))
        sizes = ic.batch_sizes(64)
        mine = batch.shard_systems(sizes, rank, world)
        gathered = [None] * world
        dist.all_gather_object(gathered, mine)
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
            f.write(repr((slowest, gathered)))
    finally:
        dist.destroy_process_group()


def test_gloo_two_ranks(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    ic = importlib.import_module(PKG_NAME + ".ic")
    sizes = ic.batch_sizes(64)
    results = [eval(open(tmp_path / f"rank{r}.txt").read()) for r in range(world)]
    for slowest, gathered in results:
        assert slowest == 10.0 + world - 1
        flat = sorted(s for shard in gathered for s in shard)
        assert flat == list(range(64))
        loads = [sum(sizes[s] ** 2 for s in shard) for shard in gathered]
        assert max(loads) - min(loads) <= max(sizes) ** 2
    assert results[0][1] == results[1][1]


def test_shard_rejects_bad_rank():
    batch = importlib.import_module(PKG_NAME + ".batch")
    with pytest.raises(ValueError):
        batch.shard_systems([10, 20], 2, 2)
