"""Multi-rank host logic on CPU: two gloo ranks, independent point shards.

The opacity path has no exchange step; what N>1 adds is the shard layout and
the max-over-ranks timing reduction.  Both are checked here with the gloo
backend, with the shards' inputs generated by the library's host generator.
"""

import os
import socket

import numpy as np
import pytest

from bns_nurates_gb300 import shards


def test_split_points_cover_exactly():
    for total in (0, 1, 7, 4096, 1000003):
        for world in (1, 2, 3, 8):
            got = [shards.split_points(total, r, world) for r in range(world)]
            assert sum(c for _, c in got) == total
            pos = 0
            for first, count in got:
                assert first == pos
                pos += count
            assert max(c for _, c in got) - min(c for _, c in got) <= 1


def test_rank_points_weak():
    assert shards.rank_points(1000, 0) == (0, 1000)
    assert shards.rank_points(1000, 3) == (3000, 1000)
    with pytest.raises(ValueError):
        shards.split_points(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, per_rank, outdir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bns_nurates_gb300 as bn
    first, count = shards.rank_points(per_rank, rank)
    eos, m1 = bn.synthetic_points(20261203, count, first=first, nthreads=1)
    np.save(os.path.join(outdir, f"eos{rank}.npy"), eos)
    np.save(os.path.join(outdir, f"m1{rank}.npy"), m1)
    # each rank "times" a different value; every rank must see the maximum
    mx = shards.max_over_ranks(1.5 + rank)
    with open(os.path.join(outdir, f"max{rank}.txt"), "w") as f:
        f.write(repr(mx))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shards_and_timing(tmp_path, lib):
    import torch.multiprocessing as mp
    world, per_rank = 2, 2048
    mp.start_processes(_rank_main, args=(world, _free_port(), per_rank, str(tmp_path)),
                       nprocs=world, join=True, start_method="spawn")
    import bns_nurates_gb300 as bn
    eos_all, m1_all = bn.synthetic_points(20261203, world * per_rank, nthreads=1)
    for r in range(world):
        sl = slice(r * per_rank, (r + 1) * per_rank)
        assert np.array_equal(np.load(tmp_path / f"eos{r}.npy"), eos_all[:, sl])
        assert np.array_equal(np.load(tmp_path / f"m1{r}.npy"), m1_all[:, sl])
        assert float((tmp_path / f"max{r}.txt").read_text()) == 1.5 + (world - 1)
