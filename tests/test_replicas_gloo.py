"""Replica (multi-rank) host logic on CPU with the gloo backend, world size 2."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

from khepri_gb300.replicas import chunk_indices


def test_chunks_are_disjoint_across_ranks_and_steps():
    world, batch, total = 4, 64, 65536
    seen = set()
    for step in range(8):
        for rank in range(world):
            idx = chunk_indices(total, batch, step, rank, world)
            assert len(idx) == batch
            s = set(idx.tolist())
            assert not (s & seen)
            seen |= s


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    from khepri_gb300.replicas import gather_results, max_over_ranks
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = max_over_ranks(1.0 + rank)
    idx = chunk_indices(1000, 10, 3, rank, world)
    allidx = gather_results(idx)
    np.save(os.path.join(out_dir, f"r{rank}.npy"), np.concatenate([[t], allidx.astype(float)]))
    dist.barrier()
    dist.destroy_process_group()


def test_gloo_two_ranks(tmp_path):
    world = 2
    port = 29500 + (os.getpid() % 1000)
    mp.spawn(_worker, args=(world, port, str(tmp_path)), nprocs=world, join=True)
    a = np.load(tmp_path / "r0.npy")
    b = np.load(tmp_path / "r1.npy")
    assert a[0] == 2.0 and b[0] == 2.0  # max over ranks seen by both
    np.testing.assert_array_equal(a[1:], b[1:])
    expect = np.concatenate([chunk_indices(1000, 10, 3, r, world) for r in range(world)])
    np.testing.assert_array_equal(a[1:], expect)
