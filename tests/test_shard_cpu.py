"""Sharding a round over ranks (CPU only): path ranges, per-task counts, and the
round's one exchange (gather + merge on rank 0) over gloo with world size 2."""
import os
import socket

import numpy as np
import pytest

from finite_root_generation_gb300 import shard


def test_shard_range_covers_round():
    for n in (0, 1, 7, 65536, 262143):
        for world in (1, 2, 3, 8):
            spans = [shard.shard_range(n, r, world) for r in range(world)]
            assert sum(c for _, c in spans) == n
            pos = 0
            for first, count in spans:
                assert first == pos
                pos += count
            counts = [c for _, c in spans]
            assert max(counts) - min(counts) <= 1
    with pytest.raises(ValueError):
        shard.shard_range(10, 2, 2)


def test_shard_paths_per_task():
    ppt = [5, 0, 3, 8]
    assert shard.shard_paths_per_task(ppt, 0, 16).tolist() == ppt
    assert shard.shard_paths_per_task(ppt, 4, 5).tolist() == [1, 0, 3, 1]
    assert shard.shard_paths_per_task(ppt, 8, 8).tolist() == [0, 0, 0, 8]
    total = np.zeros(4, np.int64)
    for r in range(3):
        first, count = shard.shard_range(16, r, 3)
        total += shard.shard_paths_per_task(ppt, first, count)
    assert total.tolist() == ppt


def _synthetic_round(rank, n=400):
    """Roots of one rank's shard: its own roots plus copies of rank 0's first roots
    (cross-shard duplicates) and a few within-shard duplicates and failures."""
    rng = np.random.default_rng(1000 + rank)
    roots = rng.normal(size=(n, 21)) + 1j * rng.normal(size=(n, 21))
    shared = np.random.default_rng(1000).normal(size=(20, 21)) + 1j * np.random.default_rng(1000).normal(size=(20, 21))
    roots[:20] = shared + 1e-9  # within dup_tol of rank 0's first roots
    roots[50:55] = roots[60:65]
    codes = np.zeros(n, np.int32)
    codes[100:110] = 3
    return roots, codes


def _worker(rank, world, port, out_path):
    import torch.distributed as dist

    import finite_root_generation_gb300 as frg

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        roots, codes = _synthetic_round(rank)
        coll = frg.Collection(1e-6)
        merged = shard.gather_merge(coll, roots, codes)
        if rank == 0:
            np.savez(out_path, codes=merged, coll=coll.roots())
        else:
            assert merged is None
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_gather_merge_gloo_two_ranks(tmp_path):
    import torch.multiprocessing as mp

    import finite_root_generation_gb300 as frg

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    out = str(tmp_path / "merged.npz")
    mp.start_processes(_worker, args=(2, port, out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    # the single-process round: one merge of the ranks' roots concatenated in rank order
    r0, c0 = _synthetic_round(0)
    r1, c1 = _synthetic_round(1)
    ref = frg.Collection(1e-6)
    ref_codes = ref.merge(np.concatenate([r0, r1]), np.concatenate([c0, c1]))
    assert np.array_equal(got["codes"], ref_codes)
    assert np.array_equal(got["coll"], ref.roots())
    assert (ref_codes == 6).sum() >= 25  # cross-shard and within-shard duplicates were found
