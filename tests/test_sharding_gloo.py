"""Multi-rank path on CPU: world_size-2 gloo process group, the query split and
the max-over-ranks timing reduction used by bench.py under torchrun."""
import os
import socket

import numpy as np
import pytest

from snch_lbvh_gb300.sharding import shard_range


def test_shard_range_partitions_exactly():
    for n in [0, 1, 7, 16_000_000, 16_000_001]:
        for world in [1, 2, 3, 8]:
            parts = [shard_range(n, r, world) for r in range(world)]
            assert parts[0][0] == 0 and parts[-1][1] == n
            assert all(parts[i][1] == parts[i + 1][0] for i in range(world - 1))
            sizes = [e - b for b, e in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle
    from snch_lbvh_gb300 import meshes
    from snch_lbvh_gb300.sharding import max_over_ranks, sum_over_ranks
    v, f = meshes.noisy_icosphere(2, 1.0, 0.01, seed=1)
    pts = meshes.box_queries(v, 1000, 1.2, seed=2)
    b, e = shard_range(len(pts), rank, world)
    tree = oracle.Tree(v, f)
    idx, dist_ = tree.nearest(pts[b:e], nthreads=1)
    t_max = max_over_ranks(float(rank + 1))
    n_sum = sum_over_ranks(float(e - b))
    q.put((rank, b, e, idx, dist_, t_max, n_sum))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_query_split_matches_single_rank():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in range(2)])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from oracle import oracle
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(2, 1.0, 0.01, seed=1)
    pts = meshes.box_queries(v, 1000, 1.2, seed=2)
    idx, dist_ = oracle.Tree(v, f).nearest(pts, nthreads=1)
    got_idx = np.concatenate([r[3] for r in res])
    got_dist = np.concatenate([r[4] for r in res])
    np.testing.assert_array_equal(got_idx, idx)
    np.testing.assert_array_equal(got_dist, dist_)
    assert all(r[5] == 2.0 for r in res)        # max over ranks of (rank + 1)
    assert all(r[6] == 1000.0 for r in res)     # every query answered exactly once
