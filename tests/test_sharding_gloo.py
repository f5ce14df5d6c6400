"""Multi-rank path on CPU: a world_size-2 gloo process group running bench.py's
replica scheme -- every rank answers the whole batch on its own copy of the
scene (queries are independent: no data-path collective) -- and the
max-over-ranks timing reduction bench.py applies under torchrun."""
import os
import socket

import numpy as np


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world), RANK=str(rank),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from oracle import oracle
    from snch_lbvh_gb300 import meshes
    assert bench.dist_env() == (world, rank, rank)
    v, f = meshes.noisy_icosphere(2, 1.0, 0.01, seed=1)
    pts = meshes.box_queries(v, 1000, 1.2, seed=2)
    idx, dist_ = oracle.Tree(v, f).nearest(pts, nthreads=1)
    t_max = bench.max_over_ranks(float(rank + 1))
    q.put((rank, idx, dist_, t_max))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_replicas_match_single_rank():
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=120) for _ in range(2)], key=lambda r: r[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from oracle import oracle
    from snch_lbvh_gb300 import meshes
    v, f = meshes.noisy_icosphere(2, 1.0, 0.01, seed=1)
    pts = meshes.box_queries(v, 1000, 1.2, seed=2)
    idx, dist_ = oracle.Tree(v, f).nearest(pts, nthreads=1)
    for r in res:  # every replica gives the single-rank answers
        np.testing.assert_array_equal(r[1], idx)
        np.testing.assert_array_equal(r[2], dist_)
    assert all(r[3] == 2.0 for r in res)  # max over ranks of (rank + 1)


def test_single_process_reduction_is_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
