"""Multi-process paths on CPU: two gloo ranks.

Clusters are independent; ranks split them by the LPT assignment of
shard_clusters with no data exchange, and bench.py combines the ranks'
timings with one max-reduction.  Both are exercised here with world size 2.
"""

import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, sizes, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import torch
    import bench
    from pycwb_gb300.likelihoodWP.batched import shard_clusters
    mine = shard_clusters(sizes, world, rank)
    load = int(np.asarray(sizes)[mine].sum())
    # every rank's clusters, gathered to check the partition
    gathered = [None] * world
    dist.all_gather_object(gathered, mine.tolist())
    worst = bench.max_over_ranks(dist, float(load), torch.device("cpu"))
    bench.barrier(dist)
    if rank == 0:
        out.put((gathered, worst))
    dist.destroy_process_group()


def test_two_ranks_partition_clusters_and_reduce_timings():
    sizes = np.random.default_rng(3).integers(20, 3000, size=101)
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, sizes, q)) for r in range(world)]
    for p in procs:
        p.start()
    gathered, worst = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    allc = sorted(c for part in gathered for c in part)
    assert allc == list(range(len(sizes)))                      # a partition
    loads = [int(sizes[part].sum()) for part in gathered]
    assert worst == max(loads)                                  # max over ranks
    assert max(loads) - min(loads) <= sizes.max()               # LPT balance bound


def test_shard_clusters_single_rank_and_errors():
    from pycwb_gb300.likelihoodWP.batched import shard_clusters
    sizes = [5, 1, 9]
    assert shard_clusters(sizes, 1, 0).tolist() == [0, 1, 2]
    with pytest.raises(ValueError):
        shard_clusters(sizes, 2, 2)
