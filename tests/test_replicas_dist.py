"""The multi-GPU path on CPU: replicas only, so the only cross-rank pieces are the replica
split and the max-over-ranks timing reduction. Two gloo ranks (127.0.0.1) check that
the shards partition the replica ids and that every rank sees the slowest rank's time."""

import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, n_replicas, out_dir):
    import torch.distributed as dist

    from oxdna import replicas
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ids = replicas.shard(n_replicas, rank, world)
    t = replicas.max_over_ranks(1.0 + rank, dist)  # the rank's "timing"
    dist.barrier()
    np.save(os.path.join(out_dir, f"rank{rank}.npy"), np.concatenate([[t], ids]))
    dist.destroy_process_group()


@pytest.mark.parametrize("n_replicas", [512, 7])
def test_two_gloo_ranks_split_replicas_and_reduce_time(tmp_path, n_replicas):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), n_replicas, str(tmp_path)), nprocs=world, join=True)
    parts = [np.load(tmp_path / f"rank{r}.npy") for r in range(world)]
    times = [p[0] for p in parts]
    ids = np.concatenate([p[1:] for p in parts]).astype(int)
    assert times == [2.0, 2.0]  # max over ranks everywhere
    assert sorted(ids.tolist()) == list(range(n_replicas))
    assert abs(len(parts[0]) - len(parts[1])) <= 1
    del torch
