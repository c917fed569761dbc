"""Replica path on CPU with gloo, world size 2: each rank traces its shard of
the rays (with the oracle: no GPU here), the shards are gathered in ray order
and must equal the single-process result; the bench's max-over-ranks timing
reduction is exercised the same way."""
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


def _worker(rank, world, port, result_path):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import sys
    from pathlib import Path
    sys.path.insert(0, str(Path(__file__).resolve().parents[1]))
    import oracle
    from radeonrays_sdk_gb300 import replicas, scenes

    v, i = scenes.heightfield(33, scenes.rng(70))
    rays = scenes.incoherent_rays(3001, v.min(0), v.max(0), scenes.rng(70, 1))
    nodes, _, _ = oracle.build_mesh(v, i)
    b, e = replicas.shard(rays.shape[0], rank, world)
    local = torch.from_numpy(oracle.trace(nodes, rays[b:e]).view(np.int32))
    full = replicas.gather_shards(local, rays.shape[0], rank, world)
    t = torch.tensor([float(rank + 1)], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    if rank == 0:
        np.save(result_path, full.numpy())
        np.save(result_path + ".max.npy", t.numpy())
    dist.barrier()
    dist.destroy_process_group()


def test_replica_shards_reassemble(tmp_path, orc):
    import torch.multiprocessing as mp
    from radeonrays_sdk_gb300 import replicas, scenes

    assert replicas.shard(10, 0, 3) == (0, 4) and replicas.shard(10, 2, 3) == (7, 10)
    with pytest.raises(ValueError):
        replicas.shard(10, 3, 3)
    out = str(tmp_path / "hits.npy")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    v, i = scenes.heightfield(33, scenes.rng(70))
    rays = scenes.incoherent_rays(3001, v.min(0), v.max(0), scenes.rng(70, 1))
    nodes, _, _ = orc.build_mesh(v, i)
    want = orc.trace(nodes, rays).view(np.int32)
    assert np.array_equal(np.load(out), want)
    assert float(np.load(out + ".max.npy")[0]) == 2.0
