"""Replica sharding and the moment-block merge across 2 gloo ranks (CPU)."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

from pincosimulator_gb300 import observables as ob
from pincosimulator_gb300 import replicas

T, B, N = 512, 16, 8


def samples(traj_ids):
    """Synthetic Wigner samples, each trajectory generated from its own id."""
    out = []
    for k in traj_ids:
        r = np.random.default_rng(1000 + int(k))
        out.append(0.7 * (r.normal(size=N) + 1j * r.normal(size=N)) + 0.4)
    return np.array(out)


def blocks(x, nb):
    edges = (np.arange(nb + 1) * len(x)) // nb
    m = np.zeros((nb, N, 3))
    for b in range(nb):
        a2 = np.abs(x[edges[b]:edges[b + 1]]) ** 2
        m[b, :, 0] = a2.sum(0)
        m[b, :, 1] = (a2 ** 2).sum(0)
    return m


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    lo, hi = replicas.shard_range(rank, world, T)
    local = blocks(samples(range(lo, hi)), replicas.shard_blocks(rank, world, B))
    merged = replicas.gather_blocks(local)
    if rank == 0:
        q.put(merged)
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_merge_is_bit_identical():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    single = blocks(samples(range(T)), B)
    assert np.array_equal(merged, single)
    o1, o2 = ob.observables(merged, T), ob.observables(single, T)
    assert np.array_equal(o1["n"], o2["n"])


def test_shard_ranges_partition():
    for world in (1, 2, 3, 8):
        r = [replicas.shard_range(k, world, 1001) for k in range(world)]
        assert r[0][0] == 0 and r[-1][1] == 1001
        assert all(r[k][1] == r[k + 1][0] for k in range(world - 1))
    with pytest.raises(ValueError):
        replicas.shard_blocks(0, 3, 16)
