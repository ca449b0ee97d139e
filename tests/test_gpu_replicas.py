"""Replica sharding on the engine itself: two processes (gloo ranks sharing
this machine's GPU, each running only its own independent kernels) step disjoint
trajectory ranges of one batch through twmc_batch_init / advance / reduce,
and the moment blocks gathered in rank order equal, bit for bit, the blocks
of one process stepping all trajectories."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp

from pincosimulator_gb300 import replicas

pytestmark = pytest.mark.gpu

T, B, FRAMES = 512, 32, 3
SHAPES = [(16, 16), (64, 64)]


def engine_blocks(nx, ny, lo, hi, nblocks):
    """Moment blocks of trajectories [lo, hi) (seed and id follow the
    trajectory index) after FRAMES frames of 50 steps."""
    from pincosimulator_gb300 import twmc

    s = twmc.System(nx=nx, ny=ny, J=1.0, gamma=1.0, dt=0.002, frame_steps=50,
                    omega=twmc.Noisy(-0.5, twmc.DISORDER_GAUSSIAN, 0.2), U=0.2, F=2.0, beta_init_sigma=0.5,
                    precision=twmc.PREC_F32, n_moment_blocks=nblocks)
    s.batch_init(s.make_tasks(hi - lo, t_end=10.0, seed0=77 + lo, id0=1 + lo))
    for _ in range(FRAMES):
        s.advance(50)
    s.reduce()
    s.sync()
    _, m = s.download(field=False, moments=True)
    s.close()
    return m


def _worker(rank, world, port, q):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        lo, hi = replicas.shard_range(rank, world, T)
        out = {}
        for nx, ny in SHAPES:
            local = engine_blocks(nx, ny, lo, hi, replicas.shard_blocks(rank, world, B))
            out[(nx, ny)] = replicas.gather_blocks(local)
        if rank == 0:
            q.put(out)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_rank_engine_blocks_are_bit_identical(built_lib):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29600 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    merged = q.get(timeout=300)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    for nx, ny in SHAPES:
        single = engine_blocks(nx, ny, 0, T, B)
        assert merged[(nx, ny)].shape == single.shape
        assert np.isfinite(single).all()
        assert np.array_equal(merged[(nx, ny)], single), (nx, ny)
