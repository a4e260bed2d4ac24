"""Host side of a multi-GPU split, on CPU with two gloo ranks: z-slab
bounds, and the one exchange step (an all-gather of per-slab vertex totals)
that places each rank's soup in the whole volume's soup.  Slab counts come
from the oracle on each slab's voxel layers."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from marching_cube_gb300 import shard, synthetic


def test_slab_bounds():
    assert shard.slab_bounds(65, 2) == [(0, 32), (32, 64)]
    assert shard.slab_bounds(66, 3) == [(0, 24), (24, 48), (48, 65)]
    b = shard.slab_bounds(10, 4)  # 9 cube layers, 2 brick layers
    assert b == [(0, 8), (8, 9), (9, 9), (9, 9)]
    for nz in (2, 9, 17, 100, 513):
        for parts in (1, 2, 3, 7):
            bb = shard.slab_bounds(nz, parts)
            assert bb[0][0] == 0 and bb[-1][1] == nz - 1
            assert all(z0 % 8 == 0 or z0 == z1 for z0, z1 in bb)
            assert all(bb[i][1] == bb[i + 1][0] for i in range(parts - 1))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, vol, result):
    import torch.distributed as dist
    import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        z0, z1 = shard.slab_bounds(vol.shape[0], world)[rank]
        n = 0
        if z1 > z0:
            _, ntri = oracle.mc_count(np.ascontiguousarray(vol[z0:z1 + 1]))
            n = 3 * ntri
        off, total = shard.exchange_offsets(n)
        result[rank] = (n, off, total)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_exchange_offsets_gloo(world):
    import oracle
    oracle.build()
    vol = synthetic.sphere_volume(49, radius=15.0, trunc=4.0, seed=5)
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        result = m.dict()
        mp.start_processes(_rank, args=(world, _free_port(), vol, result), nprocs=world, join=True,
                           start_method="spawn")
        res = dict(result)
    _, ntri = oracle.mc_count(vol)
    counts = [res[r][0] for r in range(world)]
    assert sum(counts) == 3 * ntri
    for r in range(world):
        assert res[r][1] == sum(counts[:r])
        assert res[r][2] == 3 * ntri
