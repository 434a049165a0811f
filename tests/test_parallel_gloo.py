"""Sharding across ranks (world size 2, gloo, CPU): view shards of the forward
and z-slab shards of the backprojection, computed per rank with the oracle on
each rank's own geometry, gathered and compared with the single-process
result.  Exercises the host-side sharding logic the multi-GPU path uses."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from _util import cone_params


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, params, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from ctreconstruction_gb300.parallel import slab_shard, view_shard
    from oracle.oracle import OracleGeometry
    rng = np.random.default_rng(0)
    g = OracleGeometry(params)
    x = rng.random((g.nz, g.ny, g.nx), dtype=np.float32)
    y = rng.random((g.nviews, g.nv, g.nu), dtype=np.float32)
    v0, nv = view_shard(params, rank, world)
    fwd = torch.from_numpy(g.forward(x, v0, nv))
    z0, nz, sp = slab_shard(params, rank, world)
    gs = OracleGeometry({k: getattr(sp, k) for k in sp.as_dict()})
    bp = torch.from_numpy(gs.backward_fdk(y))
    fwd_parts = [None] * world
    bp_parts = [None] * world
    dist.all_gather_object(fwd_parts, fwd)
    dist.all_gather_object(bp_parts, bp)
    if rank == 0:
        full_f = np.concatenate([p.numpy() for p in fwd_parts])
        full_b = np.concatenate([p.numpy() for p in bp_parts])
        q.put((float(np.abs(full_f - g.forward(x)).max()), float(np.abs(full_b - g.backward_fdk(y)).max())))
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_view_and_slab_shards_recompose(world):
    params = cone_params(n=(12, 10, 9), nviews=7, nu=20, nv=16)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, params, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    ef, eb = q.get(timeout=10)
    assert ef == 0.0
    assert eb < 1e-9


def test_shard_range_covers():
    from ctreconstruction_gb300.parallel import shard_range
    for n in (0, 1, 7, 720):
        for w in (1, 2, 3, 8):
            parts = [shard_range(n, r, w) for r in range(w)]
            assert sum(c for _, c in parts) == n
            assert all(parts[i][0] + parts[i][1] == parts[i + 1][0] for i in range(w - 1))
