"""Multi-rank host logic with two gloo ranks on CPU (127.0.0.1).

Each rank traces its shard of a photon list (the CPU oracle stands in for
the per-GPU trace); gathering the shards reproduces the single-rank run,
and timings reduce to their maximum over ranks.
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from marxs_gb300.sharding import strong_shard, weak_shard, max_over_ranks


def _free_port():
    with socket.socket() as s:
        s.bind(('127.0.0.1', 0))
        return s.getsockname()[1]


def _worker(rank, world, port, n, q):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        from marxs_gb300 import configs
        from oracle.raytrace import run_sequence
        inst = configs.build('c1')
        host = configs.photons_for('c1', n, seed=9)
        draws = configs.draws_for(inst.draw_slots, n, seed=9)
        a, b = strong_shard(rank, world, n)
        sub = {k: v[a:b] for k, v in host.items()}
        sub_draws = {e: {k: v[a:b] for k, v in d.items()} for e, d in draws.items()}
        out, _ = run_sequence(inst.elements, sub, sub_draws)
        parts = [None] * world
        dist.all_gather_object(parts, {k: out[k] for k in ('pos', 'facet', 'order', 'det_x')})
        t = max_over_ranks([1.0 + rank, 5.0 - rank], dist)
        if rank == 0:
            q.put((parts, t))
    finally:
        dist.destroy_process_group()


def test_shard_helpers():
    n = 1003
    ranges = [strong_shard(r, 4, n) for r in range(4)]
    assert ranges[0][0] == 0 and ranges[-1][1] == n
    assert all(ranges[i][1] == ranges[i + 1][0] for i in range(3))
    assert weak_shard(3, 100) == (300, 400)
    assert max_over_ranks([1.0, 2.0]) == [1.0, 2.0]


def test_two_gloo_ranks_reproduce_single_rank():
    from marxs_gb300 import configs
    from oracle.raytrace import run_sequence
    n, world = 3000, 2
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, n, q)) for r in range(world)]
    for p in procs:
        p.start()
    parts, t = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    inst = configs.build('c1')
    host = configs.photons_for('c1', n, seed=9)
    ref, _ = run_sequence(inst.elements, host, configs.draws_for(inst.draw_slots, n, seed=9))
    for col in ('pos', 'facet', 'order', 'det_x'):
        joined = np.concatenate([p[col] for p in parts])
        assert np.array_equal(joined, ref[col], equal_nan=True), col
    assert t == [2.0, 5.0]
