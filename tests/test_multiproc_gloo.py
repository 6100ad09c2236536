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


# ------------------------------------------------------------ adjoint shards
PER_PHOTON = ('P0', 'd0', 'alpha', 'beta', 'facet', 'order', 'energy', 'w', 'group', 'sign',
              'nsign', 'root')


class _CpuShard:
    """The per-rank interface PoseMoments drives (moments, vjp) over a
    frozen problem on the CPU: the float64 torch restatement of the frozen
    forward stands in for the kernels, the collectives are the product's."""

    def __init__(self, prob, n_groups, theta, process_group=None):
        from marxs_gb300.adjoint import group_centres, sum_over_shards
        self.prob, self.n_groups, self.process_group = prob, n_groups, process_group
        self.ref = torch.zeros((n_groups, 2), dtype=torch.float64)
        self.ref = group_centres(sum_over_shards(self.moments(theta), process_group))

    def _moments(self, theta):
        from oracle import adjoint_torch as AT
        x, y = AT.forward(theta, self.prob)
        w, g = self.prob['w'], self.prob['group']
        xr, yr = x - self.ref[g, 0], y - self.ref[g, 1]
        cols = torch.stack([w, w * xr, w * yr, w * xr * xr, w * yr * yr], 1)
        return torch.zeros((self.n_groups, 5), dtype=torch.float64).index_add(0, g, cols)

    def moments(self, theta):
        with torch.no_grad():
            return self._moments(theta)

    def vjp(self, theta, grad_moments):
        with torch.enable_grad():                # called from a backward pass
            th = theta.detach().clone().requires_grad_(True)
            (g,) = torch.autograd.grad(self._moments(th), th, grad_moments)
        return g


def _adjoint_problem():
    from marxs_gb300 import configs
    from marxs_gb300.adjoint import PoseModel
    from oracle.raytrace import run_sequence
    from test_adjoint_oracle import frozen_dict
    n, orders = 1500, list(range(-10, 3))
    inst = configs.build('c1')
    inp = configs.photons_for('c1', n, seed=11)
    traced, _ = run_sequence(inst.elements, inp, configs.draws_for(inst.draw_slots, n, seed=11))
    model = PoseModel(inst.elements)
    d, _ = frozen_dict(model, inp, traced, orders, model.theta0())
    theta = model.theta0().clone()
    theta[0] += 0.3
    theta[1 + 6 * 17 + 4] += 1e-4            # a facet rotation
    return d, len(orders), model, theta


def _loss_and_grad(stand, theta):
    from marxs_gb300.adjoint import PoseMoments, moment_stats, spot_loss
    th = theta.clone().requires_grad_(True)
    L = spot_loss(0.0, group=5)(moment_stats(PoseMoments.apply(th, stand), stand.ref))
    (g,) = torch.autograd.grad(L, th)
    return float(L.detach()), g


def _adjoint_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR='127.0.0.1', MASTER_PORT=str(port))
    dist.init_process_group('gloo', rank=rank, world_size=world)
    try:
        d, G, model, theta = _adjoint_problem()
        n = len(d['w'])
        a, b = strong_shard(rank, world, n)
        shard = {k: (v[a:b] if k in PER_PHOTON else v) for k, v in d.items()}
        stand = _CpuShard(shard, G, model.theta0(), dist.group.WORLD)
        L, g = _loss_and_grad(stand, theta)
        if rank == 0:
            q.put((L, g.numpy(), stand.ref.numpy(), n))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_sum_adjoint_moments_and_gradients():
    """Photons of one frozen problem split over two gloo ranks: the group
    centres, the loss and the whole gradient equal the single-process ones
    (one all-reduce of the moments, one of the gradient)."""
    world = 2
    ctx = mp.get_context('spawn')
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_adjoint_worker, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    L2, g2, ref2, n = q.get(timeout=240)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    d, G, model, theta = _adjoint_problem()
    assert n == len(d['w']) and n > 100
    one = _CpuShard(d, G, model.theta0())
    L1, g1 = _loss_and_grad(one, theta)
    assert np.allclose(ref2, one.ref.numpy(), rtol=1e-12, atol=1e-12)
    assert abs(L2 - L1) <= 1e-10 * abs(L1)
    g1 = g1.numpy()
    assert np.abs(g1).max() > 0
    assert np.linalg.norm(g2 - g1) <= 1e-9 * np.linalg.norm(g1)
