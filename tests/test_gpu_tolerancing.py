"""Facet poses on the device (mgpu_facet_poses) and device tolerancing runs.

* the device-posed facet tables equal the frames of the reference's element
  poses after wiggle / moveglobal / moveindividual (golden vectors from
  design/tolerancing.py) to 1e-12;
* wiggle's Philox draws follow N(offset, sigma) (KS p > 1e-3) and are keyed
  by the seed;
* a trace through device-posed facets equals the trace through the same
  poses lowered on the host (facet and order exact, positions 1e-9);
* run_tolerances with CaptureResAeff equals the host loop.
"""
import os
import sys
from types import SimpleNamespace

import numpy as np
import pytest
import torch
from scipy import stats

from conftest import load_golden

sys.path.insert(0, os.path.join(os.path.dirname(__file__), 'golden'))
from pose_case import build_pose_parallel  # noqa: E402

pytestmark = pytest.mark.gpu


def _native(g):
    from marxs_gb300 import geomath
    from marxs_gb300.optics import CATGrating, OrderSelector
    from marxs_gb300.simulator import Parallel
    ns = SimpleNamespace(Parallel=Parallel, CATGrating=CATGrating, OrderSelector=OrderSelector)
    case = {k: g[k] for k in ('positions', 'angles', 'groove', 'par_position', 'par_angles',
                              'zoom', 'blaze')}
    return build_pose_parallel(ns, case, geomath.euler2mat)


def _table(poses):
    from marxs_gb300 import _abi
    raw = poses.inst.stage_facets[poses.si].cpu().numpy()
    return raw.view(_abi.FACET_DTYPE)


def _frames(P, groove):
    v = [P[:, :3, k] for k in range(3)]
    n = [np.linalg.norm(x, axis=1) for x in v]
    ex, ey, ez = (v[k] / n[k][:, None] for k in range(3))
    sn, cs = np.sin(-groove)[:, None], np.cos(-groove)[:, None]
    return {'c': P[:, :3, 3], 'ex': ex, 'ey': ey, 'ez': ez, 'hy': n[1], 'hz': n[2],
            'l': sn * ey + cs * ez, 'dneg': -(cs * ey - sn * ez)}


def _check(tab, P, groove):
    ref = _frames(P, groove)
    for k, v in ref.items():
        assert np.allclose(tab[k], v, rtol=1e-13, atol=1e-12), k


def test_device_poses_match_reference_tolerancing():
    from marxs_gb300 import lowering as L
    from marxs_gb300.gpu import GpuSequence
    from marxs_gb300.tolerancing import DeviceFacetPoses
    g = load_golden('poses')
    gas = _native(g)
    seq = GpuSequence(elements=[gas])
    poses = DeviceFacetPoses(seq, gas)
    groove = g['groove']
    host0 = _table(poses).copy()
    _check(host0, g['base_pos4d'], groove)
    poses.set_perturbation(torch.from_numpy(g['wiggle_pert']))
    _check(_table(poses), g['wiggle_pos4d'], groove)
    poses.moveglobal(*g['global_move'])
    _check(_table(poses), g['global_pos4d'], groove)
    assert torch.equal(poses.perturbation.cpu(), torch.from_numpy(g['wiggle_pert']))
    poses.moveindividual(*g['indiv_move'])
    tab = _table(poses)
    _check(tab, g['indiv_pos4d'], groove)
    # FP32-local records follow the float64 frame
    t32 = poses.inst.stage_facets32[poses.si].cpu().numpy().view(L._abi.FACET32_DTYPE)
    ref32 = L.facets32_table(tab)
    for k in ('c_hi', 'c_lo', 'ex', 'ey', 'ez', 'l', 'dneg', 'hy', 'hz'):
        assert np.array_equal(t32[k], ref32[k]), k
    poses.reset()
    _check(_table(poses), g['base_pos4d'], groove)


def test_wiggle_draws_follow_the_reference_distribution():
    from marxs_gb300 import configs
    from marxs_gb300.gpu import GpuSequence
    from marxs_gb300.tolerancing import DeviceFacetPoses, wiggle
    inst = configs.build('c2')
    seq = GpuSequence(elements=inst.elements)
    poses = DeviceFacetPoses(seq, inst.gas)
    sigma = np.array([0.5, 0.3, 0.2, 1e-3, 2e-3, 5e-4])
    a = poses.wiggle(*sigma, seed=5).cpu().numpy()
    for k in range(6):
        assert stats.kstest(a[:, k] / sigma[k], 'norm').pvalue > 1e-3, k
    assert np.array_equal(a, poses.wiggle(*sigma, seed=5).cpu().numpy())
    wiggle(poses, *sigma)
    b = poses.perturbation.cpu().numpy()
    wiggle([poses], *sigma)
    assert not np.array_equal(b, poses.perturbation.cpu().numpy())
    # moveindividual is the same move for every facet
    m = poses.moveindividual(0.1, 0.2, 0.3, 1e-4, 2e-4, 3e-4).cpu().numpy()
    assert np.array_equal(m, np.tile([0.1, 0.2, 0.3, 1e-4, 2e-4, 3e-4], (len(m), 1)))
    with pytest.raises(RuntimeError):
        poses.moveglobal(dx=0., dy=400.)


def _host_posed_c2(pert, move=None):
    from marxs_gb300 import configs, geomath
    inst = configs.build('c2')
    inst.gas.elem_uncertainty = [geomath.compose(q[:3], geomath.euler2mat(*q[3:], 'sxyz'),
                                                 np.ones(3)) for q in pert]
    if move is not None:
        inst.gas.uncertainty = geomath.compose(move[:3], geomath.euler2mat(*move[3:], 'sxyz'),
                                               np.ones(3))
    inst.gas.generate_elements()
    return inst


def test_trace_through_device_poses_matches_host_lowering():
    from marxs_gb300 import configs
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    from marxs_gb300.tolerancing import DeviceFacetPoses
    rng = np.random.default_rng(3)
    inst = configs.build('c2')
    F = len(inst.gas.elements)
    pert = np.c_[rng.normal(0, 0.2, (F, 3)), rng.normal(0, 2e-4, (F, 3))]
    move = np.array([0.3, -0.5, 0.2, 1e-4, -2e-4, 3e-4])
    n = 200_000
    photons = configs.photons_for('c2', n, seed=8)
    out = {}
    for kind in ('device', 'host'):
        if kind == 'device':
            inst_k = configs.build('c2')
            seq = GpuSequence(elements=inst_k.elements, precision='fp64', rng='philox', seed=3)
            poses = DeviceFacetPoses(seq, inst_k.gas)
            poses.set_perturbation(pert)
            poses.moveglobal(*move)
        else:
            inst_k = _host_posed_c2(pert, move)
            seq = GpuSequence(elements=inst_k.elements, precision='fp64', rng='philox', seed=3)
        ph = DevicePhotons.from_columns(photons)
        plan, bufs = seq.allocate_columns(n)
        status, _ = seq.trace_device(ph, ph, plan, bufs)
        torch.cuda.synchronize()
        assert int(status.item()) == 0
        out[kind] = {k: v.cpu().numpy() for k, v in bufs.items()}
    d, h = out['device'], out['host']
    assert np.array_equal(d['facet'], h['facet'])
    assert np.array_equal(d['order'], h['order'], equal_nan=True)
    assert (d['facet'] >= 0).mean() > 0.3
    for k in ('det_phi', 'det_y', 'grat_y', 'grat_z'):
        a, b = d[k], h[k]
        assert np.array_equal(np.isnan(a), np.isnan(b)), k
        m = ~np.isnan(a)
        assert np.allclose(a[m], b[m], rtol=1e-9, atol=1e-9), k


def test_run_tolerances_matches_host_loop():
    from marxs_gb300 import configs
    from marxs_gb300.analysis import CaptureResAeff
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    from marxs_gb300.source import CircleAperture, DeviceSource
    from marxs_gb300.tolerancing import DeviceFacetPoses, moveglobal, run_tolerances
    inst = configs.build('c2')
    F = len(inst.gas.elements)
    seq = GpuSequence(elements=inst.elements, precision='fp64', rng='philox', seed=11)
    # rz = 1e-3 about the global origin moves the array (~11 m out) by ~11
    # mm, dy another 1 mm: beyond the default 10 mm of room
    poses = DeviceFacetPoses(seq, inst.gas, max_shift=20.0)
    poses.set_perturbation(np.zeros((F, 6)))
    ap = CircleAperture(position=[12000., 0, 0], zoom=[1, 500, 500], r_inner=300.)
    src = DeviceSource(ap, energy=0.5)
    n = 300_000
    photons = src.generate(n, seed=4)
    cap = CaptureResAeff(orders=np.arange(-8, 1), dispersion_coord='det_phi')
    params = [{'dx': 0.}, {'rx': 2e-3}, {'dy': 1.0, 'rz': 1e-3}]
    res = run_tolerances(photons, seq, moveglobal, poses, params, cap)
    assert [r['dx'] if 'dx' in r else None for r in res][0] == 0.
    for pars, r in zip(params, res):
        move = np.array([pars.get(k, 0.) for k in ('dx', 'dy', 'dz', 'rx', 'ry', 'rz')])
        host = _host_posed_c2(np.zeros((F, 6)), move)
        hseq = GpuSequence(elements=host.elements, precision='fp64', rng='philox', seed=11)
        ph = src.generate(n, seed=4)
        plan, bufs = hseq.allocate_columns(n)
        hseq.trace_device(ph, ph, plan, bufs)
        cols = dict(bufs, probability=ph.prob, energy=ph.energy)
        ref = cap(cols)
        for k in ('Aeff', 'R'):
            a = np.asarray(r[k], dtype=float)
            b = np.asarray(ref[k], dtype=float)
            assert np.array_equal(np.isnan(a), np.isnan(b)), k
            assert np.allclose(a[~np.isnan(a)], b[~np.isnan(b)], rtol=1e-9), (pars, k)
    assert res[0]['Rgrat'] > res[1]['Rgrat'] * 0.5
