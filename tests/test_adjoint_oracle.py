"""The float64 torch restatement of the frozen forward, pinned to the raytrace.

The adjoint kernel is checked against ``oracle/adjoint_torch.py``; this file
checks that restatement itself, on the CPU, against the numpy raytrace oracle
(which is bit-exact against the reference, see test_oracle_golden.py):
* at the nominal parameters it reproduces the traced detector coordinates;
* at perturbed parameters it reproduces a fresh trace of the elements moved
  by ``PoseModel.apply`` (facet and detector poses, focal length), for every
  photon whose discrete choices did not change -- so the pose
  parametrisation of the gradient is the one the raytrace sees;
* its freeze() reproduces the traced choices it must hold fixed.
"""
import numpy as np
import pytest
import torch

from oracle import adjoint_torch as AT


def frozen_dict(model, inp, traced, orders, theta):
    """torch_dict of the frozen problem, built from an oracle trace on the CPU."""
    from marxs_gb300 import _abi
    det_col = 'det_x' if model.det_kind == _abi.ADJ_DET_FLAT else 'det_phi'
    ok = np.isfinite(traced[det_col]) & (traced['facet'] >= 0) & \
        np.isfinite(traced['inplanescatter'])
    group = np.full(len(ok), -1)
    for g, m in enumerate(orders):
        group[ok & (traced['order'] == m)] = g
    sel = np.nonzero(group >= 0)[0]
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, dtype=float))
    fidx = np.array([model.facet_index[int(i)] for i in traced['facet'][sel]])
    base, det = model.facet_base, model.det_block
    d = {'P0': t(inp['pos'][sel, :3]), 'd0': t(inp['dir'][sel, :3]),
         'lens_c': t(model.lens_block[0:3]), 'lens_n': t(model.lens_block[3:6]),
         'lens_ez': t(model.lens_block[6:9]), 'lens_doff': float(model.lens_block[9]),
         'scat_c': t(model.scatter_block[0:3]), 'scat_n': t(model.scatter_block[3:6]),
         'alpha': t(traced['inplanescatter'][sel]), 'beta': t(traced['perpplanescatter'][sel]),
         'facet': torch.from_numpy(fidx).long(), 'facet_c': t(base[:, 0:3]),
         'facet_n': t(base[:, 3:6]), 'facet_l': t(base[:, 6:9]), 'facet_dneg': t(base[:, 9:12]),
         'facet_d': t(base[:, 12]), 'order': t(traced['order'][sel]),
         'energy': t(inp['energy'][sel]), 'w': t(traced['probability'][sel]),
         'group': torch.from_numpy(group[sel]).long()}
    if model.det_kind == _abi.ADJ_DET_FLAT:
        d.update(det_kind='flat', det_c=t(det[0:3]), det_n=t(det[3:6]), det_ey=t(det[6:9]),
                 det_ez=t(det[9:12]))
    else:
        d.update(det_kind='cyl', det_c=t(det[0:3]), det_Minv=t(det[12:21].reshape(3, 3)),
                 det_R=float(det[21]), det_zoomz=float(det[22]))
    cat = torch.from_numpy((model.facet_flags & _abi.ADJ_FACET_CAT) > 0)
    trans = torch.from_numpy((model.facet_flags & _abi.ADJ_FACET_TRANSMISSION) > 0)
    d.update(AT.freeze(theta, d, cat, trans, phi_lim=(det[23], det[24])))
    return d, sel


def _detector_xy(model, traced, sel):
    from marxs_gb300 import _abi
    if model.det_kind == _abi.ADJ_DET_FLAT:
        return traced['det_x'][sel], traced['det_y'][sel]
    return traced['det_phi'][sel] * model.det_block[21], traced['det_y'][sel]


def _random_theta(model, rng, scale=1.0):
    th = np.zeros(model.n_params)
    th[0] = model.focallength + 0.5 * scale
    sl = model.param_slices()
    for key, s in (('facet_translation', 0.02), ('facet_rotation', 2e-4),
                   ('detector_translation', 0.05), ('detector_rotation', 5e-4)):
        th[sl[key]] = rng.normal(0, s * scale, len(sl[key]))
    return torch.from_numpy(th)


CASES = {
    # config, photons, orders kept, energies (None: the config's spectrum)
    'c1': ('c1', 1500, list(range(-10, 3)), None),
    'c2': ('c2', 600, [-8, -7, -6, -5, -4, -3, 0], 0.5),
}


@pytest.fixture(scope='module', params=sorted(CASES))
def traced_case(request):
    from marxs_gb300 import configs
    from marxs_gb300.adjoint import PoseModel
    from oracle.raytrace import run_sequence
    cfg, n, orders, energy = CASES[request.param]
    inst = configs.build(cfg)
    if energy is None:
        inp = configs.photons_for(cfg, n, seed=11)
    else:
        inp = configs.annulus_photons(n, 11, inst.aperture_x, energies=np.full(n, energy))
    draws = configs.draws_for(inst.draw_slots, n, seed=11)
    traced, _ = run_sequence(inst.elements, inp, draws)
    model = PoseModel(inst.elements)
    d, sel = frozen_dict(model, inp, traced, orders, model.theta0())
    return inst, model, inp, draws, traced, d, sel, orders


def test_nominal_forward_reproduces_the_trace(traced_case):
    inst, model, inp, draws, traced, d, sel, orders = traced_case
    assert len(sel) > 50
    x, y = AT.forward(model.theta0(), d)
    tx, ty = _detector_xy(model, traced, sel)
    np.testing.assert_allclose(x.numpy(), tx, rtol=0, atol=1e-8)
    np.testing.assert_allclose(y.numpy(), ty, rtol=0, atol=1e-8)


def test_perturbed_forward_reproduces_a_trace_of_moved_elements(traced_case):
    from oracle.raytrace import run_sequence
    inst, model, inp, draws, traced, d, sel, orders = traced_case
    theta = _random_theta(model, np.random.default_rng(5))
    try:
        model.apply(theta)
        moved, _ = run_sequence(inst.elements, inp, draws)
    finally:
        model.restore()
    x, y = AT.forward(theta, d)
    tx, ty = _detector_xy(model, moved, sel)
    same = (moved['facet'][sel] == traced['facet'][sel]) & \
        (moved['order'][sel] == traced['order'][sel]) & np.isfinite(tx)
    assert same.mean() > 0.9
    np.testing.assert_allclose(x.numpy()[same], tx[same], rtol=0, atol=1e-8)
    np.testing.assert_allclose(y.numpy()[same], ty[same], rtol=0, atol=1e-8)
    # the perturbation moved the spots by far more than the tolerance
    assert np.max(np.abs(x.numpy()[same] - _detector_xy(model, traced, sel)[0][same])) > 1e-3


def test_restore_returns_the_nominal_geometry(traced_case):
    from oracle.raytrace import run_sequence
    inst, model, inp, draws, traced, d, sel, orders = traced_case
    model.apply(_random_theta(model, np.random.default_rng(2)))
    model.restore()
    again, _ = run_sequence(inst.elements, inp, draws)
    for k in ('facet', 'order'):
        np.testing.assert_array_equal(again[k], traced[k])
    tx, _ = _detector_xy(model, traced, sel)
    ax, _ = _detector_xy(model, again, sel)
    np.testing.assert_allclose(ax, tx, rtol=0, atol=1e-9)


def test_group_stats_match_moment_stats(traced_case):
    """The moment form used with the kernel equals the two-pass statistics."""
    from marxs_gb300.adjoint import moment_stats
    inst, model, inp, draws, traced, d, sel, orders = traced_case
    x, y = AT.forward(model.theta0(), d)
    G = len(orders)
    ref = torch.stack([torch.tensor([x[d['group'] == g].mean() for g in range(G)]),
                       torch.tensor([y[d['group'] == g].mean() for g in range(G)])], 1)
    m = torch.zeros((G, 5), dtype=torch.float64)
    for g in range(G):
        k = d['group'] == g
        w, xs, ys = d['w'][k], x[k] - ref[g, 0], y[k] - ref[g, 1]
        m[g] = torch.stack([w.sum(), (w * xs).sum(), (w * ys).sum(), (w * xs * xs).sum(),
                            (w * ys * ys).sum()])
    a = moment_stats(m, ref)
    b = AT.group_stats(x, y, d['w'], d['group'], G)
    ok = b['W'] > 0
    for k in a:
        np.testing.assert_allclose(a[k][ok].numpy(), b[k][ok].numpy(), rtol=1e-9, atol=1e-12)


def test_torch_gradient_matches_central_differences_of_itself(traced_case):
    """Sanity of the restatement's differentiability (a handful of params)."""
    from marxs_gb300.adjoint import resolving_power, spot_loss
    inst, model, inp, draws, traced, d, sel, orders = traced_case
    G = len(orders)
    counts = np.bincount(d['group'].numpy(), minlength=G)
    if 0 in orders:
        loss = resolving_power(orders.index(0), [g for g, m in enumerate(orders)
                                                 if m != 0 and counts[g] >= 5])
    else:
        loss = spot_loss(0.0, group=0)
    th0 = model.theta0()
    L, g = AT.stats_loss_and_grad(th0, d, G, loss)
    h = model.step_sizes()
    counts = np.bincount(d['facet'].numpy(), minlength=model.n_facets)
    j = int(np.argmax(counts))
    params = [0, 1 + 6 * j, 1 + 6 * j + 4, 1 + 6 * j + 5, model.n_params - 6,
              model.n_params - 2]
    for k in params:
        tp, tm = th0.clone(), th0.clone()
        tp[k] += h[k]
        tm[k] -= h[k]
        with torch.no_grad():
            fp = loss(AT.group_stats(*AT.forward(tp, d), d['w'], d['group'], G))
            fm = loss(AT.group_stats(*AT.forward(tm, d), d['w'], d['group'], G))
        fd = float((fp - fm) / (2 * h[k]))
        assert abs(fd - float(g[k])) <= 1e-4 * max(abs(float(g[k])), 1e-3 * float(g.abs().max())), k
