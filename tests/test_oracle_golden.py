"""The CPU oracle against golden vectors recorded from the MARXS reference.

Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py)
hold the reference's own outputs for seeded photon lists and the random
draws it made.  The oracle, fed those draws, must reproduce every column
bit for bit.  When the reference source tree is available, the instrument
builders are also checked against the reference's own classes.
"""
import numpy as np
import pytest

from conftest import load_golden, golden_inputs, golden_outputs, build_for_golden
from marxs_gb300 import configs
from oracle.raytrace import run_sequence


def _draws(inst, g):
    draws = {}
    for elem, kind in inst.draw_slots:
        if kind == 'scatter':
            draws[elem] = {'inplanescatter': g['draw_inplanescatter'],
                           'perpplanescatter': g['draw_perpplanescatter']}
        elif kind == 'catstack':
            draws[elem] = {k: g['draw_' + k] for k in ('order_u', 'l1_order_u', 'l1_support_u',
                                                        'l2_normal', 'l2_phi_u')}
        else:
            draws[elem] = {'order_u': g['draw_order_u']}
    return draws


@pytest.mark.parametrize('name', ['c0', 'c1', 'c2', 'c5', 'c6', 'c7', 'c8', 'c9', 'c10', 'c11'])
def test_oracle_reproduces_reference_bitwise(name):
    g = load_golden(name)
    inst = build_for_golden(name, g)
    out, stats = run_sequence(inst.elements, golden_inputs(g), _draws(inst, g))
    ref = golden_outputs(g)
    assert list(out.keys()) == [str(c) for c in g['colnames']]
    for col, b in ref.items():
        a = out[col]
        assert a.dtype == b.dtype, col
        assert np.array_equal(a, b, equal_nan=True), col
    assert stats.get('multi_hit', 0) == int(g['multi_hit'].sum())


@pytest.mark.parametrize('name', ['c1', 'c2', 'c5', 'c6', 'c8', 'c9', 'c11'])
def test_native_facet_poses_equal_reference(name):
    """Parallel.generate_elements restated on the host gives the same poses
    (C11: from the element positions the reference's RectangularGrid
    placed on its Rowland torus)."""
    g = load_golden(name)
    inst = build_for_golden(name, g)
    mine = np.array([e.geometry.pos4d for e in inst.gas.elements])
    assert np.array_equal(mine, g['facet_pos4d'])


@pytest.mark.parametrize('name', ['c7', 'c8'])
def test_native_ccd_poses_equal_reference(name):
    """The CCD poses of Parallel (C7, the reference's test layout) and of
    ParallelCalculated (C8, centres on the Rowland circle) equal the
    reference's."""
    g = load_golden(name)
    inst = configs.build(name)
    mine = np.array([e.geometry.pos4d for e in inst.detector.elements])
    assert np.array_equal(mine, g['ccd_pos4d'])


def test_ccd_workloads_are_nontrivial():
    """Every C7 chip is hit and some photons fall in the gaps; C8's strip
    catches dispersed orders on several chips."""
    ref = golden_outputs(load_golden('c7'))
    ids = ref['CCD_ID']
    assert np.array_equal(np.unique(ids), [-1, 0, 1, 2, 3])
    assert (ids == -1).mean() > 0.05
    ref = golden_outputs(load_golden('c8'))
    hit = ref['CCD'] >= 0
    assert len(np.unique(ref['CCD'][hit])) >= 10
    assert len(np.unique(ref['order'][hit & np.isfinite(ref['order'])])) >= 5


def test_golden_workloads_are_nontrivial():
    for name, lo in (('c1', 0.5), ('c2', 0.4)):
        ref = golden_outputs(load_golden(name))
        assert (ref['facet'] >= 0).mean() > lo
        orders = np.unique(ref['order'][np.isfinite(ref['order'])])
        assert len(orders) >= 10


def test_interpolated_workload_exercises_both_splines():
    """c5: the lens reflectivity lowers the probability and the interpolated
    CAT table spreads photons over many orders."""
    ref = golden_outputs(load_golden('c5'))
    inp = golden_inputs(load_golden('c5'))
    assert np.all(ref['probability'] < inp['probability'])
    orders = np.unique(ref['order'][np.isfinite(ref['order'])])
    assert len(orders) >= 10


def test_fitpack_degree1_restatement_equals_scipy():
    """bisp_k1 (FITPACK fpbisp for kx = ky = 1) against scipy's
    RectBivariateSpline.ev, inside and outside the grid, bit for bit."""
    from scipy.interpolate import RectBivariateSpline
    from oracle.raytrace import bisp_k1
    rng = np.random.default_rng(3)
    for nx, ny in ((2, 2), (5, 3), (40, 17), (100, 100)):
        x = np.sort(rng.uniform(-2, 5, nx)) if nx > 2 else np.array([0.0, 1.5])
        y = np.sort(rng.uniform(0, 0.1, ny))
        ip = RectBivariateSpline(x, y, rng.random((nx, ny)), kx=1, ky=1)
        tx, ty = ip.get_knots()
        px = np.concatenate([rng.uniform(x[0] - 1, x[-1] + 1, 3000), x, [x[0], x[-1]]])
        py = np.concatenate([rng.uniform(y[0] - 0.05, y[-1] + 0.05, 3000), y[:1].repeat(nx),
                             [y[0], y[-1]]])
        assert np.array_equal(bisp_k1(tx, ty, ip.get_coeffs(), px, py), ip.ev(px, py))


@pytest.mark.parametrize('name', ['c0', 'c1'])
def test_oracle_runs_reference_objects(reference_marxs, name):
    """Built from the reference's own classes, the oracle still matches the
    golden outputs (the oracle reads the same attributes MARXS uses)."""
    import make_golden
    g = load_golden(name)
    ns = make_golden.reference_namespace(reference_marxs)
    inst = configs.build(name, ns)
    out, _ = run_sequence(inst.elements, golden_inputs(g), _draws(inst, g))
    ref = golden_outputs(g)
    for col, b in ref.items():
        assert np.array_equal(out[col], b, equal_nan=True), col


def test_catsupportbars_semantics():
    """catsupportbars (missions/mitsnl/catgrating.py:314-324) in the oracle and
    this package's host function: facet < 0 absorbs; no facet column
    absorbs every photon."""
    from marxs_gb300 import PhotonTable
    from marxs_gb300.optics import catsupportbars
    from oracle.raytrace import support_bars
    prob = np.array([0.5, 1.0, 0.25, 0.75])
    ph = {'probability': prob.copy(), 'facet': np.array([3, -1, 0, -1])}
    assert np.array_equal(support_bars(ph)['probability'], [0.5, 0.0, 0.25, 0.0])
    assert np.array_equal(support_bars({'probability': prob.copy()})['probability'], np.zeros(4))
    t = PhotonTable({'probability': prob.copy(), 'facet': np.array([3, -1, 0, -1])})
    assert np.array_equal(np.asarray(catsupportbars(t)['probability']), [0.5, 0.0, 0.25, 0.0])
    t = PhotonTable({'probability': prob.copy()})
    assert np.array_equal(np.asarray(catsupportbars(t)['probability']), np.zeros(4))
