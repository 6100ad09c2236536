"""The analysis oracle (per-order resolving power, effective area,
CaptureResAeff, average_R_Aeff, sigma-clipped statistics) against the
reference's own analysis functions (golden vectors recorded from
marxs/analysis/gratings.py under the test shims) and against the reference's
statistical tests (analysis/tests/test_grating.py:16-80)."""
import numpy as np
import pytest

from conftest import load_golden
from oracle import analysis as A


def _same(a, b):
    return np.array_equal(np.asarray(a, dtype=float), np.asarray(b, dtype=float), equal_nan=True)


def test_resolvingpower_matches_reference():
    g = load_golden('analysis')
    for zeropos, key in ((None, 'rp'), (0.5, 'rpz')):
        res, pos, std = A.resolvingpower_from_photonlist(g['order'], g['det_x'], g['orders'],
                                                         zeropos=zeropos)
        assert _same(res, g[key + '_res'])
        assert _same(pos, g[key + '_pos'])
        assert _same(std, g[key + '_std'])
    # the > 20 rule: order 9 has 20 photons, order 10 has 21
    assert np.isnan(g['rp_pos'][19]) and np.isfinite(g['rp_pos'][20])


def test_effective_area_matches_reference():
    g = load_golden('analysis')
    aeff = A.effectivearea_from_photonlist(g['order'], g['probability'], g['orders'],
                                           len(g['order']), A_geom=2.)
    assert _same(aeff, g['aeff'])


def test_capture_res_aeff_matches_reference():
    g = load_golden('analysis')
    cap = A.capture_res_aeff(g['order'], g['det_x'], g['probability'], g['orders'], A_geom=3.)
    ccd = A.capture_res_aeff(g['order'], g['det_x'], g['probability'], g['orders'], A_geom=3.,
                             aeff_mask=g['CCD_ID'] >= 0)
    for name, out in (('cap', cap), ('ccd', ccd)):
        for k in ('Aeff0', 'Aeffgrat', 'Aeff', 'Rgrat', 'R'):
            got = np.ma.filled(np.ma.asarray(out[k], dtype=float), np.nan)
            assert _same(got, g['%s_%s' % (name, k)]), (name, k)
    few = A.capture_res_aeff(g['few_order'], g['det_x'], g['probability'], g['orders'])
    assert _same(few['R'], g['few_R']) and np.all(np.isnan(few['R']))
    assert _same(few['Aeff'], g['few_Aeff'])


def test_average_R_Aeff_matches_reference():
    from marxs_gb300.analysis import average_R_Aeff
    g = load_golden('analysis')
    for ax, key in ((None, 'none'), (0, '0'), (2, '2')):
        for fn in (A.average_R_Aeff, average_R_Aeff):
            r, a = fn(g['avg_r_in'], g['avg_aeff_in'], axis=ax)
            assert _same(np.ma.filled(np.ma.asarray(r, dtype=float), np.nan), g['avg_r_' + key])
            assert _same(a, g['avg_aeff_' + key])


def test_sigma_clip_known_answers():
    # one far outlier among zeros: removed in iteration 1, iteration 2 removes nothing
    mean, med, std, n, it = A.sigma_clipped_stats(np.r_[np.zeros(10), 1e6])
    assert (mean, med, std, n, it) == (0.0, 0.0, 0.0, 10, 2)
    # constant data: nothing removed
    assert A.sigma_clipped_stats(np.full(7, 2.5)) == (2.5, 2.5, 0.0, 7, 1)
    # non-finite values are dropped before clipping; even count -> mean of the middle two
    mean, med, std, n, it = A.sigma_clipped_stats([1., np.nan, 2., np.inf, 4., 3.])
    assert (med, n) == (2.5, 4) and mean == 2.5
    # empty
    assert np.isnan(A.sigma_clipped_stats([])[0])
    # maxiters bounds the loop
    x = np.r_[np.arange(100.), 1e3, 1e5, 1e7]
    assert A.sigma_clipped_stats(x, maxiters=1)[4] == 1
    assert A.sigma_clipped_stats(x, maxiters=1)[3] == 102


def test_reference_statistical_cases():
    """analysis/tests/test_grating.py:47-80 restated on the oracle."""
    rng = np.random.default_rng(0)
    size = 10000
    orders = [1, 2, 3]
    order = rng.choice(orders, size=size)
    col1 = 2000 + rng.normal(size=size)
    col2 = 1000 + rng.normal(size=size)
    res, pos, std = A.resolvingpower_from_photonlist(order, col1, orders, zeropos=0)
    assert res == pytest.approx(2000 / 2.3548 * np.ones(3), rel=1e-1)
    assert std == pytest.approx(np.ones(3), rel=1e-1)
    res, pos, std = A.resolvingpower_from_photonlist(order, col2, orders, zeropos=-1000)
    assert res == pytest.approx(2000 / 2.3548 * np.ones(3), rel=1e-1)
    order0 = rng.choice([0, 1, 2], size=size)
    col1[order0 == 0] = 0
    res, pos, std = A.resolvingpower_from_photonlist(order0, col1, [1, 2])
    assert res == pytest.approx(2000 / 2.3548 * np.ones(2), rel=1e-1)
    with pytest.raises(A.AnalysisError):
        A.resolvingpower_from_photonlist(np.ones(100), col1[:100], [1])
