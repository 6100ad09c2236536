"""Per-order analysis reductions on the GPU (mgpu_order_stats) against the
oracle and the reference-recorded golden vectors.

Tolerances: the median is an exact order statistic (compared with ==);
counts and clipping rounds are exact; means and effective-area sums are
sums in a different order than numpy's pairwise sum (rel 1e-12); the std
is the square root of a second such sum (rel 1e-10); derived resolving
powers rel 1e-9.
"""
import numpy as np
import pytest
import torch

from conftest import load_golden
from oracle import analysis as A

pytestmark = pytest.mark.gpu

MEAN, MEDIAN, STD, N_CLIP, N_MEMBER, AEFF, N_FINITE, ROUNDS = range(8)


def _close(a, b, rel, abs_=0.0):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    assert np.array_equal(np.isnan(a), np.isnan(b)), (a, b)
    m = ~np.isnan(a)
    assert np.all(np.abs(a[m] - b[m]) <= rel * np.abs(b[m]) + abs_), (a[m], b[m])


def _oracle_rows(order, value, prob, orders, res_filter=False, aeff_mask=None):
    rows = []
    for o in orders:
        grp = (order == o)
        val = value[grp]
        if res_filter:
            keep = np.isfinite(val) & (prob[grp] > 0)
            member, val = keep.sum(), val[keep]
        else:
            member = grp.sum()
        mean, med, std, n, it = A.sigma_clipped_stats(val)
        am = grp if aeff_mask is None else grp & aeff_mask
        rows.append((mean, med, std, n, member, prob[am].sum(), np.isfinite(val).sum(), it))
    return np.array(rows, dtype=float)


def _compare(got, ref):
    assert np.array_equal(got[:, N_CLIP], ref[:, N_CLIP])
    assert np.array_equal(got[:, N_MEMBER], ref[:, N_MEMBER])
    assert np.array_equal(got[:, N_FINITE], ref[:, N_FINITE])
    assert np.array_equal(got[:, ROUNDS], ref[:, ROUNDS]), (got[:, ROUNDS], ref[:, ROUNDS])
    assert np.array_equal(got[:, MEDIAN], ref[:, MEDIAN], equal_nan=True)
    _close(got[:, MEAN], ref[:, MEAN], 1e-12, 1e-300)
    _close(got[:, STD], ref[:, STD], 1e-10, 1e-300)
    _close(got[:, AEFF], ref[:, AEFF], 1e-12, 1e-300)


def _event_list(seed, n):
    """Orders -8..3 with NaN (no hit), Gaussian lines with Cauchy outliers,
    quantised values (ties) in order 3, mixed-sign values in order 0,
    non-finite positions, zero probabilities."""
    rng = np.random.default_rng(seed)
    order = rng.integers(-8, 4, n).astype(float)
    order[rng.random(n) < 0.05] = np.nan
    x = 25. * np.nan_to_num(order) + rng.normal(0, 0.05, n)
    out = rng.random(n) < 0.02
    x[out] += rng.standard_cauchy(out.sum())
    x[order == 3] = np.round(x[order == 3], 2)
    x[order == 0] = rng.normal(0, 1e-3, (order == 0).sum())
    x[rng.random(n) < 0.01] = np.nan
    x[rng.random(n) < 0.002] = np.inf
    prob = rng.random(n)
    prob[rng.random(n) < 0.05] = 0.0
    return order, x, prob


def test_order_stats_matches_oracle_per_group():
    from marxs_gb300.analysis import order_stats
    order, x, prob = _event_list(1, 300_000)
    orders = [-8, -7, -6, -5, -4, -3, -2, -1, 0, 1, 2, 3, 7]      # 7: no photons
    for res_filter in (False, True):
        got = order_stats(x, order, orders, probability=prob, res_filter=res_filter)
        _compare(got, _oracle_rows(order, x, prob, orders, res_filter))
    assert np.all(np.isnan(got[-1, :3])) and got[-1, N_MEMBER] == 0


def test_order_stats_integer_orders_masks_and_strided_columns():
    from marxs_gb300.analysis import order_stats
    order, x, prob = _event_list(2, 100_000)
    iorder = np.nan_to_num(order, nan=-99).astype(np.int64)
    mask = np.random.default_rng(3).random(len(x)) < 0.8
    orders = [-3, 0, 2]
    ref = _oracle_rows(iorder, x, prob, orders, aeff_mask=mask)
    for dt in (torch.int32, torch.int64):
        got = order_stats(torch.from_numpy(x).cuda(), torch.from_numpy(iorder).to(dt).cuda(),
                          orders, probability=prob, aeff_mask=mask)
        _compare(got, ref)
    # a column of an (N, 4) array read through its stride
    arr = torch.zeros((len(x), 4), dtype=torch.float64, device='cuda')
    arr[:, 2] = torch.from_numpy(x)
    got = order_stats(arr[:, 2], iorder, orders, probability=prob, aeff_mask=mask)
    _compare(got, ref)
    # repeated orders give repeated rows
    got = order_stats(x, iorder, [2, -3, 2], probability=prob)
    assert np.array_equal(got[0], got[2], equal_nan=True)


@pytest.mark.parametrize('data', [
    np.array([]),
    np.array([3.5]),
    np.array([2.0, -1.0]),
    np.full(1000, -7.25),
    np.r_[np.zeros(10), 1e6],
    np.r_[-0.0, 0.0, -0.0, 1e-300, -1e-300],
    np.r_[np.random.default_rng(4).normal(0, 1, 999), -1e150, 1e150],
    np.r_[np.random.default_rng(5).normal(-5, 1, 4096), np.nan, -np.inf],
    np.random.default_rng(6).integers(0, 3, 10_001).astype(float),
])
def test_sigma_clipped_stats_edge_cases(data):
    from marxs_gb300 import _abi
    from marxs_gb300.analysis import order_stats, sigma_clipped_stats
    mean, med, std, n, it = A.sigma_clipped_stats(data)
    r = order_stats(data)[0]
    assert r[_abi.STATS_N_CLIP] == n
    if n:
        assert r[_abi.STATS_ROUNDS] == it
    got = sigma_clipped_stats(data)
    assert got[1] == med or (np.isnan(got[1]) and np.isnan(med))
    _close([got[0]], [mean], 1e-12, 1e-300)
    _close([got[2]], [std], 1e-10, 1e-300)


def test_maxiters_and_sigma():
    from marxs_gb300.analysis import order_stats
    rng = np.random.default_rng(7)
    x = np.r_[rng.normal(0, 1, 5000), rng.standard_cauchy(500) * 10]
    for sigma, maxiters in ((3.0, 1), (3.0, 2), (2.0, 5), (1.5, 10)):
        got = order_stats(x, sigma=sigma, maxiters=maxiters)[0]
        mean, med, std, n, it = A.sigma_clipped_stats(x, sigma=sigma, maxiters=maxiters)
        assert (got[N_CLIP], got[ROUNDS], got[MEDIAN]) == (n, it, med)
        _close([got[MEAN], got[STD]], [mean, std], 1e-10)


def test_order_stats_is_deterministic():
    from marxs_gb300.analysis import order_stats
    order, x, prob = _event_list(8, 500_000)
    a = order_stats(x, order, list(range(-8, 4)), probability=prob, res_filter=True)
    b = order_stats(x, order, list(range(-8, 4)), probability=prob, res_filter=True)
    assert np.array_equal(a, b, equal_nan=True)


def test_large_list_matches_oracle():
    """2e7 photons, eleven orders of 1.8e6 values each."""
    from marxs_gb300.analysis import order_stats
    order, x, prob = _event_list(9, 20_000_000)
    orders = list(range(-8, 3))
    got = order_stats(torch.from_numpy(x).cuda(), torch.from_numpy(order).cuda(), orders,
                      probability=torch.from_numpy(prob).cuda(), res_filter=True)
    _compare(got, _oracle_rows(order, x, prob, orders, res_filter=True))


def test_reference_golden_through_device_api():
    from marxs_gb300 import analysis as G
    g = load_golden('analysis')
    photons = {k: g[k] for k in ('order', 'det_x', 'probability', 'CCD_ID')}
    for zeropos, key in ((None, 'rp'), (0.5, 'rpz')):
        res, pos, std = G.resolvingpower_from_photonlist(photons, g['orders'], col='det_x',
                                                         zeropos=zeropos)
        _close(pos, g[key + '_pos'], 1e-12, 1e-15)
        _close(std, g[key + '_std'], 1e-10)
        _close(res, g[key + '_res'], 1e-9, 1e-9)
    aeff = G.effectivearea_from_photonlist(photons, g['orders'], len(g['order']), A_geom=2.)
    _close(aeff, g['aeff'], 1e-12)
    dev = {k: torch.from_numpy(np.ascontiguousarray(v)).cuda() for k, v in photons.items()}
    for src in (photons, dev):
        for name, cap in (('cap', G.CaptureResAeff(A_geom=3., orders=g['orders'],
                                                   dispersion_coord='det_x')),
                          ('ccd', G.CaptureResAeff_CCDgaps(aeff_filter_col='CCD_ID', A_geom=3.,
                                                           orders=g['orders'],
                                                           dispersion_coord='det_x'))):
            out = cap(src)
            for k, rel in (('Aeff0', 1e-12), ('Aeffgrat', 1e-12), ('Aeff', 1e-12),
                           ('Rgrat', 1e-9), ('R', 1e-9)):
                got = np.ma.filled(np.ma.asarray(out[k], dtype=float), np.nan)
                _close(np.atleast_1d(got), np.atleast_1d(g['%s_%s' % (name, k)]), rel, 1e-12)
    few = dict(photons, order=g['few_order'])
    out = G.CaptureResAeff(orders=g['orders'], dispersion_coord='det_x')(few)
    assert np.all(np.isnan(out['R']))
    _close(out['Aeff'], g['few_Aeff'], 1e-12)
    with pytest.raises(G.AnalysisError):
        G.resolvingpower_from_photonlist(few, g['orders'], col='det_x')


def test_reference_statistical_cases_on_device():
    """analysis/tests/test_grating.py:47-80 through the device API."""
    from marxs_gb300.analysis import resolvingpower_from_photonlist
    rng = np.random.default_rng(10)
    size = 10000
    photons = {'col1': 2000 + rng.normal(size=size), 'col2': 1000 + rng.normal(size=size),
               'order': rng.choice([1, 2, 3], size=size)}
    res, pos, std = resolvingpower_from_photonlist(photons, [1, 2, 3], 'col1', zeropos=0)
    assert res == pytest.approx(2000 / 2.3548 * np.ones(3), rel=1e-1)
    assert pos == pytest.approx(2000 * np.ones(3), rel=1e-1)
    assert std == pytest.approx(np.ones(3), rel=1e-1)


def test_capture_on_traced_device_columns():
    """The event columns that trace_device leaves on the device, reduced in
    place, against the oracle on host copies."""
    from marxs_gb300 import configs
    from marxs_gb300.analysis import CaptureResAeff
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    from marxs_gb300.source import CircleAperture, DeviceSource
    inst = configs.build('c2')
    ap = CircleAperture(position=[12000., 0, 0], zoom=[1, 500, 500], r_inner=300.)
    src = DeviceSource(ap, energy=0.5)
    seq = GpuSequence(inst.elements, precision='fp32local', rng='philox', seed=4)
    n = 400_000
    ph = src.generate(n, seed=12)
    plan, bufs = seq.allocate_columns(n)
    status, _ = seq.trace_device(ph, ph, plan, bufs)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    cols = {'order': bufs['order'], 'det_phi': bufs['det_phi'], 'probability': ph.prob}
    orders = np.arange(-10, 1)
    out = CaptureResAeff(orders=orders, dispersion_coord='det_phi')(cols)
    host = {k: v.cpu().numpy() for k, v in cols.items()}
    ref = A.capture_res_aeff(host['order'], host['det_phi'], host['probability'], orders)
    for k, rel in (('Aeff', 1e-12), ('R', 1e-9), ('Rgrat', 1e-9)):
        _close(np.atleast_1d(np.ma.filled(np.ma.asarray(out[k], dtype=float), np.nan)),
               np.atleast_1d(np.ma.filled(np.ma.asarray(ref[k], dtype=float), np.nan)), rel, 1e-12)
    assert np.nanmax(out['R']) > 100


def test_order_matching_beyond_the_small_integer_table():
    """Orders outside [-64, 64] and non-integral orders go through the
    linear match; integer and float columns agree with the oracle."""
    from marxs_gb300.analysis import order_stats
    rng = np.random.default_rng(12)
    n = 60_000
    pool = np.array([-100., -3., 0., 2.5, 7., 64., 65., 1e6])
    order = rng.choice(pool, n)
    x = rng.normal(0, 1, n) + order
    prob = rng.random(n)
    orders = [65., -3., 2.5, 1e6, 64., 0., -100., 7., 8.]
    got = order_stats(x, order, orders, probability=prob)
    _compare(got, _oracle_rows(order, x, prob, orders))
    iorder = np.where(np.isin(order, [2.5]), 99, order).astype(np.int64)
    iorders = [65, -3, 99, 1000000, 64, 0, -100, 7, 2.5]
    got = order_stats(x, iorder, iorders, probability=prob)
    _compare(got, _oracle_rows(iorder, x, prob, iorders))


def test_masked_columns_leave_out_masked_values():
    """A masked dispersion column (astropy MaskedColumn semantics): masked
    entries are left out of the statistics like non-finite ones, and still
    count as order members without the resolving-power filter."""
    from marxs_gb300.analysis import order_stats
    order, x, prob = _event_list(13, 50_000)
    mask = np.random.default_rng(14).random(len(x)) < 0.1
    xm = np.ma.MaskedArray(x, mask=mask)
    got = order_stats(xm, order, [-3, 0, 2], probability=prob)
    ref = _oracle_rows(order, np.where(mask, np.nan, x), prob, [-3, 0, 2])
    _compare(got, ref)
