"""Host logic of the analysis wrappers (no GPU): the per-order step that
turns the device's per-group statistics into the reference's resolving
power, position and width (analysis/gratings.py:215-270), and the
Aeff-weighted average (:180-212), against the oracle."""
import numpy as np
import pytest

from marxs_gb300 import _abi
from marxs_gb300 import analysis as A
from oracle import analysis as O


def _device_like_stats(order, value, groups):
    """The rows mgpu_order_stats returns, filled from the oracle's clipped
    statistics (mean, std) and the group sizes."""
    r = np.full((len(groups), _abi.STATS_NRES), np.nan)
    for g, o in enumerate(groups):
        ind = order == o
        mean, median, std, n, it = O.sigma_clipped_stats(value[ind])
        r[g, _abi.STATS_MEAN], r[g, _abi.STATS_MEDIAN], r[g, _abi.STATS_STD] = mean, median, std
        r[g, _abi.STATS_N_CLIP] = n
        r[g, _abi.STATS_N_MEMBER] = ind.sum()
    return r


@pytest.mark.parametrize('zeropos', [None, 0.25])
def test_per_order_matches_the_reference_loop(zeropos):
    rng = np.random.default_rng(4)
    orders = np.array([-3, -2, -1, 1, 2])
    sizes = {-3: 500, -2: 21, -1: 20, 0: 300, 1: 5, 2: 800}     # 20 or fewer -> NaN
    order = np.concatenate([np.full(k, o) for o, k in sizes.items()]).astype(float)
    value = rng.normal(order * 3.0, 0.2 + 0.05 * np.abs(order))
    value[::37] = np.nan
    groups = list(orders.astype(float)) + ([0.0] if zeropos is None else [])
    r = _device_like_stats(order, value, groups)
    res, pos, std = A._per_order(r, zeropos, orders)
    want = O.resolvingpower_from_photonlist(order, value, orders, zeropos)
    for a, b in zip((res, pos, std), want):
        assert np.array_equal(np.isnan(a), np.isnan(b))
        m = ~np.isnan(b)
        np.testing.assert_allclose(a[m], b[m], rtol=1e-14)
    assert np.isnan(res[orders == -1]) and np.isfinite(res[orders == -2])


def test_per_order_needs_twenty_order_zero_photons():
    order = np.concatenate([np.zeros(19), np.full(100, 1.0)])
    value = np.linspace(0, 1, len(order))
    r = _device_like_stats(order, value, [1.0, 0.0])
    with pytest.raises(A.AnalysisError):
        A._per_order(r, None, np.array([1]))
    with pytest.raises(O.AnalysisError):
        O.resolvingpower_from_photonlist(order, value, np.array([1]))


def test_average_R_Aeff_matches_the_reference():
    rng = np.random.default_rng(6)
    r = rng.uniform(500, 2000, (4, 7))
    r[1, 3] = np.nan
    aeff = rng.uniform(0, 1, (4, 7))
    for axis in (None, 0, 1):
        a = A.average_R_Aeff(r, aeff, axis=axis)
        b = O.average_R_Aeff(r, aeff, axis=axis)
        np.testing.assert_allclose(np.ma.filled(a[0], np.nan), np.ma.filled(b[0], np.nan))
        np.testing.assert_allclose(a[1], b[1])
