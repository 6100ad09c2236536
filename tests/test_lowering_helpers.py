"""Host-made constants of the FP32-local chain (no GPU): the exactness the
kernels rely on when they decide on integers instead of float64."""
import numpy as np
import pytest

from marxs_gb300 import lowering as L


@pytest.mark.parametrize('x', [0.0, 0.25, 0.3, 0.5, 0.7853981633974483, 0.9999999999999999, 1.0,
                               1.5, -0.2, 2.0 ** -60, 0.1 + 2.0 ** -54])
def test_u53_threshold_decides_u_greater_than_x_exactly(x):
    """For a 53-bit draw U (u = U * 2^-53, exact in float64), u > x exactly
    when U > u53_threshold(x) -- the float64 kernel's comparison."""
    t = L.u53_threshold(x)
    rng = np.random.default_rng(5)
    U = rng.integers(0, 2 ** 53, size=20000, dtype=np.int64)
    near = np.clip(np.array([t - 2, t - 1, t, t + 1, t + 2], dtype=np.int64), 0, 2 ** 53 - 1)
    U = np.concatenate([U, near])
    u = U.astype(np.float64) * 2.0 ** -53
    assert np.array_equal(u > x, U > t)


def test_u53_threshold_bounds():
    assert L.u53_threshold(-5.0) == -1
    assert L.u53_threshold(float('inf')) >= 2 ** 53
    assert L.u53_threshold(float('-inf')) == -1


class _Sel:
    def __init__(self, energy, n_orders=3):
        self.energy = np.asarray(energy, dtype=np.float64)
        self.by_energy = True
        cdf = np.cumsum(np.full((len(energy), n_orders), 1.0 / n_orders), axis=1)
        self.cdf = cdf


def test_selector_rows32_midpoints_give_the_nearest_row():
    """Row j+1 when e > mid_j reproduces argmin |E - e| (first index on a
    tie) for e anywhere in the table."""
    rng = np.random.default_rng(8)
    E = np.sort(rng.uniform(0.2, 2.0, 64))
    mid, e0, scale = L.selector_rows32(_Sel(E))
    assert mid.dtype == np.float64 and len(mid) == len(E) - 1
    assert e0 == np.float32(E[0]) and scale == np.float32(63 / (E[-1] - E[0]))
    e = np.concatenate([rng.uniform(E[0], E[-1], 50000), E, mid])
    lo = np.searchsorted(E, e, side='right') - 1            # largest j with E_j <= e
    lo = np.clip(lo, 0, len(E) - 1)
    nxt = np.minimum(lo + 1, len(E) - 1)
    row = np.where((lo + 1 < len(E)) & (e > mid[np.minimum(lo, len(mid) - 1)]), nxt, lo)
    want = np.argmin(np.abs(E[None, :] - e[:, None]), axis=1)
    # exact midpoints are ties of |E - e| up to rounding: both rows are nearest
    tie = np.isin(e, mid)
    assert np.array_equal(row[~tie], want[~tie])
    d_row = np.abs(E[row] - e)
    d_want = np.abs(E[want] - e)
    assert np.all(np.abs(d_row[tie] - d_want[tie]) <= 4e-16 * np.abs(e[tie]))


def test_selector_rows32_only_for_sorted_energy_rows():
    assert L.selector_rows32(_Sel([1.0])) is None
    assert L.selector_rows32(_Sel([1.0, 0.5, 2.0])) is None
    s = _Sel([0.5, 1.0])
    s.by_energy = False
    assert L.selector_rows32(s) is None


def test_split_ff_array_round_trip():
    rng = np.random.default_rng(3)
    x = np.concatenate([rng.uniform(-1e4, 1e4, 1000), [0.0, 1.0, 2.0 ** -40, 7.123456789012345]])
    p = L.split_ff_array(x)
    assert p.dtype == np.float32 and p.shape == (len(x), 2)
    back = p[:, 0].astype(np.float64) + p[:, 1].astype(np.float64)
    assert np.all(np.abs(back - x) <= 2.0 ** -46 * np.abs(x))
    # the pairs keep the order of the float64 values (knot searches rely on it)
    xs = np.sort(x)
    ps = L.split_ff_array(xs)
    key = [(a, b) for a, b in ps]
    assert key == sorted(key)


class _FakeSpline:
    degrees = (1, 1)

    def __init__(self, tx, ty):
        self.tx, self.ty = np.asarray(tx, float), np.asarray(ty, float)

    def get_knots(self):
        return self.tx, self.ty

    def get_coeffs(self):
        return np.zeros((len(self.tx) - 2) * (len(self.ty) - 2))


def test_spline_tables_need_two_grid_points_per_axis():
    ok = _FakeSpline([0, 0, 1, 1], [0, 0, 2, 2])
    tx, ty, c = L.spline1_arrays(ok, 'test')
    assert len(tx) == 4 and c.size == 4
    with pytest.raises(NotImplementedError):
        L.spline1_arrays(_FakeSpline([0, 0, 0], [0, 0, 1, 1]), 'test')
    with pytest.raises(NotImplementedError):
        L.spline1_arrays(_FakeSpline([0, 0, 2, 1, 1], [0, 0, 1, 1]), 'test')
    from scipy.interpolate import RectBivariateSpline
    sp = RectBivariateSpline([0., 1.], [0., 1., 2.], np.ones((2, 3)), kx=1, ky=1)
    tx, ty, c = L.spline1_arrays(sp, 'scipy')
    assert len(tx) == 4 and len(ty) == 5 and c.size == 6


def test_order_selectors_and_tables_are_checked():
    from marxs_gb300.optics import OrderSelector, EfficiencyFile
    spec = L.lower_selector(OrderSelector([0, 1, 2], p=[0.2, 0.3, 0.5]))
    assert spec.cdf.shape == (1, 3) and spec.total[0] == pytest.approx(1.0)
    with pytest.raises(ValueError):
        L.lower_selector(OrderSelector([]))
    with pytest.raises(ValueError):
        L._interp_table([], [])
    with pytest.raises(ValueError):
        L._interp_table([1.0, 0.5], [0.1, 0.2])
    x, y = L._interp_table([0.5], [0.3])
    assert x[0] == 0.5 and y[0] == 0.3


@pytest.mark.parametrize('name, kinds', [('c0', [1, 2, 3]), ('c1', [1, 2, 4, 3]),
                                         ('c2', [1, 2, 4, 5]), ('c5', [1, 2, 4, 5]),
                                         ('c6', [1, 2, 4, 6, 5])])
def test_every_workload_lowers_on_the_host(name, kinds):
    """Lowering (stage descriptors, facet tables, candidate grid parameters,
    selector and stack tables) is host work and runs without a GPU."""
    from marxs_gb300 import configs
    stages = L.lower_elements(configs.build(name).elements)
    assert [s.kind for s in stages] == kinds
    for st in stages:
        if st.facets is not None:
            assert len(st.facets) > 0 and st.grid is not None
            assert st.grid['nu'] * st.grid['nv'] <= 1 << 20


@pytest.mark.parametrize('name', ['c0', 'c1', 'c2', 'c5', 'c6'])
def test_column_plan_reproduces_the_reference_columns(name):
    """The column plan (which stage creates which column, in which order,
    float or id) gives the reference's own output table: the column names in
    the order MARXS created them (add_output_cols, base/base.py:249-286) and
    their kinds, as recorded in the golden fixture."""
    import sys
    import os
    sys.path.insert(0, os.path.dirname(__file__))
    from conftest import load_golden, golden_inputs, golden_outputs
    from marxs_gb300 import configs
    from marxs_gb300.gpu import ColumnPlan
    g = load_golden(name)
    inputs = list(golden_inputs(g))
    stages = L.lower_elements(configs.build(name).elements)
    plan = ColumnPlan(stages, existing=set(inputs))
    cols = list(inputs)
    for names in plan.order:            # every stage hits photons in the fixture
        for c in names:
            if c not in cols:
                cols.append(c)
    assert cols == [str(c) for c in g['colnames']]
    out = golden_outputs(g)
    for c, kind in plan.columns.items():
        want = np.float64 if kind == 'f8' else np.integer
        assert np.issubdtype(out[c].dtype, want), (c, kind, out[c].dtype)
