"""The candidate grid's depth model (host logic, no GPU).

A ray with slopes (su, sv) <= slope_max that hits a facet at X is looked up
at (u0, v0) + (su, sv) D(u0, v0), D the quadric depth model fitted to the
facet surface.  The builder grows each facet's footprint by
slope_max (max |depth - D| over the facet + L slope_max max |depth|) +
margin; these tests check that bound on random rays, the exact deviation
against dense sampling, and that the model shrinks the growth of the
Rowland-torus array.
"""
import numpy as np

from marxs_gb300 import configs
from marxs_gb300 import lowering as L


def _grating_stage(name):
    inst = configs.build(name)
    return [s for s in L.lower_elements(inst.elements) if s.grid is not None][0]


def _frame(g):
    return g['o'], g['n'], g['a'], g['b']


def _corners(f):
    return np.stack([f['c'] + (sy * f['hy'])[:, None] * f['ey'] + (sz * f['hz'])[:, None] * f['ez']
                     for sy in (-1, 1) for sz in (-1, 1)], axis=1)


def test_deviation_is_the_maximum_over_the_facet():
    st = _grating_stage('c2')
    f, g = st.facets, st.grid
    o, n, a, b = _frame(g)
    dev = L.facet_depth_deviation(f, o, n, a, b, g['depth'])
    s = np.linspace(-1, 1, 41)
    S, T = np.meshgrid(s, s)
    for k in range(0, len(f), 97):
        p = (f['c'][k] + (S[..., None] * f['hy'][k]) * f['ey'][k] +
             (T[..., None] * f['hz'][k]) * f['ez'][k] - o)
        q = np.abs(p @ n - L.depth_at(g['depth'], p @ a, p @ b))
        assert q.max() <= dev[k] + 1e-9
        assert dev[k] <= q.max() + 1e-3          # the sampled grid misses little


def test_lookup_shift_stays_within_the_growth():
    st = _grating_stage('c2')
    f, g = st.facets, st.grid
    o, n, a, b = _frame(g)
    d, lip, smax = g['depth'], g['depth_lip'], g['slope_max']
    dev = L.facet_depth_deviation(f, o, n, a, b, d)
    dmax = np.abs((_corners(f) - o) @ n).max(axis=1)
    bound = smax * (dev + lip * smax * dmax)
    rng = np.random.default_rng(4)
    m = 200000
    k = rng.integers(0, len(f), m)
    s, t = rng.uniform(-1, 1, m), rng.uniform(-1, 1, m)
    X = f['c'][k] + (s * f['hy'][k])[:, None] * f['ey'][k] + (t * f['hz'][k])[:, None] * f['ez'][k] - o
    uX, vX, hX = X @ a, X @ b, X @ n
    su, sv = rng.uniform(-smax, smax, m), rng.uniform(-smax, smax, m)
    su[:1000], sv[:1000] = smax, -smax                     # the corners of the slope box
    u0, v0 = uX - su * hX, vX - sv * hX                    # where the ray crosses the plane
    D = L.depth_at(d, u0, v0)
    u1, v1 = u0 + su * D, v0 + sv * D                      # where it is looked up
    assert np.all(np.abs(u1 - uX) <= bound[k] + 1e-9)
    assert np.all(np.abs(v1 - vX) <= bound[k] + 1e-9)


def test_depth_model_shrinks_the_torus_growth():
    st = _grating_stage('c2')
    f, g = st.facets, st.grid
    o, n, a, b = _frame(g)
    dmax = np.abs((_corners(f) - o) @ n).max(axis=1)
    dev = L.facet_depth_deviation(f, o, n, a, b, g['depth'])
    grow = g['slope_max'] * (dev + g['depth_lip'] * g['slope_max'] * dmax)
    plane = g['slope_max'] * dmax
    assert dmax.max() > 20.0                               # the torus' sagitta over the mean plane
    assert grow.max() < 0.1 * plane.max()


def test_flat_array_keeps_the_plane():
    """Fewer than six facets, or a model that does not pay: the plane."""
    st = _grating_stage('c1')
    g = st.grid
    f = st.facets
    o, n, a, b = _frame(g)
    dmax = np.abs((_corners(f) - o) @ n).max(axis=1)
    dev = L.facet_depth_deviation(f, o, n, a, b, g['depth'])
    grow = g['slope_max'] * (dev + g['depth_lip'] * g['slope_max'] * dmax)
    assert grow.max() <= g['slope_max'] * dmax.max() + 1e-12
