"""Candidate grids against the all-facet scan, on the GPU.

The grid of a facet stage only narrows the facets each ray is tested
against; the nearest hit must be the one the scan of every facet finds
(``GpuSequence.use_grid = False``), bit for bit, in both precision modes:
on the workloads' own photons and on rays aimed at random facet points,
and just past their edges, at slopes up to the grid's limit (where the
footprints' depth-model growth is tightest).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _trace(elements, host, precision, use_grid):
    from marxs_gb300 import PhotonTable
    from marxs_gb300.gpu import GpuSequence
    seq = GpuSequence(elements=elements, precision=precision, rng='philox', seed=7)
    seq.use_grid = use_grid
    return seq(PhotonTable({k: np.array(v, copy=True) for k, v in host.items()}))


def _same(a, b):
    assert list(a.colnames) == list(b.colnames)
    for col in a.colnames:
        x, y = np.asarray(a[col]), np.asarray(b[col])
        assert np.array_equal(x, y, equal_nan=x.dtype.kind == 'f'), col


@pytest.mark.parametrize('precision', ['fp64', 'fp32local'])
@pytest.mark.parametrize('name', ['c2', 'c8'])
def test_grid_matches_all_facet_scan(name, precision):
    from marxs_gb300 import configs
    inst = configs.build(name)
    host = configs.photons_for(name, 100000, seed=31)
    _same(_trace(inst.elements, host, precision, True),
          _trace(inst.elements, host, precision, False))


@pytest.mark.parametrize('precision', ['fp64', 'fp32local'])
def test_grid_matches_scan_at_the_slope_limit(precision):
    from marxs_gb300 import configs
    from marxs_gb300 import lowering as L
    inst = configs.build('c2')
    gas = inst.gas
    st = [s for s in L.lower_elements([gas]) if s.grid is not None][0]
    f, g = st.facets, st.grid
    n, a, b, smax = g['n'], g['a'], g['b'], g['slope_max']
    rng = np.random.default_rng(33)
    m = 200000
    k = rng.integers(0, len(f), m)
    # points on the facets and up to 2 mm past their edges
    s = rng.uniform(-1, 1, m) * (1 + 2.0 / f['hy'][k])
    t = rng.uniform(-1, 1, m) * (1 + 2.0 / f['hz'][k])
    X = f['c'][k] + (s * f['hy'][k])[:, None] * f['ey'][k] + (t * f['hz'][k])[:, None] * f['ez'][k]
    su = rng.uniform(-1, 1, m) * smax * (1 - 1e-7)
    sv = rng.uniform(-1, 1, m) * smax * (1 - 1e-7)
    su[: m // 10] = np.sign(su[: m // 10]) * smax * (1 - 1e-7)   # the slope limit itself
    sv[: m // 10] = np.sign(sv[: m // 10]) * smax * (1 - 1e-7)
    beam = -1.0 if n[0] > 0 else 1.0                               # the C2 beam runs along -x
    d = beam * n[None, :] + su[:, None] * a + sv[:, None] * b
    d /= np.linalg.norm(d, axis=1)[:, None]
    pos = X - 200.0 * d
    pol = np.cross(d, np.array([0.0, 0.0, 1.0]))
    pol /= np.linalg.norm(pol, axis=1)[:, None]
    e = configs.photons_for('c2', m, seed=35)['energy']
    host = {'pos': np.c_[pos, np.ones(m)], 'dir': np.c_[d, np.zeros(m)],
            'polarization': np.c_[pol, np.zeros(m)], 'energy': e, 'probability': np.ones(m)}
    a_ = _trace([gas], host, precision, True)
    b_ = _trace([gas], host, precision, False)
    assert (np.asarray(b_['facet']) >= 0).mean() > 0.5
    _same(a_, b_)
