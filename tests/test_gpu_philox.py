"""In-kernel Philox randomness: distributions match the reference algorithm.

With ``rng='philox'`` the kernels draw their own uniforms and normals, so
results cannot equal the oracle photon by photon; they must follow the same
distributions.  The oracle is driven by numpy draws of the reference's
distributions (U[0,1) for orders, sigma * N(0,1) for scatter angles) on the
same photon inputs, and two-sample tests compare:
* the order histogram (chi-square), per precision mode;
* detector positions det_x / det_y (Kolmogorov-Smirnov);
* the drawn scatter angles against N(0, sigma) (KS).
Significance threshold p > 1e-3 for each test.
"""
import numpy as np
import pytest
from scipy import stats

pytestmark = pytest.mark.gpu

N = 200000


def _gpu(inst, host, precision, seed=1234):
    from marxs_gb300 import PhotonTable
    from marxs_gb300.gpu import GpuSequence
    seq = GpuSequence(elements=inst.elements, precision=precision, rng='philox', seed=seed)
    return seq(PhotonTable({k: np.array(v, copy=True) for k, v in host.items()}))


def _oracle(inst, host, seed):
    from marxs_gb300 import configs
    from oracle.raytrace import run_sequence
    n = len(host['energy'])
    out, _ = run_sequence(inst.elements, host, configs.draws_for(inst.draw_slots, n, seed))
    return out


@pytest.fixture(scope='module')
def c1_runs():
    from marxs_gb300 import configs
    inst = configs.build('c1')
    host = configs.photons_for('c1', N, seed=31)
    return inst, host, _oracle(inst, host, 97)


@pytest.mark.parametrize('precision', ['fp64', 'fp32local'])
def test_order_distribution(c1_runs, precision):
    inst, host, ref = c1_runs
    out = _gpu(inst, host, precision)
    orders = np.arange(-10, 3)
    a = np.array([(np.asarray(out['order']) == m).sum() for m in orders])
    b = np.array([(ref['order'] == m).sum() for m in orders])
    chi2, p, _, _ = stats.chi2_contingency(np.vstack([a, b]))
    assert p > 1e-3, (p, a, b)


@pytest.mark.parametrize('precision', ['fp64', 'fp32local'])
def test_detector_position_distribution(c1_runs, precision):
    inst, host, ref = c1_runs
    out = _gpu(inst, host, precision)
    for col in ('det_x', 'det_y'):
        a = np.asarray(out[col])
        b = ref[col]
        a, b = a[np.isfinite(a)], b[np.isfinite(b)]
        assert abs(len(a) - len(b)) < 5 * np.sqrt(len(b))     # hit counts agree
        res = stats.ks_2samp(a, b)
        assert res.pvalue > 1e-3, (col, res)


@pytest.mark.parametrize('precision', ['fp64', 'fp32local'])
def test_scatter_angles_are_gaussian(precision):
    from marxs_gb300 import configs
    inst = configs.build('c0')
    host = configs.photons_for('c0', N, seed=5)
    out = _gpu(inst, host, precision, seed=77)
    for col, sigma in (('inplanescatter', inst.scatter.inplanescatter),
                       ('perpplanescatter', inst.scatter.perpplanescatter)):
        x = np.asarray(out[col]) / sigma
        res = stats.kstest(x, 'norm')
        assert res.pvalue > 1e-3, (col, res)
        assert abs(np.std(x) - 1) < 0.01


def test_philox_streams_are_keyed_by_global_photon_id():
    """Tracing two halves with their row offsets equals tracing the whole."""
    from marxs_gb300 import configs, PhotonTable
    from marxs_gb300.gpu import GpuSequence
    inst = configs.build('c2')
    n = 20000
    host = configs.photons_for('c2', n, seed=8)
    seq = GpuSequence(elements=inst.elements, precision='fp64', rng='philox', seed=5)
    whole = seq(PhotonTable({k: v.copy() for k, v in host.items()}))
    h = n // 2
    a = seq(PhotonTable({k: v[:h].copy() for k, v in host.items()}), row_base=0)
    b = seq(PhotonTable({k: v[h:].copy() for k, v in host.items()}), row_base=h)
    for col in ('pos', 'dir', 'order', 'facet', 'det_phi'):
        joined = np.concatenate([np.asarray(a[col]), np.asarray(b[col])])
        assert np.array_equal(joined, np.asarray(whole[col]), equal_nan=True), col


def test_cat_stack_distributions():
    """CATL1L2Stack facets with in-kernel draws: membrane and L1 order
    histograms (chi-square) and L2 scatter angles (KS) follow the oracle fed
    numpy draws of the reference distributions."""
    from marxs_gb300 import configs
    inst = configs.build('c6')
    n = 30000
    host = configs.photons_for('c6', n, seed=13)
    out = _gpu(inst, host, 'fp64', seed=21)
    ref = _oracle(inst, host, 44)
    for col, orders in (('order', np.arange(-12, 3)), ('order_L1', np.arange(-4, 5))):
        a = np.array([(np.asarray(out[col]) == m).sum() for m in orders])
        b = np.array([(ref[col] == m).sum() for m in orders])
        keep = (a + b) > 0
        chi2, p, _, _ = stats.chi2_contingency(np.vstack([a[keep], b[keep]]))
        assert p > 1e-3, (col, p, a, b)
    x = np.asarray(out['L2Diffraction'])
    y = ref['L2Diffraction']
    x, y = x[np.isfinite(x)], y[np.isfinite(y)]
    assert abs(len(x) - len(y)) < 5 * np.sqrt(len(y))
    assert stats.ks_2samp(x, y).pvalue > 1e-3
