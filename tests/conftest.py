import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, 'tests', 'golden')
for p in (ROOT, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line('markers', 'gpu: needs a CUDA GPU (GB300, sm_103a)')


def load_golden(name):
    """Golden fixture recorded from the reference (see tests/golden/make_golden.py)."""
    with np.load(os.path.join(GOLDEN, name + '.npz'), allow_pickle=False) as f:
        return {k: f[k] for k in f.files}


def build_for_golden(name, g):
    """This package's instrument of a golden workload (C11's facet positions
    come from the reference's RectangularGrid, recorded in the fixture)."""
    from marxs_gb300 import configs
    if name == 'c11':
        return configs.build(name, elem_pos=g['gas_elem_pos'])
    return configs.build(name)


def golden_inputs(g):
    return {k[3:]: g[k] for k in g if k.startswith('in_')}


def golden_outputs(g):
    return {k[4:]: g[k] for k in g if k.startswith('out_')}


def close_rel(a, b, rtol, scale):
    """|a - b| <= rtol * max(|b|, scale), NaN positions must agree."""
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    na, nb = np.isnan(a), np.isnan(b)
    if not np.array_equal(na, nb):
        return False
    ok = ~na
    return bool(np.all(np.abs(a[ok] - b[ok]) <= rtol * np.maximum(np.abs(b[ok]), scale)))


@pytest.fixture(scope='session')
def reference_marxs():
    import reference_loader
    if not reference_loader.available():
        pytest.skip('MARXS reference source tree not available')
    return reference_loader.load()
