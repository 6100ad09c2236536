"""Edge cases of the trace: empty inputs, and results that do not depend on
how photons fall into warps and blocks.

* An empty photon table comes back unchanged, without stage columns: the
  reference's elements return at once when no photon meets them
  (optics/base.py:176-177), so none of them adds a column.
* An empty device-plane trace is a no-op that succeeds.
* A row of the result depends only on that row (the reference processes the
  table column-wise, every photon on its own), so any slice of a table,
  traced with its Philox rows offset to the slice's first photon
  (``row_base``), must give exactly the rows of the whole table's trace,
  bit for bit.  The slices move every photon to another lane, warp and
  block: single photons, part-warps and part-blocks then go through the
  warp votes of the nearest-facet search (the brute-force warp scan of rays
  the grid cannot bound, e.g. the tilted rays of the CCD test photons) and
  the kernels' tail handling.  A column that a slice never creates (no
  photon of the slice met its element) must hold its fill value (NaN, -1)
  on those rows of the whole trace.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONFIGS = ['c0', 'c1', 'c2', 'c6', 'c7', 'c8', 'c9']
SLICES = [(0, 1), (5, 6), (37, 70), (100, 357), (1000, 1031), (2999, 3001)]
N = 3001


def _table(host, a=None, b=None):
    from marxs_gb300 import PhotonTable
    return PhotonTable({k: np.array(np.asarray(v)[a:b], copy=True) for k, v in host.items()})


def _seq(inst, precision):
    from marxs_gb300.gpu import GpuSequence
    return GpuSequence(elements=inst.elements, precision=precision, rng='philox', seed=97)


@pytest.mark.parametrize('precision', ['fp64', 'fp32local'])
@pytest.mark.parametrize('name', CONFIGS)
def test_slices_equal_the_rows_of_the_whole_trace(name, precision):
    from marxs_gb300 import configs
    inst = configs.build(name)
    host = configs.photons_for(name, N, seed=41)
    seq = _seq(inst, precision)
    whole = seq(_table(host))
    for a, b in SLICES:
        part = seq(_table(host, a, b), row_base=a)
        assert len(part) == b - a
        for col in part.colnames:
            x, y = np.asarray(part[col]), np.asarray(whole[col])[a:b]
            assert x.dtype == y.dtype, (col, a, b)
            assert np.array_equal(x, y, equal_nan=x.dtype.kind == 'f'), (col, a, b)
        for col in set(whole.colnames) - set(part.colnames):
            y = np.asarray(whole[col])[a:b]
            fill = np.isnan(y) if y.dtype.kind == 'f' else (y == -1)
            assert fill.all(), (col, a, b)


@pytest.mark.parametrize('precision', ['fp64', 'fp32local'])
def test_empty_table_comes_back_unchanged(precision):
    from marxs_gb300 import configs
    inst = configs.build('c2')
    host = configs.photons_for('c2', 10, seed=3)
    t = _table(host, 0, 0)
    names = list(t.colnames)
    out = _seq(inst, precision)(t)
    assert len(out) == 0
    assert list(out.colnames) == names


@pytest.mark.parametrize('precision', ['fp64', 'fp32local'])
def test_empty_device_trace_is_a_no_op(precision):
    import torch
    from marxs_gb300 import configs
    from marxs_gb300.gpu import DevicePhotons
    inst = configs.build('c2')
    seq = _seq(inst, precision)
    din, dout = DevicePhotons(0), DevicePhotons(0)
    plan, bufs = seq.allocate_columns(0)
    status = torch.zeros(1, dtype=torch.int32, device='cuda')
    seq.trace_device(din, dout, plan, bufs, status=status)
    torch.cuda.synchronize()
    assert int(status.item()) == 0
