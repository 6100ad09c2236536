"""The drop-in boundary on genuine MARXS objects (host logic, no GPU).

``GpuSequence`` takes the element objects a MARXS user builds.  The GPU
tests build their instruments from this package's look-alike classes; here
the same instruments are built from the reference's own classes (its
``PerfectLens``, ``RadialMirrorScatter``, ``FlatGrating``, ``CATGrating``,
``CATL1L2Stack``, ``Parallel``, ``EfficiencyFile``,
``InterpolateEfficiencyTable``, ``FlatDetector``, ``CircularDetector``,
``ParallelCalculated``,
imported from the MARXS source tree under the test stand-ins for astropy
and transforms3d), and everything the lowering derives from them -- stage
specs, facet records, order tables, splines, stack constants, candidate
grids, the FP32-local constant blocks and the column plan -- must be
byte-identical to the look-alike build.  Any attribute the lowering reads
that differs between the two object families fails here.  Skipped when the
MARXS source tree is not available.
"""
import numpy as np
import pytest

from marxs_gb300 import _abi, configs
from marxs_gb300 import lowering as L
from marxs_gb300.gpu import ColumnPlan


def _arrays(x):
    """Every array / scalar of a lowered object, flattened to comparable bytes."""
    if x is None:
        return ['None']
    if isinstance(x, np.ndarray):
        return [(str(x.dtype), x.shape, np.ascontiguousarray(x).tobytes())]
    if isinstance(x, (bytes, str, int, float, bool, np.integer, np.floating)):
        return [repr(x) if not isinstance(x, bytes) else x]
    if isinstance(x, dict):
        out = []
        for k in sorted(x):
            out += [k] + _arrays(x[k])
        return out
    if isinstance(x, (list, tuple)):
        out = []
        for v in x:
            out += _arrays(v)
        return out
    raise TypeError(type(x))


def _selector(s):
    rows32 = L.selector_rows32(s)
    return (_arrays([s.energy, s.cdf, s.total, s.orders, bool(s.by_energy), int(s.kind)]) +
            _arrays(s.spline) + _arrays(L.selector_thresholds(s)) +
            _arrays(L.selector_guide(s) if s.kind == _abi.SEL_CDF else None) +
            _arrays(rows32))


def lowered(stages):
    """Everything the kernels receive from a lowered chain, per stage."""
    out = []
    for st in stages:
        rec = {'kind': st.kind, 'id_num': st.id_num, 'frame': _arrays(st.frame),
               'cyl': _arrays(st.cyl), 'p': _arrays(st.p),
               'out_names': repr(st.out_names), 'id_col': repr(st.id_col),
               'new_col_order': repr(st.new_col_order), 'draw_names': repr(st.draw_names),
               'reads': repr(st.reads),
               'host_eval': None if st.host_eval is None else
               (sorted(st.host_eval['d']), sorted(st.host_eval['blaze']))}
        rec['facets'] = _arrays(None if st.facets is None else st.facets.view(np.uint8))
        rec['selectors'] = [_selector(s) for s in st.selectors]
        rec['spline'] = _arrays(st.spline)
        rec['stack'] = _arrays(st.stack)
        rec['grid'] = _arrays(st.grid)
        rec['facet_cyl'] = _arrays(st.facet_cyl)
        if st.kind in (_abi.STAGE_LENS, _abi.STAGE_SCATTER, _abi.STAGE_FLATDET):
            rec['fp32'] = L.flat32_block(st)
        elif st.kind == _abi.STAGE_CYLDET:
            blk, table = L.cyl32_block(st)
            rec['fp32'] = _arrays([blk, table])
        elif st.kind in _abi.FACET_STAGES:
            t32 = L.facets32_table(st.facets, detectors=st.kind == _abi.STAGE_DETARRAY)
            if st.facet_cyl is not None:
                t32 = np.zeros(0, dtype=_abi.FACET32_DTYPE)       # float64 mode only
            rec['fp32'] = _arrays(t32.view(np.uint8))
            if st.grid is not None:
                rec['grid32'] = L.grid32_block(st.grid)
        out.append(rec)
    plan = ColumnPlan(stages)
    return out, (repr(plan.columns), repr(plan.first_writer), repr(plan.order))


@pytest.mark.parametrize('name', ['c0', 'c1', 'c2', 'c5', 'c6', 'c7', 'c8', 'c9', 'c10', 'c11'])
def test_reference_objects_lower_like_the_lookalikes(name, reference_marxs):
    import make_golden
    ns = make_golden.reference_namespace(reference_marxs)
    ref = configs.build(name, ns=ns)
    if name == 'c11':
        # the reference's RectangularGrid (a ParallelCalculated on its Rowland
        # torus) against a plain Parallel at the positions it chose
        assert 'RectangularGrid' in {c.__name__ for c in type(ref.gas).__mro__}
        nat = configs.build(name, elem_pos=np.array(ref.gas.elem_pos))
    else:
        nat = configs.build(name)
    # the reference build really holds the reference's classes
    assert type(ref.elements[0]).__module__.startswith('marxs.')
    assert type(nat.elements[0]).__module__.startswith('marxs_gb300.')
    a_stages, a_plan = lowered(L.lower_elements(ref.elements))
    b_stages, b_plan = lowered(L.lower_elements(nat.elements))
    assert len(a_stages) == len(b_stages)
    for k, (a, b) in enumerate(zip(a_stages, b_stages)):
        assert a.keys() == b.keys()
        for key in a:
            assert a[key] == b[key], (name, k, key)
    assert a_plan == b_plan
    # the change watch works on the reference objects too
    w = L.ChangeWatch(ref.elements)
    assert not w.changed(ref.elements)
    g = ref.elements[-1].geometry
    g.pos4d = g.pos4d.copy()
    assert not w.changed(ref.elements)
    g.pos4d[0, 3] += 1e-6
    assert w.changed(ref.elements)


def test_lowering_reads_reference_attributes(reference_marxs):
    """A changed reference attribute reaches the lowered stages: the test
    above would not notice an attribute the lowering ignores, so change a
    few on the reference objects and require a different lowering."""
    import make_golden
    ns = make_golden.reference_namespace(reference_marxs)
    inst = configs.build('c1', ns=ns)
    base, _ = lowered(L.lower_elements(inst.elements))
    inst.lens.focallength = inst.lens.focallength + 1.0
    inst.detector.pixsize = inst.detector.pixsize * 2
    facet = inst.gas.elements[7]
    facet._d = facet._d * 1.01
    moved, _ = lowered(L.lower_elements(inst.elements))
    assert moved[0]['p'] != base[0]['p']
    assert moved[-1]['p'] != base[-1]['p']
    assert moved[2]['facets'] != base[2]['facets']


def test_astropy_table_columns_are_attached_without_a_copy(reference_marxs):
    """The astropy ``Table`` branch of the column attach: new columns go in
    with ``add_column(..., copy=False)`` (the device result's host array is
    not copied again), existing ones are written back in place."""
    from astropy.table import Table
    from marxs_gb300.gpu import _attach_column, _host_target, _write_back
    import torch
    t = Table({'energy': np.arange(5.0), 'pos': np.zeros((5, 4))})
    new = np.arange(5, dtype=np.int32) * 3
    _attach_column(t, 'facet', new)
    assert t.colnames[-1] == 'facet'
    assert np.shares_memory(np.asarray(t['facet']), new)
    # an existing float64 column is the host target itself
    dev = torch.zeros(5, 4, dtype=torch.float64)
    host, fin = _host_target(t, 'pos', dev)
    assert fin is None and np.shares_memory(host.numpy(), np.asarray(t['pos']))
    # an int64 column receiving an int32 device column goes through a staging buffer
    t['id'] = np.full(5, -1, dtype=np.int64)
    _write_back(t, 'id', np.arange(5, dtype=np.int32))
    assert np.asarray(t['id']).dtype == np.int64
    assert np.array_equal(np.asarray(t['id']), np.arange(5))
