"""GPU parity against golden vectors recorded from the MARXS reference.

Each golden fixture holds a photon list, the per-photon random draws the
reference made, and every output column of the reference's own Sequence
(see tests/golden/make_golden.py).  The float64 GPU chain, fed the same
draws, must reproduce them:

* ``facet``, ``order`` (and ``order_L1`` of CAT stacks) and the CCD id
  columns of detector arrays bit-exact for every photon;
* every float column within 1e-9 relative, |a - b| <= 1e-9 * max(|b|, s)
  with s the column's natural scale (1 mm, 1 for unit vectors, 1 pixel,
  1e-3 rad), and NaN exactly where the reference has NaN;
* the same column names in the same order.
"""
import numpy as np
import pytest

from conftest import load_golden, golden_inputs, golden_outputs, build_for_golden, close_rel

pytestmark = pytest.mark.gpu

SCALES = {'pos': 1.0, 'dir': 1.0, 'polarization': 1.0, 'probability': 1.0, 'energy': 1.0,
          'mirror_x': 1.0, 'mirror_y': 1.0, 'y': 1.0, 'z': 1.0, 'inplanescatter': 1e-6,
          'perpplanescatter': 1e-6, 'grat_y': 1.0, 'grat_z': 1.0, 'blaze': 1e-3,
          'det_x': 1.0, 'det_y': 1.0, 'det_phi': 1e-3, 'detpix_x': 1.0, 'detpix_y': 1.0,
          'blaze_L1': 1e-3, 'L2Diffraction': 1e-6}
RTOL = 1e-9


def _run_gpu(name, precision='fp64'):
    from marxs_gb300 import configs, PhotonTable
    from marxs_gb300.gpu import GpuSequence
    g = load_golden(name)
    inst = build_for_golden(name, g)
    draws = {}
    for elem, kind in inst.draw_slots:
        if kind == 'scatter':
            draws[elem] = {'inplanescatter': g['draw_inplanescatter'],
                           'perpplanescatter': g['draw_perpplanescatter']}
        elif kind == 'catstack':
            draws[elem] = {k: g['draw_' + k] for k in ('order_u', 'l1_order_u', 'l1_support_u',
                                                        'l2_normal', 'l2_phi_u')}
        else:
            draws[elem] = {'order_u': g['draw_order_u']}
    seq = GpuSequence(elements=inst.elements, precision=precision, rng='predrawn')
    out = seq(PhotonTable(golden_inputs(g)), draws=draws)
    return g, out


def _column_report(out, ref, ok):
    """Per-column (passed, worst relative error) against the golden outputs."""
    report = {}
    for col, b in ref.items():
        a = np.asarray(out[col])
        if a.dtype != b.dtype:
            report[col] = (False, 'dtype %s vs %s' % (a.dtype, b.dtype))
            continue
        if col in ('facet', 'order', 'order_L1', 'CCD_ID', 'CCD'):
            same = np.array_equal(a[ok], b[ok], equal_nan=True)
            report[col] = (same, int(np.sum(~((a[ok] == b[ok]) | (np.isnan(a[ok].astype(float)) &
                                                                 np.isnan(b[ok].astype(float)))))))
            continue
        fin = ~np.isnan(b[ok])
        nan_ok = np.array_equal(np.isnan(a[ok]), np.isnan(b[ok]))
        scale = SCALES[col]
        err = np.abs(a[ok][fin] - b[ok][fin]) / np.maximum(np.abs(b[ok][fin]), scale)
        worst = float(err.max()) if err.size else 0.0
        passed = nan_ok and close_rel(a[ok], b[ok], RTOL, scale)
        if col in ('blaze', 'blaze_L1'):
            # arccos is ill-conditioned near normal incidence: an ulp in the
            # cosine moves the angle by up to sqrt(2 * 2.2e-16) ~ 2e-8 rad
            d = np.abs(a[ok][fin] - b[ok][fin])
            passed = nan_ok and bool(np.all(d <= RTOL * np.maximum(np.abs(b[ok][fin]), scale)
                                            + BLAZE_ABS))
            worst = float(d.max()) if d.size else 0.0
        report[col] = (passed, worst if nan_ok else 'NaN pattern differs')
    return report


BLAZE_ABS = 5e-8


@pytest.mark.parametrize('name', ['c0', 'c1', 'c2', 'c5', 'c6', 'c7', 'c8', 'c9', 'c10', 'c11'])
def test_golden_parity_fp64(name):
    g, out = _run_gpu(name)
    ref = golden_outputs(g)
    assert list(out.colnames) == [str(c) for c in g['colnames']]
    ok = ~g['multi_hit']
    report = _column_report(out, ref, ok)
    bad = {k: v for k, v in report.items() if not v[0]}
    assert not bad, 'columns out of tolerance: %s (all: %s)' % (bad, report)


@pytest.mark.parametrize('name', ['c1', 'c2', 'c5', 'c6', 'c9', 'c10'])
def test_golden_hits_are_counted(name):
    from marxs_gb300 import configs
    g, out = _run_gpu(name)
    ref = golden_outputs(g)
    assert (np.asarray(out['facet']) >= 0).sum() == (ref['facet'] >= 0).sum() > 0


@pytest.mark.parametrize('name,idc', [('c7', 'CCD_ID'), ('c8', 'CCD')])
def test_ccd_array_ids_and_misses(name, idc):
    """A Parallel of FlatDetectors: the chip each photon lands on is the
    reference's (bit-exact, -1 for gaps and misses), per-chip hit counts
    match, and the C7 layout numbers its chips 0..3 as the reference's own
    Parallel test requires (simulator/tests/test_parallel.py:11-23)."""
    g, out = _run_gpu(name)
    ref = golden_outputs(g)
    ids = np.asarray(out[idc])
    assert ids.dtype == ref[idc].dtype
    assert np.array_equal(ids, ref[idc])
    assert np.array_equal(np.bincount(ids[ids >= 0]), np.bincount(ref[idc][ref[idc] >= 0]))
    miss = ids < 0
    assert miss.any() and np.all(np.isnan(np.asarray(out['det_x'])[miss]))


def test_cat_stack_l1_order_column():
    """CATL1L2Stack facets: the L1 order column is exact (the reference's
    own L1 draws decide it)."""
    g, out = _run_gpu('c6')
    ref = golden_outputs(g)
    assert np.array_equal(np.asarray(out['order_L1']), ref['order_L1'], equal_nan=True)


def test_catsupportbars_stage():
    """catsupportbars as a chain stage: probability 0 where facet < 0, the
    rest unchanged (float64 and FP32-local, device and table paths); with
    no facet column every photon is absorbed; an int64 facet column that
    the input table already holds is read."""
    from marxs_gb300 import configs, PhotonTable
    from marxs_gb300.gpu import DevicePhotons, GpuSequence
    from marxs_gb300.optics import catsupportbars
    import torch
    inst = configs.build('c2')
    n = 50_000
    host = configs.photons_for('c2', n, seed=3)
    for prec in ('fp64', 'fp32local'):
        res = {}
        for key, elems in (('plain', inst.elements),
                           ('bars', inst.elements[:3] + [catsupportbars] + inst.elements[3:])):
            seq = GpuSequence(elems, precision=prec, rng='philox', seed=5)
            ph = DevicePhotons.from_columns(host)
            plan, bufs = seq.allocate_columns(n)
            status, _ = seq.trace_device(ph, ph, plan, bufs)
            torch.cuda.synchronize()
            assert int(status.item()) == 0
            res[key] = (ph.prob.cpu().numpy(), bufs['facet'].cpu().numpy())
        (p0, f0), (p1, f1) = res['plain'], res['bars']
        assert np.array_equal(f0, f1)
        assert np.array_equal(p1[f1 >= 0], p0[f0 >= 0]) and np.all(p1[f1 < 0] == 0)
        assert (f1 < 0).any() and (f1 >= 0).any()
    # no facet column: everything absorbed
    t = PhotonTable({k: np.array(v, copy=True) for k, v in host.items()})
    GpuSequence([inst.lens, catsupportbars], precision='fp64', rng='philox')(t)
    assert np.all(np.asarray(t['probability']) == 0)
    # a facet column already in the table
    t = PhotonTable({k: np.array(v, copy=True) for k, v in host.items()})
    t['facet'] = np.where(np.arange(n) % 3 == 0, -1, 7).astype(np.int64)
    GpuSequence([catsupportbars], precision='fp64', rng='philox')(t)
    p = np.asarray(t['probability'])
    assert np.all(p[np.arange(n) % 3 == 0] == 0)
    assert np.array_equal(p[np.arange(n) % 3 != 0], host['probability'][np.arange(n) % 3 != 0])


def test_host_changes_reach_the_device():
    """One GpuSequence traced, then facets moved the way the reference's
    tolerancing moves them (a new pos4d assigned, design/tolerancing.py:133),
    one edited in place, an order selector swapped (as
    analysis/gratings.py:117-124 does) and the lens refocused: the next call
    must trace the changed instrument, equal to the oracle on it."""
    from marxs_gb300 import configs, PhotonTable
    from marxs_gb300.gpu import GpuSequence
    from marxs_gb300.optics import OrderSelector
    from oracle.raytrace import run_sequence
    n = 20000
    inst = configs.build('c1')
    photons = configs.photons_for('c1', n, seed=31)
    draws = configs.draws_for(inst.draw_slots, n, seed=31)
    seq = GpuSequence(elements=inst.elements, precision='fp64', rng='predrawn')
    first = seq(PhotonTable(photons), draws=draws)
    hits0 = np.bincount(np.asarray(first['facet'])[np.asarray(first['facet']) >= 0],
                        minlength=200)
    busy = np.argsort(hits0)[::-1][:3]
    facets = inst.elements[2].elements
    # moves inside the 2 mm gaps of the 22 mm pitch: facets never overlap,
    # where the sequential Parallel and the nearest hit would differ
    move = np.eye(4)
    move[1, 3] = 1.5
    g = facets[busy[0]].geometry
    g.pos4d = move @ g.pos4d
    facets[busy[1]].geometry.pos4d[2, 3] -= 1.5
    facets[busy[2]].order_selector = OrderSelector([2])
    inst.elements[0].focallength = inst.elements[0].focallength + 25.0
    out = seq(PhotonTable(photons), draws=draws)
    ref, stats = run_sequence(inst.elements, photons, draws)
    ok = ~stats.get('multi_hit_mask', np.zeros(n, dtype=bool))
    fa, fr = np.asarray(out['facet']), ref['facet']
    assert np.array_equal(fa[ok], fr[ok])
    assert np.array_equal(np.asarray(out['order'])[ok], ref['order'][ok], equal_nan=True)
    assert not np.array_equal(np.asarray(first['facet']), fa)
    assert np.all(np.asarray(out['order'])[fa == busy[2]] == 2)
    for key in ('pos', 'dir'):
        a, b = np.asarray(out[key])[ok], ref[key][ok]
        assert np.array_equal(np.isnan(a), np.isnan(b))
        m = ~np.isnan(b)
        assert np.all(np.abs(a[m] - b[m]) <= 1e-9 * np.maximum(np.abs(b[m]), 1.0)), key


def test_sequence_with_steps_equals_the_fused_chain():
    """preprocess_steps / postprocess_steps make the chain run element by
    element on the table (float64 round trips between elements are exact):
    with pre-drawn randomness the result equals the fused chain's, and the
    steps ran around every element."""
    from marxs_gb300 import configs, PhotonTable
    from marxs_gb300.gpu import GpuSequence
    n = 20000
    inst = configs.build('c1')
    photons = configs.photons_for('c1', n, seed=41)
    draws = configs.draws_for(inst.draw_slots, n, seed=41)
    calls = []
    fused = GpuSequence(elements=inst.elements, precision='fp64', rng='predrawn')
    steps = GpuSequence(elements=inst.elements, precision='fp64', rng='predrawn',
                        preprocess_steps=[lambda t: calls.append('pre')],
                        postprocess_steps=[lambda t: calls.append('post')])
    a = fused(PhotonTable(photons), draws=draws)
    b = steps(PhotonTable(photons), draws=draws)
    assert calls == ['pre', 'post'] * len(inst.elements)
    assert sorted(a.colnames) == sorted(b.colnames)
    for col in a.colnames:
        assert np.array_equal(np.asarray(a[col]), np.asarray(b[col]), equal_nan=True), col


def test_chirped_facets_use_their_callables():
    """C9: the facets' own callables decide the diffraction.  The golden
    parity above holds; here the same trace with the chirp removed (every
    facet's constant d) must move the dispersed photons, and the blaze
    column of the facets with a modifier carries it."""
    from marxs_gb300 import configs, PhotonTable
    from marxs_gb300.gpu import GpuSequence
    g, out = _run_gpu('c9')
    inst = configs.build('c9')
    ref = golden_outputs(g)
    disp = np.isfinite(ref['order']) & (ref['order'] != 0) & np.isfinite(ref['det_x'])
    assert disp.sum() > 100
    plain = configs.build('c1', seed=9)
    draws = {plain.scatter: {'inplanescatter': g['draw_inplanescatter'],
                             'perpplanescatter': g['draw_perpplanescatter']},
             plain.gas: {'order_u': g['draw_order_u']}}
    flat = GpuSequence(elements=plain.elements, precision='fp64', rng='predrawn')(
        PhotonTable(golden_inputs(g)), draws=draws)
    moved = np.abs(np.asarray(flat['det_x'])[disp] - np.asarray(out['det_x'])[disp])
    # photons the unchirped gratings send off the detector are NaN there
    assert np.isfinite(moved).mean() > 0.5
    assert np.nanmedian(moved) > 1e-3
    facet = np.asarray(out['facet'])
    mod = np.isin(facet, [e.id_num for k, e in enumerate(inst.gas.elements) if k % 3 == 0])
    assert np.any(np.asarray(out['blaze'])[mod] != np.asarray(flat['blaze'])[mod])


def test_bent_gratings_float64_only():
    """C10 (gratings bent onto cylinders): the float64 mode matches the
    reference (golden parity above, local coordinates (phi, z)); the
    FP32-local mode refuses the chain rather than treat the facets as
    flat."""
    from marxs_gb300 import configs, PhotonTable
    from marxs_gb300.gpu import GpuSequence
    g, out = _run_gpu('c10')
    ref = golden_outputs(g)
    hit = np.asarray(out['facet']) >= 0
    assert hit.mean() > 0.5
    assert np.nanmax(np.abs(np.asarray(out['grat_y']))) < 0.01        # phi, rad
    inst = configs.build('c10')
    with pytest.raises(NotImplementedError):
        GpuSequence(elements=inst.elements, precision='fp32local', rng='philox')(
            PhotonTable(golden_inputs(g)))
