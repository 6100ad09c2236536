"""FP32-local precision mode against the float64 path and the golden vectors.

The FP32-local kernel re-centres every ray on the element it meets (positions
are float-float), does the element arithmetic in float32 and keeps float64
only for the final detector coordinates.  Both modes draw the same Philox
numbers, so per photon they must pick the same facet and order (except for
rays within ~1e-5 mm of a facet edge) and land within a fraction of a
micron of each other.

Tolerances, stated as the acceptance bar of the precision mode:
* detector-position error over photons whose facet and order agree:
  RMS <= 0.5 um, max <= 5 um (global x, y, z and (det_phi * R, det_y));
* facet/order disagreement (plus CAT sign decisions taken within float32
  noise of zero, blaze < 2e-7 rad) in at most 1e-4 of the photons;
* against the reference's golden vectors (pre-drawn draws): the same bars,
  directions within 1e-6, polarization within 1e-5 (float32 transport of
  nearly parallel directions), probability within 2e-6 relative (1e-5
  through CATL1L2Stack facets, a product of five float32 factors).
* every other column, over the photons whose decisions agree
  (``COLUMN_BARS``): local coordinates in mm (mirror_x/y, y, z, grat_y/z,
  det_x, det_y) RMS <= 0.5 um and max <= 5 um like positions; det_phi
  times the cylinder radius the same; detector pixels times the pixel size
  the same; blaze angles within 1e-6 rad; scatter angles within 1e-4 of
  the column's largest magnitude (+1e-12 rad: Box-Muller with the fast
  float32 log); NaN exactly where the float64 result has NaN.
"""
import numpy as np
import pytest

from conftest import load_golden, golden_inputs, golden_outputs, build_for_golden

pytestmark = pytest.mark.gpu

UM = 1e-3   # mm
# |p . d| below this is within a few float32 roundings of zero (6e-8 each)
SIGN_BAND = 2e-7


def _trace(inst, host, precision, rng='philox', draws=None):
    from marxs_gb300 import PhotonTable
    from marxs_gb300.gpu import GpuSequence
    seq = GpuSequence(elements=inst.elements, precision=precision, rng=rng, seed=424242)
    return seq(PhotonTable({k: np.array(v, copy=True) for k, v in host.items()}), draws=draws)


def _agree(a, b):
    """Photons whose discrete decisions agree: same facet, same order, and a
    CAT sign decision sign(p . d) that is not within float32 noise of zero
    (blaze angle of the float64 result >= SIGN_BAND, or order 0)."""
    fa, fb = np.asarray(a['facet']), np.asarray(b['facet'])
    oa, ob = np.asarray(a['order']), np.asarray(b['order'])
    same = (fa == fb) & ((oa == ob) | (np.isnan(oa) & np.isnan(ob)))
    if 'blaze' in b:
        bl = np.asarray(b['blaze'])
        with np.errstate(invalid='ignore'):
            same &= ~((bl < SIGN_BAND) & (ob != 0))
    return same


def _pos_err(a, b, mask):
    pa, pb = np.asarray(a['pos'])[mask, :3], np.asarray(b['pos'])[mask, :3]
    fin = np.all(np.isfinite(pb), axis=1)
    d = np.linalg.norm(pa[fin] - pb[fin], axis=1)
    return d


# column -> kind of bar (see the module docstring)
COLUMN_BARS = {'mirror_x': 'mm', 'mirror_y': 'mm', 'y': 'mm', 'z': 'mm', 'grat_y': 'mm',
               'grat_z': 'mm', 'det_x': 'mm', 'det_y': 'mm', 'det_phi': 'phi',
               'detpix_x': 'pix', 'detpix_y': 'pix', 'blaze': 'rad', 'blaze_L1': 'rad',
               'inplanescatter': 'rel', 'perpplanescatter': 'rel', 'L2Diffraction': 'rel'}
EXACT = ('facet', 'order', 'order_L1', 'CCD_ID', 'CCD', 'energy')


def _detector_scales(inst):
    """(pixel size in mm, cylinder radius in mm or None) of the chain's detector."""
    from marxs_gb300.geomath import decompose44
    det = inst.detector
    first = det.elements[0] if hasattr(det, 'elements') else det
    R = None
    if 'CircularDetector' in {c.__name__ for c in type(det).__mro__}:
        R = float(decompose44(np.asarray(det.geometry.pos4d))[2][0])
    return float(first.pixsize), R


def check_columns(a, b, agree, inst):
    """Every output column of the FP32-local result ``a`` against the float64
    (or reference) result ``b`` within its bar; returns the worst errors."""
    pix, R = _detector_scales(inst)
    worst = {}
    for col in (b.colnames if hasattr(b, 'colnames') else list(b)):
        if col in ('pos', 'dir', 'polarization', 'probability') or col in EXACT:
            continue
        x = np.asarray(a[col], dtype=float)[agree]
        y = np.asarray(b[col], dtype=float)[agree]
        assert np.array_equal(np.isnan(x), np.isnan(y)), col
        fin = ~np.isnan(y)
        if not fin.any():
            continue
        d = np.abs(x[fin] - y[fin])
        kind = COLUMN_BARS[col]
        if kind in ('mm', 'phi', 'pix'):
            scale = {'mm': 1.0, 'phi': R, 'pix': pix}[kind]
            dm = d * scale
            worst[col] = (np.sqrt(np.mean(dm ** 2)) / UM, dm.max() / UM)
            assert np.sqrt(np.mean(dm ** 2)) <= 0.5 * UM and dm.max() <= 5 * UM, (col, worst[col])
        elif kind == 'rad':
            worst[col] = d.max()
            assert d.max() <= 1e-6, (col, d.max())
        else:
            # float32 angles: the scatter draws go through Box-Muller with the
            # fast float32 log, 1e-4 of the column's largest magnitude
            scale = np.max(np.abs(y[fin]))
            worst[col] = d.max() / scale
            assert d.max() <= 1e-4 * scale + 1e-12, (col, worst[col])
    return worst


@pytest.mark.parametrize('n', [400000])
def test_fp32local_vs_fp64_cat_array(n):
    from marxs_gb300 import configs
    inst = configs.build('c2')
    host = configs.photons_for('c2', n, seed=21)
    a = _trace(inst, host, 'fp32local')
    b = _trace(inst, host, 'fp64')
    agree = _agree(a, b)
    assert (~agree).sum() <= max(1, 1e-4 * n), (~agree).sum()
    d = _pos_err(a, b, agree)
    rms, mx = np.sqrt(np.mean(d ** 2)), d.max()
    R = 5900.0
    hit = agree & np.isfinite(np.asarray(b['det_phi']))
    dphi = np.abs(np.asarray(a['det_phi'])[hit] - np.asarray(b['det_phi'])[hit]) * R
    dy = np.abs(np.asarray(a['det_y'])[hit] - np.asarray(b['det_y'])[hit])
    report = dict(mismatch=int((~agree).sum()), rms_um=rms / UM, max_um=mx / UM,
                  phi_rms_um=np.sqrt(np.mean(dphi ** 2)) / UM, phi_max_um=dphi.max() / UM,
                  dety_max_um=dy.max() / UM)
    print('fp32local vs fp64:', report)
    assert rms <= 0.5 * UM and mx <= 5 * UM, report
    assert np.sqrt(np.mean(dphi ** 2)) <= 0.5 * UM and dphi.max() <= 5 * UM, report
    assert dy.max() <= 5 * UM, report
    # the lean chain keeps the probability in float64: the float64 product
    pa, pb = np.asarray(a['probability'])[agree], np.asarray(b['probability'])[agree]
    assert np.array_equal(pa, pb)
    print('columns:', check_columns(a, b, agree, inst))


@pytest.mark.parametrize('name', ['c0', 'c1', 'c2', 'c5', 'c6', 'c7', 'c8', 'c9', 'c11'])
def test_fp32local_golden(name):
    from marxs_gb300 import configs
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
    out = _trace(inst, golden_inputs(g), 'fp32local', rng='predrawn', draws=draws)
    ref = golden_outputs(g)
    assert list(out.colnames) == [str(c) for c in g['colnames']]
    agree = np.ones(g['n'], dtype=bool)
    if 'facet' in ref:
        agree = _agree(out, ref)
        assert (~agree).sum() <= 1, (~agree).sum()
    for idc in ('CCD_ID', 'CCD'):
        if idc in ref:
            agree &= np.asarray(out[idc]) == ref[idc]
            assert (~agree).sum() <= 1, (idc, (~agree).sum())
    d = _pos_err(out, ref, agree)
    assert np.sqrt(np.mean(d ** 2)) <= 0.5 * UM and d.max() <= 5 * UM, (d.max(), name)
    for col, tol in (('dir', 1e-6), ('polarization', 1e-5)):
        x, y = np.asarray(out[col])[agree], ref[col][agree]
        assert np.nanmax(np.abs(x - y)) <= tol, (col, np.nanmax(np.abs(x - y)))
    # float32 probability (products of the element factors; a CAT stack
    # multiplies five of them: membrane order, quality factor, L1, L2Abs)
    x, y = np.asarray(out['probability'])[agree], ref['probability'][agree]
    ptol = 1e-5 if name == 'c6' else 2e-6
    assert np.max(np.abs(x - y) / np.maximum(y, 1e-30)) <= ptol
    check_columns(out, ref, agree, inst)


def test_fp32local_vs_fp64_cat_stack():
    """CATL1L2Stack facets (C6) in FP32-local against the float64 path with
    the same Philox draws: the membrane and L1 orders agree, the L2 scatter
    angle to float32 precision, positions to the precision bar."""
    from marxs_gb300 import configs
    n = 200000
    inst = configs.build('c6')
    host = configs.photons_for('c6', n, seed=23)
    a = _trace(inst, host, 'fp32local')
    b = _trace(inst, host, 'fp64')
    agree = _agree(a, b)
    l1a, l1b = np.asarray(a['order_L1']), np.asarray(b['order_L1'])
    agree &= (l1a == l1b) | (np.isnan(l1a) & np.isnan(l1b))
    assert (~agree).sum() <= max(1, 1e-4 * n), (~agree).sum()
    assert (np.asarray(b['facet']) >= 0).mean() > 0.3
    d = _pos_err(a, b, agree)
    rms, mx = np.sqrt(np.mean(d ** 2)), d.max()
    assert rms <= 0.5 * UM and mx <= 5 * UM, (rms / UM, mx / UM)
    x, y = np.asarray(a['L2Diffraction'])[agree], np.asarray(b['L2Diffraction'])[agree]
    fin = np.isfinite(y)
    assert np.array_equal(np.isfinite(x), fin)
    assert np.max(np.abs(x[fin] - y[fin])) <= 1e-6 * np.max(np.abs(y[fin])) + 1e-12
    pa, pb = np.asarray(a['probability'])[agree], np.asarray(b['probability'])[agree]
    assert np.max(np.abs(pa - pb) / np.maximum(pb, 1e-30)) <= 1e-5
    check_columns(a, b, agree, inst)


def test_fp32local_vs_fp64_ccd_strip():
    """C8 (CAT array and a 16-chip strip on the Rowland circle) in
    FP32-local against float64 with the same Philox draws: the chip each
    photon lands on agrees (up to float32 edge decisions), every column
    within its bar."""
    from marxs_gb300 import configs
    n = 400000
    inst = configs.build('c8')
    host = configs.photons_for('c8', n, seed=25)
    a = _trace(inst, host, 'fp32local')
    b = _trace(inst, host, 'fp64')
    agree = _agree(a, b) & (np.asarray(a['CCD']) == np.asarray(b['CCD']))
    assert (~agree).sum() <= max(1, 1e-4 * n), (~agree).sum()
    assert (np.asarray(b['CCD']) >= 0).mean() > 0.1
    d = _pos_err(a, b, agree)
    assert np.sqrt(np.mean(d ** 2)) <= 0.5 * UM and d.max() <= 5 * UM
    check_columns(a, b, agree, inst)


@pytest.mark.parametrize('name', ['c0', 'c1', 'c2', 'c5', 'c6', 'c8'])
def test_specialised_kernels_match_generic(name):
    """The kernels specialised for a stage sequence (stage kinds and
    constants fixed at compile time, the order's energy row found at the
    start of the photon; for the common lens and efficiency-table
    configuration that configuration compiled in alone, c5's spline
    selector and lens reflectivity the full one) give the same result bits as the generic stage
    loop on the same chain (``GpuSequence.specialised = False``); the
    probability, which the lean chains keep in float64 and the generic loop
    in float32, to float32 rounding."""
    from marxs_gb300 import configs, PhotonTable
    from marxs_gb300.gpu import GpuSequence
    n = 100000
    inst = configs.build(name)
    host = configs.photons_for(name, n, seed=27)
    outs = []
    for specialised in (True, False):
        seq = GpuSequence(elements=inst.elements, precision='fp32local', rng='philox', seed=99)
        seq.specialised = specialised
        outs.append(seq(PhotonTable({k: np.array(v, copy=True) for k, v in host.items()})))
    a, b = outs
    assert list(a.colnames) == list(b.colnames)
    for col in a.colnames:
        x, y = np.asarray(a[col]), np.asarray(b[col])
        if col == 'probability':
            assert np.all(np.abs(x - y) <= 2.0 ** -24 * np.abs(y)), col
            continue
        assert np.array_equal(x, y, equal_nan=x.dtype.kind == 'f'), col


def test_split_launches_match_one_launch():
    """Launches beyond 2^30 photons are split, every column pointer and the
    Philox row moved to each part's first photon; splitting every 4096
    photons (``GpuSequence.split_launches``) runs that path at a testable
    size and must give the same result bits, through the table path
    ((N, 4) host columns) and on device planes."""
    from marxs_gb300 import configs, PhotonTable
    from marxs_gb300.gpu import GpuSequence, DevicePhotons
    n = 100003
    inst = configs.build('c2')
    host = configs.photons_for('c2', n, seed=37)
    tables, planes = [], []
    for split in (False, True):
        seq = GpuSequence(elements=inst.elements, precision='fp32local', rng='philox', seed=5)
        seq.split_launches = split
        tables.append(seq(PhotonTable({k: np.array(v, copy=True) for k, v in host.items()}),
                          row_base=1000))
        hits_table = seq.last_hits
        din, dout = DevicePhotons.from_columns(host), DevicePhotons(n)
        plan, bufs = seq.allocate_columns(n)
        seq.trace_device(din, dout, plan, bufs)
        planes.append({'pos': dout.pos.cpu().numpy(), 'dir': dout.dir.cpu().numpy(),
                       'pol': dout.pol.cpu().numpy(), 'prob': dout.prob.cpu().numpy(),
                       **{k: v.cpu().numpy() for k, v in bufs.items()}, 'hits': hits_table})
    a, b = tables
    assert list(a.colnames) == list(b.colnames)
    for col in a.colnames:
        x, y = np.asarray(a[col]), np.asarray(b[col])
        assert np.array_equal(x, y, equal_nan=x.dtype.kind == 'f'), col
    for key in planes[0]:
        x, y = planes[0][key], planes[1][key]
        assert np.array_equal(x, y, equal_nan=x.dtype.kind == 'f'), key
