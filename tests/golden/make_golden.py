"""Generate golden raytrace vectors by running the MARXS reference itself.

Run from the repository root (needs the reference source tree, see
``reference_loader.py``)::

    python tests/golden/make_golden.py

For each workload (c0, c1, c2, c5, c6) this builds the instrument from the
reference's own classes, traces a small seeded photon list through the
reference's ``Sequence`` with numpy's global RNG seeded, and records every
random draw the reference makes.  The draws are mapped back to photons
(element call order, photon row order within each call), giving per-photon
arrays that the oracle and the GPU kernels consume in pre-drawn mode.

Outputs ``tests/golden/<config>.npz`` with: input columns (``in_*``),
per-photon draws (``draw_*``), every output column (``out_*``), the facet
poses the reference generated, and the count of photons that crossed more
than one facet (excluded from parity).
"""
import io
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
sys.path.insert(0, ROOT)

import reference_loader  # noqa: E402
from marxs_gb300 import configs  # noqa: E402

N_PHOTONS = {'c0': 2000, 'c1': 3000, 'c2': 3000, 'c5': 3000, 'c6': 3000, 'c7': 2000, 'c8': 3000,
             'c9': 3000, 'c10': 3000, 'c11': 3000}
GLOBAL_SEED = 20261203


class Recorder:
    """Wraps numpy's global-RNG functions the reference calls and logs draws
    against the element call that is running."""

    def __init__(self):
        self.calls = []          # list of (element, intersect mask, [draw arrays])
        self.current = None
        self._orig = {}

    def install(self):
        rnd = np.random
        self._orig = {'normal': rnd.normal, 'choice': rnd.choice, 'rand': rnd.rand}
        orig = self._orig
        rec = self

        def normal(loc=0.0, scale=1.0, size=None):
            v = orig['normal'](loc, scale, size)
            rec.current[2].append(('normal', np.array(v, copy=True)))
            return v

        def choice(a, size=None, replace=True, p=None):
            # legacy RandomState.choice with p: one uniform per draw and
            # cdf.searchsorted(u, side='right'); checked against numpy below
            p = np.asarray(p, dtype=float)
            cdf = p.cumsum()
            cdf /= cdf[-1]
            u = np.random.random_sample(size)
            idx = cdf.searchsorted(u, side='right')
            rec.current[2].append(('uniform', np.array(u, copy=True)))
            return np.asarray(a)[idx]

        def rand(*args):
            v = orig['rand'](*args)
            rec.current[2].append(('uniform', np.atleast_1d(np.array(v, copy=True))))
            return v

        def uniform(low=0.0, high=1.0, size=None):
            # legacy RandomState.uniform = low + (high - low) * random_sample
            u = np.random.random_sample(size)
            rec.current[2].append(('uniform', np.atleast_1d(np.array(u, copy=True))))
            return low + (high - low) * u

        self._orig['uniform'] = rnd.uniform
        rnd.normal, rnd.choice, rnd.rand, rnd.uniform = normal, choice, rand, uniform

    def uninstall(self):
        for k, v in self._orig.items():
            setattr(np.random, k, v)

    def wrap(self, elem):
        orig = elem.specific_process_photons
        rec = self

        def wrapped(photons, intersect, interpos, intercoos):
            rec.current = (elem, np.array(intersect, copy=True), [])
            out = orig(photons, intersect, interpos, intercoos)
            rec.calls.append(rec.current)
            rec.current = None
            return out
        elem.specific_process_photons = wrapped


def check_choice_restatement():
    """The recorded choice() must equal numpy's legacy implementation."""
    p = np.array([0.1, 0.05, 0.3, 0.2, 0.35])
    np.random.seed(5)
    a = np.random.choice(np.arange(5), size=1000, p=p)
    np.random.seed(5)
    cdf = p.cumsum()
    cdf /= cdf[-1]
    b = cdf.searchsorted(np.random.random_sample(1000), side='right')
    assert np.array_equal(a, b)


def reference_namespace(marxs):
    import astropy.units as u
    from types import SimpleNamespace
    from marxs.optics import (PerfectLens, RadialMirrorScatter, FlatDetector, CircularDetector,
                              FlatGrating, CATGrating, OrderSelector, EfficiencyFile)
    from marxs.math.geometry import Cylinder
    from marxs.simulator import Parallel, ParallelCalculated, Sequence
    from marxs.design.rowland import RowlandTorus, RectangularGrid

    def interpolated(wave_nm, blaze_deg, probs, orders):
        # the reference class reads a flattened (wavelength, blaze) table
        from astropy.table import Column, Table
        from marxs.missions.mitsnl.catgrating import InterpolateEfficiencyTable
        ww, bb = np.meshgrid(wave_nm, blaze_deg, indexing='ij')
        cols = [Column(ww.ravel(), name='wave', unit=u.nm),
                Column(bb.ravel(), name='blaze', unit=u.deg)]
        cols += [Column(np.asarray(probs[i]).ravel(), name=str(int(o)))
                 for i, o in enumerate(orders)]
        return InterpolateEfficiencyTable(Table(cols), k=1)

    def eff(table, orders):
        if isinstance(table, np.ndarray):
            buf = io.StringIO()
            np.savetxt(buf, table, fmt='%.17g')
            buf.seek(0)
            return EfficiencyFile(buf, orders)
        return EfficiencyFile(table, orders)

    def cat_stack_class():
        # the reference stack, with the L1 support transmission given as a
        # table (the reference reads it from its Si data file)
        from scipy.interpolate import interp1d
        from marxs.missions.mitsnl.catgrating import CATL1L2Stack

        class Stack(CATL1L2Stack):
            def __init__(self, l1_transmission=None, **kwargs):
                super().__init__(**kwargs)
                if l1_transmission is not None:
                    self.elements[2].transfunc = interp1d(*l1_transmission)
        return Stack

    from marxs.missions.mitsnl.catgrating import catsupportbars
    return SimpleNamespace(PerfectLens=PerfectLens, RadialMirrorScatter=RadialMirrorScatter,
                           CATL1L2Stack=cat_stack_class(), catsupportbars=catsupportbars,
                           FlatDetector=FlatDetector, CircularDetector=CircularDetector,
                           FlatGrating=FlatGrating, CATGrating=CATGrating,
                           OrderSelector=OrderSelector, EfficiencyFile=eff,
                           InterpolateEfficiencyTable=interpolated, Cylinder=Cylinder,
                           Parallel=Parallel, ParallelCalculated=ParallelCalculated,
                           RowlandTorus=RowlandTorus, RectangularGrid=RectangularGrid,
                           Sequence=Sequence, angle=lambda r: r * u.rad)


def leaves(elements):
    out = []
    for e in elements:
        if hasattr(e, 'elements'):
            out.extend(leaves(e.elements))
        else:
            out.append(e)
    return out


def generate(name):
    marxs = reference_loader.load()
    from astropy.table import Table
    ns = reference_namespace(marxs)
    inst = configs.build(name, ns)
    n = N_PHOTONS[name]
    ph = configs.photons_for(name, n, seed=int(name[1:]))
    table = Table({k: v.copy() for k, v in ph.items()})

    rec = Recorder()
    for e in leaves(inst.elements):
        if hasattr(e, 'specific_process_photons'):      # not the plain-function elements
            rec.wrap(e)
    seq = ns.Sequence(elements=inst.elements)
    np.random.seed(GLOBAL_SEED + zlib.crc32(name.encode()) % 1000)
    rec.install()
    try:
        out = seq(table)
    finally:
        rec.uninstall()

    # map recorded draws to per-photon arrays
    draw = {'inplanescatter': np.zeros(n), 'perpplanescatter': np.zeros(n),
            'order_u': np.full(n, np.nan), 'l1_order_u': np.full(n, np.nan),
            'l1_support_u': np.full(n, np.nan), 'l2_normal': np.full(n, np.nan),
            'l2_phi_u': np.full(n, np.nan)}
    seen = np.zeros(n, dtype=int)
    for elem, mask, logged in rec.calls:
        rows = np.nonzero(mask)[0]
        cname = type(elem).__name__
        if cname == 'RadialMirrorScatter':
            kinds = [k for k, _ in logged]
            vals = [v for _, v in logged]
            j = 0
            if elem.inplanescatter != 0:
                assert kinds[j] == 'normal'
                draw['inplanescatter'][rows] = vals[j]
                j += 1
            if elem.perpplanescatter != 0:
                assert kinds[j] == 'normal'
                draw['perpplanescatter'][rows] = vals[j]
        elif cname in ('FlatGrating', 'CATGrating', 'NonParallelCATGrating'):
            u = np.concatenate([v for k, v in logged if k == 'uniform'])
            assert len(u) == len(rows)
            draw['order_u'][rows] = u
            seen[rows] += 1
        elif cname == 'L1':
            # order draw (choice), then the support draw (rand)
            assert [k for k, _ in logged] == ['uniform', 'uniform']
            draw['l1_order_u'][rows] = logged[0][1]
            draw['l1_support_u'][rows] = logged[1][1]
        elif cname == 'L2Diffraction':
            # scatter angle (normal), then the direction around the ray (uniform)
            assert [k for k, _ in logged] == ['normal', 'uniform']
            draw['l2_normal'][rows] = logged[0][1]
            draw['l2_phi_u'][rows] = logged[1][1]
        else:
            assert not logged, cname
    multi = seen > 1
    res = {'n': n, 'multi_hit': multi}
    for k, v in ph.items():
        res['in_' + k] = v
    for k, v in draw.items():
        if k in ('inplanescatter', 'perpplanescatter', 'order_u') or not np.all(np.isnan(v)):
            res['draw_' + k] = v
    for k in out.colnames:
        res['out_' + k] = np.asarray(out[k])
    if hasattr(inst, 'gas'):
        res['facet_pos4d'] = np.array([e.geometry.pos4d for e in inst.gas.elements])
        if name == 'c11':
            res['gas_elem_pos'] = np.array(inst.gas.elem_pos)
    if hasattr(getattr(inst, 'detector', None), 'elements'):
        res['ccd_pos4d'] = np.array([e.geometry.pos4d for e in inst.detector.elements])
    res['colnames'] = np.array(out.colnames)
    np.savez_compressed(os.path.join(HERE, name + '.npz'), **res)
    print(name, 'n=%d' % n, 'columns:', out.colnames, 'multi-hit:', int(multi.sum()))
    return res


def check_uniform_restatement():
    """numpy's legacy uniform(low, high) is low + (high - low) * random_sample."""
    np.random.seed(6)
    a = np.random.uniform(0.3, 2.7, 1000)
    np.random.seed(6)
    b = 0.3 + (2.7 - 0.3) * np.random.random_sample(1000)
    assert np.array_equal(a, b)


def generate_source():
    """Point-source photons through a CircleAperture, from the reference's
    own RandomArbitraryPdf, polarization_vectors and CircleAperture; the
    unpolarized angle draw is the reference's np.random.uniform(0, 2 pi, n)
    (basesources.py:203-204).  Every uniform is recorded."""
    reference_loader.load()
    from astropy.table import Table
    from marxs.math.random import RandomArbitraryPdf
    from marxs.math.polarization import polarization_vectors
    from marxs.optics.aperture import CircleAperture
    n = 4000
    rng = np.random.default_rng(31)
    x = np.linspace(0.2, 2.0, 60)
    flux = rng.random(60) + 0.05
    flux[7] = 0.0
    pdf_in = np.hstack(([0], flux[1:]))       # Source.generate_energies, basesources.py:190-196
    log = []
    orig = {'uniform': np.random.uniform, 'rand': np.random.rand}

    def uniform(low=0.0, high=1.0, size=None):
        u = np.random.random_sample(size)
        log.append(np.array(u, copy=True))
        return low + (high - low) * u

    def rand(*args):
        u = np.random.random_sample(args if args else None)
        log.append(np.array(u, copy=True))
        return u

    np.random.seed(GLOBAL_SEED + 7)
    np.random.uniform, np.random.rand = uniform, rand
    try:
        sampler = RandomArbitraryPdf(x, pdf_in)
        energies = sampler(n)
        angles = np.random.uniform(0, 2 * np.pi, n)
        dirs = np.tile([-1., 0., 0., 0.], (n, 1))
        pol = polarization_vectors(dirs, angles)
        photons = Table({'dir': dirs, 'energy': energies, 'polarization': pol,
                         'probability': np.ones(n)})
        ap = CircleAperture(position=[12000., 0, 0], zoom=[1, 500, 500], r_inner=300.,
                            phi=[0.1, 5.9])
        photons = ap(photons)
    finally:
        np.random.uniform, np.random.rand = orig['uniform'], orig['rand']
    assert len(log) == 5 and all(len(v) == n for v in log)
    res = {'n': n, 'x': x, 'pdf_in': pdf_in, 'ap_pos4d': np.asarray(ap.geometry.pos4d),
           'r_inner': 300., 'phi': np.array([0.1, 5.9]), 'draws': np.stack(log),
           'cdf': sampler.cdf, 'sortindex': sampler.sortindex, 'bin_width': sampler.bin_width}
    for k in ('pos', 'dir', 'energy', 'polarization', 'probability'):
        res['out_' + k] = np.asarray(photons[k])
    np.savez_compressed(os.path.join(HERE, 'source.npz'), **res)
    print('source n=%d' % n)
    return res


def analysis_photons(seed=41, n=20_000):
    """A synthetic event list: orders -10..10 (float, NaN = no grating hit),
    Gaussian dispersion positions with a few far outliers, some non-finite
    positions, probabilities with zeros, a CCD_ID column with gaps (-1).
    Orders -10, 9 and 10 get 25, 20 and 21 photons (either side of the
    reference's > 20 rule)."""
    rng = np.random.default_rng(seed)
    orders = np.arange(-10, 11)
    weights = np.exp(-0.5 * ((orders + 4) / 3.) ** 2) + 0.05
    order = rng.choice(orders, size=n, p=weights / weights.sum()).astype(float)
    order[np.isin(order, [-10, 9, 10])] = -1.0
    order[rng.random(n) < 0.05] = np.nan
    special = np.zeros(n, dtype=bool)
    for o, k in ((-10, 25), (9, 20), (10, 21)):
        idx = rng.choice(np.flatnonzero((order == -1) & ~special), size=k, replace=False)
        order[idx] = o
        special[idx] = True
    det_x = 30. * order + rng.normal(0, 0.02 + 0.002 * np.abs(np.nan_to_num(order)), n)
    out = (rng.random(n) < 0.01) & ~special
    det_x[out] += rng.standard_cauchy(out.sum()) * 5.
    det_x[(rng.random(n) < 0.01) & ~special] = np.nan
    det_x[np.isnan(order)] = np.nan
    prob = rng.random(n)
    prob[rng.random(n) < 0.03] = 0.0
    ccd = rng.integers(0, 8, n)
    ccd[rng.random(n) < 0.1] = -1
    return {'order': order, 'det_x': det_x, 'probability': prob, 'CCD_ID': ccd}


def generate_analysis():
    """The reference's per-order analysis functions (analysis/gratings.py) on a
    synthetic event list; astropy's sigma_clipped_stats is the oracle's
    restatement (refshim/astropy/stats)."""
    reference_loader.load()
    from astropy.table import Table
    from marxs.analysis import gratings as G
    cols = analysis_photons()
    photons = Table({k: v for k, v in cols.items()})
    orders = np.arange(-10, 11)
    res = {k: v for k, v in cols.items()}
    res['orders'] = orders
    r, pos, std = G.resolvingpower_from_photonlist(photons, orders, col='det_x')
    res['rp_res'], res['rp_pos'], res['rp_std'] = r, pos, std
    r, pos, std = G.resolvingpower_from_photonlist(photons, orders, col='det_x', zeropos=0.5)
    res['rpz_res'], res['rpz_pos'], res['rpz_std'] = r, pos, std
    res['aeff'] = G.effectivearea_from_photonlist(photons, orders, len(photons), A_geom=2.)
    for name, cap in (('cap', G.CaptureResAeff(A_geom=3., orders=orders, dispersion_coord='det_x')),
                      ('ccd', G.CaptureResAeff_CCDgaps(aeff_filter_col='CCD_ID', A_geom=3.,
                                                       orders=orders, dispersion_coord='det_x'))):
        out = cap(photons)
        for k in ('Aeff0', 'Aeffgrat', 'Aeff', 'Rgrat', 'R'):
            res['%s_%s' % (name, k)] = np.ma.filled(np.ma.asarray(out[k], dtype=float), np.nan)
    # too few zeroth-order photons: R of every order is NaN
    few = {k: v.copy() for k, v in cols.items()}
    zero = np.flatnonzero(few['order'] == 0)
    few['order'][zero[19:]] = np.nan
    out = G.CaptureResAeff(orders=orders, dispersion_coord='det_x')(Table(few))
    res['few_order'] = few['order']
    res['few_R'] = np.asarray(out['R'], dtype=float)
    res['few_Aeff'] = np.asarray(out['Aeff'], dtype=float)
    rng = np.random.default_rng(43)
    r = rng.random((2, 4, 5)) * 4000
    r[rng.random(r.shape) < 0.3] = np.nan
    a = rng.random((2, 4, 5)) * 50
    res['avg_r_in'], res['avg_aeff_in'] = r, a
    for ax, key in ((None, 'none'), (0, '0'), (2, '2')):
        ra, aa = G.average_R_Aeff(r, a, axis=ax)
        res['avg_r_' + key] = np.ma.filled(np.ma.asarray(ra, dtype=float), np.nan)
        res['avg_aeff_' + key] = np.asarray(aa, dtype=float)
    np.savez_compressed(os.path.join(HERE, 'analysis.npz'), **res)
    print('analysis n=%d' % len(photons))
    return res


from pose_case import build_pose_parallel, pose_case  # noqa: E402


def generate_poses():
    """The reference's wiggle, moveglobal and moveindividual
    (design/tolerancing.py:45-111) on a Parallel of CAT facets; the normal
    draws of generate_facet_uncertainty are recorded."""
    marxs = reference_loader.load()
    from transforms3d.euler import euler2mat
    from marxs.simulator import Parallel
    from marxs.optics import CATGrating, OrderSelector
    from marxs.design import tolerancing as T
    from types import SimpleNamespace
    ns = SimpleNamespace(Parallel=Parallel, CATGrating=CATGrating, OrderSelector=OrderSelector)
    case = pose_case()
    gas = build_pose_parallel(ns, case, euler2mat)
    res = dict(case)
    res['base_pos4d'] = np.stack([e.geometry.pos4d for e in gas.elements])
    log = []
    orig = np.random.normal

    def normal(loc=0.0, scale=1.0, size=None):
        z = np.random.standard_normal(size)
        log.append(np.array(z, copy=True))
        return loc + scale * z

    np.random.seed(GLOBAL_SEED + 11)
    np.random.normal = normal
    try:
        T.wiggle(gas, dx=0.5, dy=0.3, dz=0.2, rx=1e-3, ry=2e-3, rz=5e-4)
    finally:
        np.random.normal = orig
    assert len(log) == 2
    res['wiggle_sigma'] = np.array([0.5, 0.3, 0.2, 1e-3, 2e-3, 5e-4])
    res['wiggle_pert'] = np.hstack([0 + res['wiggle_sigma'][:3] * log[0],
                                    0 + res['wiggle_sigma'][3:] * log[1]])
    res['wiggle_pos4d'] = np.stack([e.geometry.pos4d for e in gas.elements])
    res['global_move'] = np.array([1.0, -2.0, 0.5, 1e-3, -1e-3, 2e-3])
    T.moveglobal(gas, *res['global_move'])
    res['global_pos4d'] = np.stack([e.geometry.pos4d for e in gas.elements])
    res['indiv_move'] = np.array([0.1, 0.2, 0.3, 1e-4, 2e-4, 3e-4])
    T.moveindividual(gas, *res['indiv_move'])
    res['indiv_pos4d'] = np.stack([e.geometry.pos4d for e in gas.elements])
    np.savez_compressed(os.path.join(HERE, 'poses.npz'), **res)
    print('poses n=%d' % len(gas.elements))
    return res


if __name__ == '__main__':
    check_choice_restatement()
    check_uniform_restatement()
    names = sys.argv[1:] or ['c0', 'c1', 'c2', 'c5', 'c6', 'c7', 'c8', 'c9', 'c10', 'c11',
                             'source', 'analysis', 'poses']
    for name in names:
        if name == 'source':
            generate_source()
        elif name == 'analysis':
            generate_analysis()
        elif name == 'poses':
            generate_poses()
        else:
            generate(name)
