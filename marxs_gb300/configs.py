"""Seeded synthetic instruments and photon lists for the benchmark workloads.

All coordinates are in the MARXS frame: optical axis along +x, photons
travel from large x towards the focus at the origin.

* ``C0`` telescope: annulus aperture r in [300, 500] mm, PerfectLens f=10 m,
  RadialMirrorScatter (5", 1"), FlatDetector 60x60 mm at the focus,
  0.024 mm pixels.
* ``C1`` grating spectrometer: C0 front end, a 20x10 grid of 20x20 mm
  FlatGrating facets (pitch 22 mm, i.e. 2 mm gaps) centred at x=1500 mm,
  each tilted by N(0, 0.1 deg) about its in-plane axes (y, z); d=2e-4 mm;
  an EfficiencyFile-style 64-energy x 13-order table (orders -10..+2,
  Dirichlet(1) rows); FlatDetector 200x60 mm at the focus.
* ``C2`` CAT array: lens f=12 m at x=12000, 1000 CATGrating facets of
  25x25 mm (25 along the dispersion direction y x 40 along z, pitch
  26.5 mm, so that |y| <= 318 mm keeps every photon on the blaze side:
  relative incidence y / 11800 < 1.8 deg) on a Rowland torus R=r=5900 mm,
  blaze 1.8 deg (rotation about the groove axis), N(0, 30") pose jitter
  about three axes; energies from a piecewise-linear spectrum on 200 knots
  in [0.2, 2] keV; CircularDetector (R=5900) on the Rowland circle.
* ``C7`` CCD array: the reference's own Parallel test layout
  (simulator/tests/test_parallel.py:11-23), four 10x10 mm FlatDetectors
  (0.01 mm pixels, 0.2 mm gaps) in one Parallel with id column CCD_ID,
  photons spread over the four chips, the gaps and beyond.
* ``C9`` chirped spectrometer: C1 with every facet's grating constant a
  function of the position on the facet, installed as
  design/bendgratings.py:180-192 does (a RectBivariateSpline, kx = ky = 2,
  of d * corr(y) over the facet, bound as the facet's ``_d``; corr within
  +-1 %), and every third facet with a blaze_angle_modifier linear in the
  local y.
* ``C10`` bent gratings: C1 (facet tilts seeded 10) with every facet bent
  onto a cylinder of radius 1500 mm along its local y, as
  design/bendgratings.py:24-60 bends a facet (the facet's geometry becomes
  a Cylinder whose axis lies 1500 mm behind the facet centre, phi limits
  +-arctan(half width / radius), keeping the groove angle).
* ``C11`` C2 with the CAT facets placed by the reference's own
  RectangularGrid (design/rowland.py:647-700) on its RowlandTorus
  (R = r = 5900 mm), 26.5 mm pitch over y in [-318, 318], z in [-530, 530]
  (960 facets): the placement missions use.  The golden records the grid's
  element positions; this package's build places the facets through a
  Parallel with those positions (the placement is set-up, not the path).
* ``C8`` CAT array + CCD strip: C2 with the CircularDetector replaced by
  16 FlatDetectors of 24.576 mm (0.024 mm pixels, 2.4 mm gaps) tangent to
  the Rowland circle, chip 7 on the focus, placed by ParallelCalculated
  (normals from the circle centre, one side parallel to the circle's axis),
  id column CCD.

The builders take a namespace of element classes so the same instrument
can be assembled from this package's classes or from MARXS itself.
"""
import math
from types import SimpleNamespace

import numpy as np

from . import geomath

ARCSEC = math.pi / 180. / 3600.


def native_namespace():
    from . import optics, simulator
    return SimpleNamespace(
        PerfectLens=optics.PerfectLens, RadialMirrorScatter=optics.RadialMirrorScatter,
        FlatDetector=optics.FlatDetector, CircularDetector=optics.CircularDetector,
        FlatGrating=optics.FlatGrating, CATGrating=optics.CATGrating,
        OrderSelector=optics.OrderSelector, EfficiencyFile=optics.EfficiencyFile,
        InterpolateEfficiencyTable=optics.InterpolateEfficiencyTable.from_grid,
        CATL1L2Stack=optics.CATL1L2Stack, catsupportbars=optics.catsupportbars,
        Cylinder=optics.Cylinder, Parallel=simulator.Parallel, Sequence=simulator.Sequence,
        ParallelCalculated=simulator.ParallelCalculated, angle=lambda rad: rad)


# ---------------------------------------------------------------------------
# photons
# ---------------------------------------------------------------------------
def annulus_photons(n, seed, x0, r_in=300., r_out=500., energy=(0.3, 2.0), energies=None):
    """Photons on an annulus in the plane x=x0, travelling along -x.

    Positions follow the CircleAperture recipe (marxs/optics/aperture.py:138-146):
    phi ~ U(0, 2 pi), r = sqrt(U(r_in^2/r_out^2, 1)) * r_out.  Polarization
    angles ~ U[0, pi) are turned into vectors as polarization_vectors does.
    """
    rng = np.random.default_rng(seed)
    n = int(n)
    phi = rng.uniform(0, 2 * np.pi, n)
    r = np.sqrt(rng.uniform((r_in / r_out) ** 2, 1., n)) * r_out
    if energies is None:
        energies = rng.uniform(energy[0], energy[1], n)
    polangle = rng.uniform(0, np.pi, n)
    pos = np.empty((n, 4))
    pos[:, 0] = x0
    pos[:, 1] = r * np.cos(phi)
    pos[:, 2] = r * np.sin(phi)
    pos[:, 3] = 1.
    dirs = np.zeros((n, 4))
    dirs[:, 0] = -1.
    pol = np.zeros((n, 4))
    # polarization_vectors for dir = -x: v1 = +y, v2 = r x v1 = -z
    pol[:, 1] = np.cos(polangle)
    pol[:, 2] = -np.sin(polangle)
    return {'pos': pos, 'dir': dirs, 'energy': np.asarray(energies, dtype=float),
            'polarization': pol, 'probability': np.ones(n)}


def spectrum_knots(seed, lo=0.2, hi=2.0, n_knots=200):
    """Knots (keV) and flux densities of the seeded CAT-workload spectrum."""
    rng = np.random.default_rng(seed + 1000)
    knots = np.linspace(lo, hi, n_knots)
    w = rng.uniform(0.2, 1.0, n_knots)
    w[rng.integers(0, n_knots, 6)] += rng.uniform(2, 6, 6)     # a few lines
    return knots, w


def piecewise_linear_energies(n, seed, lo=0.2, hi=2.0, n_knots=200):
    """Inverse-CDF samples of a seeded piecewise-linear spectrum on n_knots."""
    knots, w = spectrum_knots(seed, lo, hi, n_knots)
    h = np.diff(knots)
    cum = np.concatenate([[0.], np.cumsum(0.5 * (w[1:] + w[:-1]) * h)])
    target = np.random.default_rng(seed + 2000).uniform(0, 1, int(n)) * cum[-1]
    j = np.clip(np.searchsorted(cum, target, side='right') - 1, 0, n_knots - 2)
    # mass inside segment j: h (w0 t + (w1 - w0) t^2 / 2) for t in [0, 1]
    w0, w1, hj = w[j], w[j + 1], h[j]
    m = (target - cum[j]) / hj
    a = 0.5 * (w1 - w0)
    disc = np.sqrt(np.maximum(w0 * w0 + 4 * a * m, 0.))
    with np.errstate(invalid='ignore', divide='ignore'):
        t = np.where(np.abs(a) > 1e-12, (disc - w0) / (2 * a), m / w0)
    return knots[j] + np.clip(t, 0, 1) * hj


def draws_for(elements_with_draws, n, seed):
    """Per-photon pre-drawn randomness keyed by element object.

    ``elements_with_draws`` lists (element, kind) with kind 'scatter',
    'order' or 'catstack'.  Scatter angles are sigma * N(0, 1); order draws
    are U[0, 1); a CAT stack adds the L1 order and support uniforms, the L2
    scatter's N(0, 1) and the uniform of its turn about the ray.
    """
    rng = np.random.default_rng(seed + 77)
    out = {}
    for elem, kind in elements_with_draws:
        if kind == 'scatter':
            out[elem] = {'inplanescatter': elem.inplanescatter * rng.standard_normal(n),
                         'perpplanescatter': elem.perpplanescatter * rng.standard_normal(n)}
        elif kind == 'catstack':
            out[elem] = {'order_u': rng.uniform(0, 1, n), 'l1_order_u': rng.uniform(0, 1, n),
                         'l1_support_u': rng.uniform(0, 1, n),
                         'l2_normal': rng.standard_normal(n), 'l2_phi_u': rng.uniform(0, 1, n)}
        else:
            out[elem] = {'order_u': rng.uniform(0, 1, n)}
    return out


# ---------------------------------------------------------------------------
# instruments
# ---------------------------------------------------------------------------
def efficiency_table(seed, orders, n_energy=64, lo=0.2, hi=2.0, total=1.0):
    rng = np.random.default_rng(seed + 500)
    e = np.linspace(lo, hi, n_energy)
    p = rng.dirichlet(np.ones(len(orders)), size=n_energy) * total
    # keep every row total <= 1 after rounding (the element protocol rejects
    # probabilities above 1, marxs/optics/base.py:43-46)
    while np.any(np.sum(p, axis=1) > total):
        over = np.sum(p, axis=1) > total
        p[over] *= (1 - 2 ** -50)
    return np.column_stack([e, p])


def build_c0(ns):
    lens = ns.PerfectLens(focallength=10000., position=[10000., 0, 0], zoom=[1, 600, 600])
    rms = ns.RadialMirrorScatter(inplanescatter=ns.angle(5 * ARCSEC),
                                 perpplanescatter=ns.angle(1 * ARCSEC),
                                 position=[10000., 0, 0], zoom=[1, 600, 600])
    det = ns.FlatDetector(zoom=[1, 30, 30], pixsize=0.024)
    return SimpleNamespace(elements=[lens, rms, det], lens=lens, scatter=rms, detector=det,
                           draw_slots=[(rms, 'scatter')], aperture_x=10000.)


def c1_facet_poses(seed, ny=20, nz=10, pitch=22., x=1500., tilt_deg=0.1):
    rng = np.random.default_rng(seed + 300)
    ys = (np.arange(ny) - (ny - 1) / 2) * pitch
    zs = (np.arange(nz) - (nz - 1) / 2) * pitch
    yy, zz = np.meshgrid(ys, zs, indexing='ij')
    positions = [[x, a, b] for a, b in zip(yy.ravel(), zz.ravel())]
    tilts = rng.normal(0, np.deg2rad(tilt_deg), size=(len(positions), 2))
    uncert = [geomath.mat2aff(geomath.euler2mat(0., t[0], t[1], 'sxyz')) for t in tilts]
    return positions, uncert


def build_c1(ns, seed=1, efficiency_file=None):
    front = build_c0(ns)
    orders = list(range(-10, 3))
    table = efficiency_table(seed, orders)
    eff = ns.EfficiencyFile(table if efficiency_file is None else efficiency_file, orders)
    positions, uncert = c1_facet_poses(seed)
    gas = ns.Parallel(elem_class=ns.FlatGrating,
                      elem_args={'d': 2e-4, 'zoom': [1, 10, 10], 'order_selector': eff},
                      elem_pos={'position': positions}, id_col='facet')
    gas.elem_uncertainty = uncert
    gas.generate_elements()
    det = ns.FlatDetector(zoom=[1, 100, 30], pixsize=0.024, ignore_pixel_warning=True)
    return SimpleNamespace(elements=[front.lens, front.scatter, gas, det], lens=front.lens,
                           scatter=front.scatter, gas=gas, detector=det, selector=eff,
                           efficiency_table=table,
                           draw_slots=[(front.scatter, 'scatter'), (gas, 'order')],
                           aperture_x=10000.)


class RowlandTorusGeometry:
    """Torus with symmetry axis y (marxs/design/rowland.py:61-100), identity pose."""

    def __init__(self, R, r):
        self.R = R
        self.r = r
        self.pos4d = np.eye(4)

    def outer_point(self, y, z):
        """Point of the outer branch at given (y, z), found along x."""
        rho = self.R + np.sqrt(self.r ** 2 - y ** 2)
        return np.array([np.sqrt(rho ** 2 - z ** 2), y, z])

    def normal(self, xyz):
        """Outward unit normal (rowland.py:281-337) on the outer branch."""
        x, y, z = xyz
        s = np.sign(np.sqrt(x ** 2 + z ** 2) - self.R)
        theta = np.arcsin(s * y / self.r) + (s < 0) * np.pi
        factor = self.R + self.r * np.cos(theta)
        phi = np.arctan2(z / factor, x / factor)
        return np.array([np.cos(theta) * np.cos(phi), np.sin(theta), np.cos(theta) * np.sin(phi)])


def c2_facet_poses(seed, ny=25, nz=40, pitch=26.5, R=5900., r=5900., jitter_arcsec=30.):
    """Facet poses on the torus (ElementsOnTorus placement, rowland.py:560-580)."""
    torus = RowlandTorusGeometry(R, r)
    ys = (np.arange(ny) - (ny - 1) / 2) * pitch
    zs = (np.arange(nz) - (nz - 1) / 2) * pitch
    poses = []
    for yv in ys:
        for zv in zs:
            p = torus.outer_point(yv, zv)
            nrm = -torus.normal(p)
            rot = geomath.ex2vec_fix(nrm, np.array([0., 1., 0.]))
            poses.append(geomath.compose(p, rot, np.ones(3)))
    rng = np.random.default_rng(seed + 400)
    ang = rng.normal(0, jitter_arcsec * ARCSEC, size=(len(poses), 3))
    uncert = [geomath.compose(np.zeros(3), geomath.euler2mat(a[0], a[1], a[2], 'sxyz'), np.ones(3))
              for a in ang]
    return poses, uncert, torus


def cat_efficiency_grid(seed, orders, total=0.8):
    """Synthetic CAT order efficiencies on a (wavelength nm, blaze deg) grid:
    27 wavelengths in [0.5, 7] nm x 17 blaze angles in [0, 4] deg, Dirichlet(1)
    split of ``total`` over the orders at every node; (n_orders, 27, 17)."""
    rng = np.random.default_rng(seed + 900)
    wave = np.linspace(0.5, 7.0, 27)
    blaze = np.linspace(0.0, 4.0, 17)
    p = rng.dirichlet(np.ones(len(orders)), size=(len(wave), len(blaze))) * total
    while np.any(np.sum(p, axis=-1) > total):
        over = np.sum(p, axis=-1) > total
        p[over] *= (1 - 2 ** -50)
    return wave, blaze, np.moveaxis(p, -1, 0)


def lens_reflectivity(seed):
    """Synthetic mirror reflectivity R(energy keV, grazing angle rad) as a
    degree-1 RectBivariateSpline (the form of PerfectLens's
    reflectivity_interpolator, optics/mirror.py:45-48, 73-79): 30 energies in
    [0.1, 3] keV x 21 angles in [0, 0.02] rad."""
    from scipy.interpolate import RectBivariateSpline
    rng = np.random.default_rng(seed + 950)
    e = np.linspace(0.1, 3.0, 30)
    a = np.linspace(0.0, 0.02, 21)
    ee, aa = np.meshgrid(e, a, indexing='ij')
    R = 0.95 - 0.08 * ee - 12.0 * aa + 0.02 * rng.standard_normal(ee.shape)
    return RectBivariateSpline(e, a, np.clip(R, 0.0, 1.0), kx=1, ky=1)


def l1_transmission_table():
    """Synthetic transmission of a CAT facet's L1 support (energy keV,
    fraction): smooth, rising from 0.04 at 0.05 keV to 0.96 at 5 keV."""
    e = np.linspace(0.05, 5.0, 400)
    return e, 0.96 * np.exp(-(0.12 / e) ** 1.5)


def build_c2(ns, seed=2, efficiency_file=None, n_facets=1000, interpolated=False,
             cat_stack=False):
    """The CAT array; ``interpolated`` gives the lens a reflectivity
    interpolator and the facets an InterpolateEfficiencyTable selector;
    ``cat_stack`` makes every facet a CATL1L2Stack (grating, quality factor,
    L1 and L2 supports) and puts catsupportbars after the array, as the
    Arcus design does (missions/arcus/arcus.py:263-278)."""
    lens_kw = {'reflectivity_interpolator': lens_reflectivity(seed)} if interpolated else {}
    lens = ns.PerfectLens(focallength=12000., position=[12000., 0, 0], zoom=[1, 600, 600],
                          **lens_kw)
    rms = ns.RadialMirrorScatter(inplanescatter=ns.angle(5 * ARCSEC),
                                 perpplanescatter=ns.angle(1 * ARCSEC),
                                 position=[12000., 0, 0], zoom=[1, 600, 600])
    orders = list(range(-12, 3))
    if interpolated:
        table = cat_efficiency_grid(seed, orders)
        eff = ns.InterpolateEfficiencyTable(table[0], table[1], table[2], orders)
    else:
        table = efficiency_table(seed, orders, total=0.8)
        eff = ns.EfficiencyFile(table if efficiency_file is None else efficiency_file, orders)
    poses, uncert, torus = c2_facet_poses(seed)
    poses, uncert = poses[:n_facets], uncert[:n_facets]
    blaze = geomath.axangle2mat(np.array([0, 0, 1.]), np.deg2rad(1.8))
    if cat_stack:
        gas = ns.Parallel(elem_class=ns.CATL1L2Stack,
                          elem_args={'d': 2e-4, 'zoom': [1, 12.5, 12.5], 'orientation': blaze,
                                     'order_selector': eff,
                                     'l1_transmission': l1_transmission_table()},
                          elem_pos=poses, id_col='facet')
    else:
        gas = ns.Parallel(elem_class=ns.CATGrating,
                          elem_args={'d': 2e-4, 'zoom': [1, 12.5, 12.5], 'orientation': blaze,
                                     'order_selector': eff},
                          elem_pos=poses, id_col='facet')
    gas.elem_uncertainty = uncert
    gas.generate_elements()
    cyl = ns.Cylinder.from_rowland(torus, 50., rotation=np.pi,
                                   kwargs={'phi_lim': [-np.pi / 2, np.pi / 2]})
    det = ns.CircularDetector(geometry=cyl, pixsize=0.024)
    elements = [lens, rms, gas, ns.catsupportbars, det] if cat_stack else [lens, rms, gas, det]
    return SimpleNamespace(elements=elements, lens=lens, scatter=rms, gas=gas,
                           detector=det, selector=eff, efficiency_table=table,
                           draw_slots=[(rms, 'scatter'), (gas, 'catstack' if cat_stack else 'order')],
                           aperture_x=12000.)


def ccd_test_photons(n, seed):
    """Rays towards the C7 chips (the x = 0 plane): starts at x = 100 with
    (y, z) uniform in [-16, 6] mm (chips, gaps and the surroundings),
    directions (-1, N(0, 0.01), N(0, 0.01)) normalised, energies U(0.3, 2)
    keV, random linear polarization, probability 1."""
    rng = np.random.default_rng(seed + 300)
    pos = np.zeros((n, 4))
    pos[:, 0] = 100.
    pos[:, 1:3] = rng.uniform(-16., 6., size=(n, 2))
    pos[:, 3] = 1.
    d = np.column_stack([-np.ones(n), rng.normal(0, 0.01, n), rng.normal(0, 0.01, n)])
    d /= np.sqrt(np.sum(d * d, axis=1))[:, None]
    dirs = geomath.e2h(d, 0)
    pol = geomath.polarization_vectors(dirs, rng.uniform(0, np.pi, n))
    return {'pos': pos, 'dir': dirs, 'energy': rng.uniform(0.3, 2.0, n),
            'polarization': pol, 'probability': np.ones(n)}


def build_c7(ns):
    pos = [[0, -10.1, -10.1], [0, .1, -10.1], [0, -10.1, .1], [0, .1, .1]]
    det = ns.Parallel(elem_class=ns.FlatDetector, elem_args={'pixsize': 0.01, 'zoom': 5},
                      elem_pos={'position': pos}, id_col='CCD_ID')
    return SimpleNamespace(elements=[det], detector=det, draw_slots=[])


def rowland_ccd_centres(cyl_pos4d, n_ccd=16, pitch=27.0):
    """Centres (homogeneous) of n_ccd chips at ``pitch`` mm of arc along the
    circle of a Rowland cylinder, chip n_ccd / 2 - 1 centred on the focus
    (the origin), and the circle's centre and axis."""
    T, R, Z, _ = geomath.decompose44(cyl_pos4d)
    r = Z[0]
    phi_f = math.atan2(np.dot(-T, R[:, 1]), np.dot(-T, R[:, 0]))
    phis = phi_f + (np.arange(n_ccd) - n_ccd // 2 + 1) * (pitch / r)      # chip 7 on the focus
    cen = T + r * (np.cos(phis)[:, None] * R[:, 0] + np.sin(phis)[:, None] * R[:, 1])
    return geomath.e2h(cen, 1), T, R[:, 2]


def build_c8(ns, seed=8):
    inst = build_c2(ns, seed=seed)
    xyzw, centre, axis = rowland_ccd_centres(inst.detector.geometry.pos4d)
    ccds = ns.ParallelCalculated(pos_spec=xyzw, normal_spec=geomath.e2h(centre, 1),
                                 parallel_spec=geomath.e2h(axis, 0), elem_class=ns.FlatDetector,
                                 elem_args={'pixsize': 0.024, 'zoom': [1, 12.288, 12.288]},
                                 id_col='CCD')
    return SimpleNamespace(elements=[inst.lens, inst.scatter, inst.gas, ccds], lens=inst.lens,
                           scatter=inst.scatter, gas=inst.gas, detector=ccds,
                           selector=inst.selector, draw_slots=inst.draw_slots)


def chirp_facets(gratings, seed, d=2e-4):
    """Position-dependent grating constants and blaze modifiers on the
    facets of a grating array (any MARXS-like FlatGrating objects): the
    chirp as design/bendgratings.py:180-192 installs it, with a seeded
    correction instead of the optimiser's; a linear blaze modifier on every
    third facet."""
    import types
    from scipy.interpolate import RectBivariateSpline
    rng = np.random.default_rng(seed + 900)
    uarray = np.array([-.999, 0, .999])
    for k, g in enumerate(gratings):
        pos4d = np.asarray(g.geometry.pos4d, dtype=float)
        ly = np.linalg.norm(pos4d[:3, 1])
        lz = np.linalg.norm(pos4d[:3, 2])
        corr = 1.0 + 0.01 * np.tanh(rng.standard_normal(3))
        corr = np.tile(corr, (3, 1)).T
        g.spline = RectBivariateSpline(ly * uarray, lz * uarray, d * corr,
                                       bbox=[-ly, ly, -lz, lz], kx=2, ky=2)

        def func(self, intercoos):
            return self.spline(intercoos[:, 0], intercoos[:, 1], grid=False)
        g._d = types.MethodType(func, g)
        if k % 3 == 0:
            a, b = 1e-3 * rng.standard_normal(), 1e-4 * rng.standard_normal()

            def modifier(self, intercoos, a=a, b=b):
                return a + b * intercoos[:, 0]
            g.blaze_angle_modifier = types.MethodType(modifier, g)


def bend_facets(gratings, radius, ns):
    """Each flat grating's geometry replaced by a Cylinder through its
    centre, curved along the local y, as design/bendgratings.py:24-60 does
    for a facet: axis ``radius`` behind the centre along e_x, zoom
    [radius, radius, z], phi limits +-arctan(half width / radius), the
    geometry dict (groove angle) kept."""
    for e in gratings:
        t, rot, z, _ = geomath.decompose44(np.asarray(e.geometry.pos4d, dtype=float))
        d_phi = np.arctan(z[1] / radius)
        c = ns.Cylinder({'position': t - radius * geomath.h2e(e.geometry['e_x']),
                         'orientation': rot, 'zoom': [radius, radius, z[2]],
                         'phi_lim': [-d_phi, d_phi]})
        c._geometry = e.geometry._geometry
        e.geometry = c


def build_c10(ns, seed=10, radius=1500.):
    inst = build_c1(ns, seed=seed)
    bend_facets(inst.gas.elements, radius, ns)
    return inst


def build_c11(ns, seed=11, elem_pos=None):
    """C2 with RectangularGrid facets; ``elem_pos``: the grid's element
    positions (required unless ``ns`` holds the reference's RowlandTorus
    and RectangularGrid)."""
    inst = build_c2(ns, seed=seed)
    blaze = geomath.axangle2mat(np.array([0, 0, 1.]), np.deg2rad(1.8))
    args = {'d': 2e-4, 'zoom': [1, 12.5, 12.5], 'orientation': blaze,
            'order_selector': inst.selector}
    if elem_pos is None:
        torus = ns.RowlandTorus(5900., 5900.)
        gas = ns.RectangularGrid(rowland=torus, d_element=[26.5, 26.5], y_range=[-318., 318.],
                                 z_range=[-530., 530.], elem_class=ns.CATGrating,
                                 elem_args=args, id_col='facet')
    else:
        gas = ns.Parallel(elem_class=ns.CATGrating, elem_args=args,
                          elem_pos=[np.asarray(p, dtype=float) for p in elem_pos], id_col='facet')
    return SimpleNamespace(elements=[inst.lens, inst.scatter, gas, inst.detector], lens=inst.lens,
                           scatter=inst.scatter, gas=gas, detector=inst.detector,
                           selector=inst.selector, draw_slots=[(inst.scatter, 'scatter'),
                                                               (gas, 'order')])


def build_c9(ns, seed=9):
    inst = build_c1(ns, seed=seed)
    chirp_facets(inst.gas.elements, seed)
    return inst


def photons_for(config_name, n, seed):
    if config_name == 'c7':
        return ccd_test_photons(n, seed)
    if config_name in ('c2', 'c5', 'c6', 'c8', 'c11'):
        e = piecewise_linear_energies(n, seed)
        return annulus_photons(n, seed, 12000., energies=e)
    return annulus_photons(n, seed, 10000.)


def build(config_name, ns=None, seed=None, **kwargs):
    ns = native_namespace() if ns is None else ns
    if config_name == 'c0':
        return build_c0(ns)
    if config_name == 'c1':
        return build_c1(ns, seed=1 if seed is None else seed)
    if config_name == 'c2':
        return build_c2(ns, seed=2 if seed is None else seed)
    if config_name == 'c5':
        return build_c2(ns, seed=5 if seed is None else seed, interpolated=True)
    if config_name == 'c6':
        return build_c2(ns, seed=6 if seed is None else seed, interpolated=True, cat_stack=True)
    if config_name == 'c7':
        return build_c7(ns)
    if config_name == 'c8':
        return build_c8(ns, seed=8 if seed is None else seed)
    if config_name == 'c9':
        return build_c9(ns, seed=9 if seed is None else seed)
    if config_name == 'c10':
        return build_c10(ns, seed=10 if seed is None else seed)
    if config_name == 'c11':
        return build_c11(ns, seed=11 if seed is None else seed, **kwargs)
    raise ValueError(config_name)
