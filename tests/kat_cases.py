"""Known-answer cases restated from the MARXS reference's own unit tests.

Each case takes a runner and asserts the reference's known answers:
* geometry: marxs/math/tests/test_geometry.py:11-240
* polarization transport: marxs/math/tests/test_polarization.py:36-72
* gratings: marxs/optics/tests/test_grating.py:16-223
* detector pixels: marxs/optics/tests/test_detector.py:16-36
* lens: marxs/optics/tests/test_mirror.py:14-80
* scatter special cases: marxs/optics/tests/test_scatter.py:46-74

A runner provides ``plane_intersect(geometry, dir, pos)``,
``cylinder_intersect(geometry, dir, pos)``, ``transport(d1, d2, pol)`` and
``trace(elements, photons, draws=None)`` (dict of output columns).  The CPU
runner is the oracle; the GPU runner goes through the CUDA library.
"""
import numpy as np

from marxs_gb300 import optics, geomath
from marxs_gb300.optics import (FinitePlane, Cylinder, FlatGrating, CATGrating, OrderSelector,
                                FlatDetector, PerfectLens, RadialMirrorScatter)

ENERGY2WAVE = 1.2398419292004202e-06


def test_photons(n=1):
    """n identical photons: pos (1,0,0), dir -x, pol +y, 1 keV (marxs/utils.py:16-51)."""
    return {'pos': np.tile([1., 0., 0., 1.], (n, 1)), 'dir': np.tile([-1., 0., 0., 0.], (n, 1)),
            'energy': np.ones(n), 'polarization': np.tile([0., 1., 0., 0.], (n, 1)),
            'probability': np.ones(n)}


def closeornan(a, b):
    a, b = np.asarray(a, dtype=float), np.asarray(b, dtype=float)
    if not np.array_equal(np.isnan(a), np.isnan(b)):
        return False
    m = ~np.isnan(a)
    return np.allclose(a[m], b[m])


# ----------------------------------------------------------------- geometry
def case_plane_forwards(r):
    pos = np.array([[20., 0., 0.8, 1.], [0., .0, 0.4, 1.], [-5., .1, -.2, 1]])
    dir = np.array([[-.1, 0., 0., 0], [-1., 0, 0.02, 0.], [-2., -0.02, 0.023, 0.]])
    plane = FinitePlane()
    i, _, _ = r.plane_intersect(plane, dir, pos)
    assert list(i) == [True, True, False]
    i, _, _ = r.plane_intersect(plane, -dir, pos)
    assert list(i) == [False, True, True]


def case_plane_zoomed(r):
    pos = np.array([[1., 4., 0.8, 1.], [1., -4., 8., 1.], [1., -6., -8., 1]])
    dir = np.array([[-.1, 0., 0., 0], [-1., 0, 0.02, 0.], [-2., -0.02, 0.023, 0.]])
    plane = FinitePlane({'zoom': [1, 5, 10]})
    i, ip, loc = r.plane_intersect(plane, dir, pos)
    assert list(i) == [True, True, False]
    assert np.all(ip[0, :] == [0, 4, .8, 1])
    assert np.all(loc[0] == [4, .8])
    assert np.all(np.isnan(ip[2, :3])) and np.all(np.isnan(loc[2]))


def case_plane_moved(r):
    pos = np.array([[4.1, 5.5, 6.8, 1.], [5., 4.1, 4.99, 1.], [4.1, 3., 6., 1]])
    dir = np.array([[-.1, 0., 0., 0], [-1., 0, 0.02, 0.], [-2., -0.02, 0.023, 0.]])
    plane = FinitePlane({'position': [4, 5, 6]})
    i, ip, loc = r.plane_intersect(plane, dir, pos)
    assert list(i) == [True, True, False]
    assert np.all(ip[1, :] == [4, 4.1, 5.01, 1])
    assert np.allclose(loc[1, :], [-0.9, -.99])


def case_tube_miss(r):
    circ = Cylinder()
    s, p, l = r.cylinder_intersect(circ, np.array([[1., 0., .1, 0], [-1., -1., 0., 0.]]),
                                   np.array([[0, -1.1, 0., 1.], [2., 0., 0., 1.]]))
    assert np.all(~s) and np.all(np.isnan(p)) and np.all(np.isnan(l))
    s, p, l = r.cylinder_intersect(circ, np.array([[0., 0.1, 1., 0]]), np.array([[0.5, 0.5, 0., 1.]]))
    assert np.all(~s) and np.all(np.isnan(p)) and np.all(np.isnan(l))
    circ = Cylinder({'position': [0.8, 0.8, 1.2]})
    s, p, l = r.cylinder_intersect(circ, np.array([[1., 0., .0, 0], [1., 0., 0., 0.]]),
                                   np.array([[0., 0., 0., 1.], [0., -0.3, 1., 1.]]))
    assert np.all(~s) and np.all(np.isnan(p)) and np.all(np.isnan(l))


def case_tube_forward(r):
    pos = np.array([[20., 0., 0.8, 1.], [0., .0, 0.4, 1.], [-5., .1, -.2, 1]])
    dir = np.array([[-.1, 0., 0., 0], [-1., 0, 0.02, 0.], [-2., -0.02, 0.023, 0.]])
    circ = Cylinder({'zoom': [1, 1, 1]})
    i, _, _ = r.cylinder_intersect(circ, dir, pos)
    assert list(i) == [True, True, False]
    i, _, _ = r.cylinder_intersect(circ, -dir, pos)
    assert list(i) == [False, True, True]


def case_tube_hitmiss_zoomed(r):
    dir = np.array([[-.1, 0., 0., 0], [-1., 0, 0.2, 0.]])
    pos = np.array([[20., 0., 0.8, 1.], [2., .0, 0.4, 1.]])
    i, _, _ = r.cylinder_intersect(Cylinder({'zoom': [1, 1, 1]}), dir, pos)
    assert np.all(i)
    i, p, l = r.cylinder_intersect(Cylinder({'zoom': [1, 1, .5]}), dir, pos)
    assert np.all(~i) and np.all(np.isnan(p)) and np.all(np.isnan(l))


def case_tube_2points(r):
    dir = np.array([[-.1, 0., 0., 0], [-0.5, 0, 0., 0.], [-1., 0., 0., 0.]])
    pos = np.array([[50., 0., 0., 1.], [10., .5, 0., 1.], [2, 0, .3, 1.]])
    i, ip, loc = r.cylinder_intersect(Cylinder(), dir, pos)
    assert np.all(i)
    assert np.allclose(ip[:, :3], [[1., 0., 0.], [np.sqrt(0.75), 0.5, 0.], [1, 0., .3]])
    assert np.allclose(loc, np.array([[0., np.arcsin(0.5), 0.], [0., 0., 0.3]]).T)


def case_tube_2points_transformed(r):
    pos = np.array([[50., 0., 0., 1.], [10., .5, 0., 1.], [2, 0, .3, 1.]])
    dir = np.array([[-.1, 0., 0., 0], [-0.5, 0, 0., 0.], [-1., 0., 0., 0.]])
    exp_loc = np.array([[0., np.arcsin(0.5), 0.], [0., 0., 0.3]]).T
    exp_ip = np.array([[1., 0., 0.], [np.sqrt(0.75), 0.5, 0.], [1, 0., .3]])
    i, ip, loc = r.cylinder_intersect(Cylinder({'zoom': [1, 1., 5.]}), dir, pos)
    assert np.all(i) and np.allclose(ip[:, :3], exp_ip) and np.allclose(loc, exp_loc)
    orient = geomath.axangle2mat([0, 0, 1], -.3)
    i, ip, loc = r.cylinder_intersect(Cylinder({'orientation': orient}), dir, pos)
    assert np.all(i) and np.allclose(ip[:, :3], exp_ip)
    assert np.allclose(loc, np.array([[0.3, 0.3 + np.arcsin(0.5), 0.3], [0., 0., 0.3]]).T)
    i, ip, loc = r.cylinder_intersect(Cylinder({'position': [-.3, 0, 0]}), dir, pos)
    assert np.all(i)
    assert np.allclose(ip[:, :3], [[.7, 0, 0], [np.sqrt(0.75) - .3, 0.5, 0.], [.7, 0., .3]])
    assert np.allclose(loc, exp_loc)


def case_tube_phi_lim(r):
    pos = np.array([[50., 0., 0., 1.], [10., .5, 0., 1.], [2, 0, .3, 1.]])
    dir = np.array([[-.1, 0., 0., 0], [-0.5, 0, 0., 0.], [-1., 0., 0., 0.]])
    i, ip, loc = r.cylinder_intersect(Cylinder({'phi_lim': [.6, np.pi]}), dir, pos)
    assert np.all(i)
    assert np.allclose(ip[:, :3], [[-1., 0., 0.], [-np.sqrt(0.75), 0.5, 0.], [-1, 0., .3]])
    assert np.allclose(loc, np.array([[np.pi, np.pi - np.arcsin(0.5), np.pi], [0., 0., 0.3]]).T)
    i, ip, loc = r.cylinder_intersect(Cylinder({'phi_lim': [-.4, -.3]}), dir, pos)
    assert np.all(~i) and np.all(np.isnan(ip)) and np.all(np.isnan(loc))


def case_tube_translation(r):
    circ = Cylinder({'position': [0.8, 0.8, 1.2], 'zoom': [1, 1, 2]})
    s, p, _ = r.cylinder_intersect(circ, np.array([[1., 0., .0, 0], [1., 0., 0., 0.]]),
                                   np.array([[0., 0., 0., 1.], [0., 0., 1., 1.]]))
    assert np.all(s)
    assert np.allclose(p[:, :3], [[.2, 0., 0.], [.2, 0., 1.]])


# ------------------------------------------------------------- polarization
def case_parallel_transport(r):
    dir1 = geomath.norm_vector(np.array([[1, -1, 0]] * 5, dtype=float))
    dir2 = geomath.norm_vector(np.array([[1, -1, 0], [1, 1, 0], [1, 1, 0], [1, 0.2, 0],
                                         [1, 0.2, 0]], dtype=float))
    polin = geomath.norm_vector(np.array([[1, 1, 1], [0, 0, 1], [1, 1, 0], [0, 0, 1], [1, 1, 0]],
                                         dtype=float))
    out = r.transport(dir1, dir2, polin)[:, :3]
    assert np.allclose(polin[0], out[0])                     # dir1 == dir2: unchanged
    assert np.allclose(polin[:, 2], out[:, 2])               # s component unchanged
    assert np.allclose(np.linalg.norm(out, axis=1), 1)
    assert np.allclose(np.einsum('ij,ij->i', out, dir2), 0)  # perpendicular to dir2


# ----------------------------------------------------------------- gratings
def case_grating_zero_order(r):
    rng = np.random.default_rng(3)
    dir = rng.random((10, 4))
    dir[:, 1:] = 0              # photons at x in [-1, 0) moving along +x
    dir[:, 0] += 0.1
    ph = {'pos': np.c_[rng.random((10, 3)) - 1, np.ones(10)], 'dir': dir,
          'energy': rng.random(10) + 0.1,
          'polarization': geomath.polarization_vectors(dir, rng.random(10)),
          'probability': np.ones(10)}
    g0 = FlatGrating(d=1. / 500., order_selector=OrderSelector([0]), zoom=np.array([1., 50., 50.]))
    out = r.trace([g0], ph, {g0: {'order_u': np.full(10, 0.5)}})
    d_in = geomath.norm_vector(dir[:, :3])
    d_out = geomath.norm_vector(out['dir'][:, :3])
    assert np.allclose(d_in, d_out)
    assert np.allclose(out['pos'][:, 0], 0.)


def case_grating_angle_dependence(r):
    d = 0.001
    beta = np.deg2rad([0., 5., 10., 20.])
    dir = np.zeros((4, 4))
    dir[:, 1] = np.sin(beta)
    dir[:, 0] = -np.cos(beta)
    ph = {'pos': np.ones((4, 4)), 'dir': dir, 'energy': np.ones(4),
          'polarization': geomath.polarization_vectors(dir, [1, 2, 3, 4]), 'probability': np.ones(4)}
    g = FlatGrating(d=d, order_selector=OrderSelector([1]), zoom=20)
    out = r.trace([g], ph, {g: {'order_u': np.full(4, 0.5)}})
    alpha = np.arctan2(out['dir'][:, 1], -out['dir'][:, 0])
    assert np.allclose(np.sin(alpha), np.sin(beta) + ENERGY2WAVE / d)


def case_grating_order_dependence(r):
    ph = {'pos': np.ones((5, 4)), 'dir': np.tile([-1., 0, 0, 0], (5, 1)), 'energy': np.ones(5),
          'polarization': np.tile([0., 1., 0., 0.], (5, 1)), 'probability': np.ones(5)}
    g = FlatGrating(d=1. / 500, order_selector=OrderSelector([-2, -1, 0, 1, 2]))
    out = r.trace([g], ph, {g: {'order_u': (np.arange(5) + 0.5) / 5}})
    assert list(out['order']) == [-2, -1, 0, 1, 2]
    assert np.allclose(out['dir'][:, 2], 0.)
    assert np.allclose(out['dir'][[0, 1], 1], - out['dir'][[4, 3], 1])
    assert np.abs(out['dir'][4, 1] / out['dir'][3, 1] - 2) < 0.00001


def case_grating_energy_dependence(r):
    ph = {'pos': np.ones((5, 4)), 'dir': np.tile([-1., 0, 0, 0], (5, 1)),
          'energy': np.arange(1., 6), 'polarization': np.tile([0, 1., 0., 0.], (5, 1)),
          'probability': np.ones(5)}
    g = FlatGrating(d=1. / 500, order_selector=OrderSelector([1]))
    out = r.trace([g], ph, {g: {'order_u': np.full(5, 0.3)}})
    assert np.allclose(out['dir'][:, 2], 0.)
    lam = ENERGY2WAVE / out['energy']
    theta = np.arctan2(out['dir'][:, 1], out['dir'][:, 0])
    assert np.allclose(1. * lam, 1. / 500. * np.sin(theta))


def case_grating_translation_invariance(r):
    ph = test_photons(2)
    ph['dir'] = np.tile(np.array([-1., 2., 3., 0.]), (2, 1))
    ph['polarization'] = geomath.polarization_vectors(ph['dir'], [2., 4.])
    delta = np.array([0, .23, -.34, 0.])
    ph['pos'][1, :] += delta
    for order in [-1, 0, 1]:
        g = FlatGrating(d=1. / 500, order_selector=OrderSelector([order]), zoom=20)
        out = r.trace([g], {k: v.copy() for k, v in ph.items()}, {g: {'order_u': np.full(2, .5)}})
        assert np.all(out['order'] == order)
        assert np.allclose(out['pos'][:, 0], 0)
        assert np.allclose(out['dir'][0, :], out['dir'][1, :])
        assert np.allclose(out['pos'][0, :], out['pos'][1, :] - delta)


def case_cat_order_convention(r):
    dirs = np.array([[-1, 0., 0., 0], [-1, 0.01, -0.01, 0], [-1, 0.01, 0.01, 0],
                     [-1, -0.01, 0.01, 0], [-1, -0.01, -0.01, 0]])
    ph = {'pos': np.ones((5, 4)), 'dir': dirs, 'energy': np.ones(5),
          'polarization': geomath.polarization_vectors(dirs, np.arange(5)), 'probability': np.ones(5)}
    gp = CATGrating(d=1. / 5000, order_selector=OrderSelector([5]), zoom=2)
    p5 = r.trace([gp], {k: v.copy() for k, v in ph.items()}, {gp: {'order_u': np.full(5, .5)}})
    gm = CATGrating(d=1. / 5000, order_selector=OrderSelector([-5]), zoom=2)
    m5 = r.trace([gm], {k: v.copy() for k, v in ph.items()}, {gm: {'order_u': np.full(5, .5)}})
    assert np.all(p5['dir'][1:3, 1] > 0)
    assert np.all(p5['dir'][3:, 1] < 0)
    assert np.all(m5['dir'][1:3, 1] < 0)
    assert np.all(m5['dir'][3:, 1] > 0)


def case_cat_misses_are_nan(r):
    ph = test_photons(5)
    ph['pos'][:, 1] = np.arange(5)
    cat = CATGrating(d=1. / 5000, order_selector=OrderSelector([5]), zoom=2)
    out = r.trace([cat], ph, {cat: {'order_u': np.full(5, .5)}})
    assert np.all(np.isnan(out['order'][3:]))
    assert np.all(np.isnan(out['grat_y'][3:]))
    assert np.all(out['order'][:3] == 5)


# ----------------------------------------------------------------- detector
def case_detector_pixels(r):
    pos = np.array([[0, 0., -0.25, 1.], [0., 9.9, 1., 1.], [0., 10.1, 1., 1.]])
    dir = np.ones((3, 4))
    dir[:, 3] = 0.
    pol = np.zeros((3, 4))
    pol[:, 1] = 1
    ph = {'pos': pos, 'dir': dir, 'energy': np.array([1, 2., 3.]), 'polarization': pol,
          'probability': np.ones(3)}
    det = FlatDetector(zoom=[1., 10., 5.], pixsize=0.5)
    assert det.npix == [40, 20] and det.centerpix == [19.5, 9.5]
    out = r.trace([det], ph)
    assert closeornan(out['det_x'], [0, 9.9, np.nan])
    assert closeornan(out['det_y'], [-0.25, 1., np.nan])
    assert closeornan(out['detpix_x'], [19.5, 39.3, np.nan])
    assert closeornan(out['detpix_y'], [9, 11.5, np.nan])


# --------------------------------------------------------------------- lens
def case_perfect_lens_focus(r):
    f = 1000.
    for ra in (0., 30., -60.):
        a = np.deg2rad(ra)
        n = 60
        rng = np.random.default_rng(int(ra) + 100)
        y, z = rng.uniform(-2, 2, n), rng.uniform(-2, 2, n)
        # parallel rays from a source at angle ra in the x-z plane, on the lens plane x = 0
        dirs = np.tile([-np.cos(a), 0., np.sin(a), 0.], (n, 1))
        ph = {'pos': np.c_[np.zeros(n), y, z, np.ones(n)], 'dir': dirs, 'energy': np.ones(n),
              'polarization': geomath.polarization_vectors(dirs, rng.random(n)),
              'probability': np.ones(n)}
        lens = PerfectLens(focallength=f, zoom=400)
        d = f * np.cos(a)
        det = FlatDetector(pixsize=0.01, position=np.array([-d, 0, 0]), zoom=1e5)
        out = r.trace([lens, det], ph)
        assert np.std(out['det_x']) < 1e-4 and np.std(out['det_y']) < 1e-4
        det2 = FlatDetector(pixsize=0.01, position=np.array([-2 * d, 0, 0]), zoom=1e5)
        out2 = r.trace([lens, det2], {k: v.copy() for k, v in ph.items()})
        assert np.std(out2['det_x']) > 1e-4 and np.std(out2['det_y']) > 1e-4


def case_perfect_lens_offset(r):
    lens = PerfectLens(focallength=100, position=[0, 0, 10], zoom=400)
    lens2 = PerfectLens(focallength=100, position=[0, 0, 0], zoom=400, d_center_optical_axis=-10)
    p1 = r.trace([lens], test_photons(1))
    p2 = r.trace([lens2], test_photons(1))
    assert np.allclose(p1['dir'], p2['dir'])


def case_perfect_lens_reflectivity(r):
    """test_PerfectLens_refl (test_mirror.py:62-80): a degree-1 spline of
    exp(-sqrt((x/2)^2 + y^2)) on a 100 x 100 grid, at (1 keV, 0 rad), squared."""
    from scipy.interpolate import RectBivariateSpline
    xarr = np.linspace(-3, 3, 100)
    yarr = np.linspace(-3, 3, 100)
    xgrid, ygrid = np.meshgrid(xarr, yarr, indexing='ij')
    zdata = np.exp(-np.sqrt((xgrid / 2) ** 2 + ygrid ** 2))
    interp = RectBivariateSpline(xarr, yarr, zdata, kx=1, ky=1)
    lens = PerfectLens(focallength=123.0, reflectivity_interpolator=interp)
    out = r.trace([lens], test_photons(1))
    assert np.allclose(out['energy'], 1)
    assert np.allclose(out['polarization'], [0, 1, 0, 0])
    assert np.allclose(out['probability'], 0.367205)


# ------------------------------------------------------------------ scatter
def case_scatter_zero_sigma(r):
    ph = test_photons(500)
    ph['pos'] = np.tile(np.array([0., 1., 0., 1.]), (500, 1))
    rms = RadialMirrorScatter(inplanescatter=0., perpplanescatter=0.)
    det = FlatDetector(position=[-1, 0, 0], zoom=1000)
    out = r.trace([rms, det], ph, {rms: {'inplanescatter': np.zeros(500),
                                         'perpplanescatter': np.zeros(500)}})
    assert np.all(out['det_x'] == 1.0)
    assert np.all(out['det_y'] == 0)


def case_grating_d_callable(r):
    """marxs/optics/tests/test_grating.py:297-311: d can be a function of the
    local coordinates; the photon at local y < 0 sees half the grating
    constant and leaves at twice the angle."""
    photons = test_photons(5)
    photons['pos'][0, 1] = 1.
    photons['pos'][1, 1] = -1.

    def dfunc(intercoos):
        darr = np.ones(intercoos.shape[0]) * 2e-4
        return np.where(intercoos[:, 0] >= 0, darr, darr / 2.)

    grat = FlatGrating(order_selector=OrderSelector([1]), zoom=2, d=dfunc)
    p = r.trace([grat], photons, {grat: {'order_u': np.full(5, 0.5)}})
    assert np.abs(p['dir'][1, 1] / p['dir'][0, 1] - 2) < 0.00001


def case_grating_blaze_angle_modifier(r):
    """An overridden blaze_angle_modifier (grating.py:222-231) adds to the
    blaze angle at each photon's local coordinates: at normal incidence the
    blaze column is the modifier itself."""
    photons = test_photons(4)
    photons['pos'][:, 1] = [-1.5, -0.5, 0.5, 1.5]
    grat = FlatGrating(order_selector=OrderSelector([0]), zoom=2, d=2e-4)
    grat.blaze_angle_modifier = lambda intercoos: 0.01 + 0.001 * intercoos[:, 0]
    p = r.trace([grat], photons, {grat: {'order_u': np.full(4, 0.5)}})
    assert np.allclose(p['blaze'], 0.01 + 0.001 * np.array([-1.5, -0.5, 0.5, 1.5]),
                       rtol=0, atol=1e-12)


CASES = [v for k, v in sorted(globals().items()) if k.startswith('case_')]
