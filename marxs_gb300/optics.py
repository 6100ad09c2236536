"""Element descriptors that mirror the MARXS element classes on the raytrace path.

They carry exactly the parameters the GPU backend lowers, under the same
attribute names the MARXS classes use, so that ``GpuSequence`` lowers either
these objects or genuine MARXS objects (duck-typed).  They do no photon
arithmetic themselves: calling one through ``GpuSequence`` runs the CUDA
kernels.  Constructor keywords follow the reference:

* ``FinitePlane`` / ``Cylinder``        -- marxs/math/geometry.py:196-281, 379-626
* ``OrderSelector`` / ``EfficiencyFile`` -- marxs/optics/grating.py:12-96
* ``FlatGrating`` / ``CATGrating``      -- marxs/optics/grating.py:99-301
* ``PerfectLens``                       -- marxs/optics/mirror.py:11-82
* ``RadialMirrorScatter``               -- marxs/optics/scatter.py:24-77
* ``FlatDetector`` / ``CircularDetector`` -- marxs/optics/detector.py:18-118
"""
import warnings

import math

import numpy as np

from .geomath import parse_position_keywords, decompose44, compose, axangle2mat


class GeometryError(Exception):
    pass


class SimulationSetupWarning(Warning):
    pass


def _to_rad(value):
    """Accept a float in rad or a quantity-like object with ``.to(unit)``."""
    if hasattr(value, 'to') and hasattr(value, 'unit'):
        try:
            import astropy.units as u  # only when the caller passes quantities
            return float(value.to(u.rad).value)
        except ImportError:  # pragma: no cover
            pass
    return float(value)


class Geometry:
    loc_coos_name = ['y', 'z']

    def __init__(self, kwargs=None):
        kwargs = {} if kwargs is None else kwargs
        self.pos4d = parse_position_keywords(kwargs)
        self._geometry = {}

    def __getitem__(self, key):
        if key == 'center':
            return self.pos4d[:, 3]
        if key in ('v_x', 'e_x'):
            val = self.pos4d[:, 0]
        elif key in ('v_y', 'e_y'):
            val = self.pos4d[:, 1]
        elif key in ('v_z', 'e_z'):
            val = self.pos4d[:, 2]
        else:
            val = self._geometry[key]
            if isinstance(val, np.ndarray) and val.shape[-1] == 4:
                val = np.dot(self.pos4d, val)
        if key[:2] == 'e_':
            return val / np.linalg.norm(val)
        return val


class FinitePlane(Geometry):
    """Flat rectangle in the local y-z plane spanning +-v_y, +-v_z."""
    shape = 'box'
    loc_coos_name = ['y', 'z']


class Cylinder(Geometry):
    """Tube of unit radius along local z (scaled by the pose's zoom)."""
    loc_coos_name = ['phi', 'z']
    shape = 'surface'

    def __init__(self, kwargs=None):
        kwargs = {} if kwargs is None else dict(kwargs)
        self.coos_limits = [np.asanyarray(kwargs.pop('phi_lim', [-np.pi, np.pi])),
                            np.array([-1, 1])]
        super().__init__(kwargs)

    def __getitem__(self, value):
        if value == 'R':
            return decompose44(self.pos4d)[2][0]
        return super().__getitem__(value)

    @classmethod
    def from_rowland(cls, rowland, width, rotation=0., kwargs=None):
        rot = axangle2mat(np.array([0, 0, 1.]), rotation)
        pos4d_circ = compose([rowland.R, 0, 0], rot, [rowland.r, rowland.r, width])
        pos4d_circ = np.dot(rowland.pos4d, pos4d_circ)
        det_kwargs = {'pos4d': pos4d_circ}
        det_kwargs.update(kwargs or {})
        return cls(det_kwargs)


class OrderSelector:
    """Energy-independent order probabilities (marxs/optics/grating.py:12-57)."""

    def __init__(self, orderlist, p=None):
        self.orderlist = orderlist
        if p is None:
            self.p = np.ones(len(orderlist)) / len(orderlist)
        else:
            p = np.asanyarray(p)
            if len(p) != len(orderlist):
                raise ValueError('Number of elements in orderlist and probabilities does not match.')
            if p.sum() > 1.:
                raise ValueError('Sum of all probabilities must be <= 1.')
            if np.any(p < 0):
                raise ValueError('Probabilities cannot be negative')
            self.p = p


class EfficiencyFile:
    """Order probabilities on an energy grid, nearest row (grating.py:60-96).

    ``filename`` is a text file (first column energy in keV, one column per
    order) or an ``(n_energy, 1 + n_orders)`` array with the same layout.
    """

    def __init__(self, filename, orders):
        if isinstance(filename, np.ndarray):
            dat = np.array(filename, dtype=float)
        else:
            dat = np.loadtxt(filename)
        self.energy = dat[:, 0]
        if len(orders) != (dat.shape[1] - 1):
            raise ValueError('orders has len={0}, but data files has {1} order columns.'.format(
                len(orders), dat.shape[1] - 1))
        self.orders = np.array(orders)
        self.prob = dat[:, 1:]
        self.totalprob = np.sum(self.prob, axis=1)
        self.cumprob = np.cumsum(self.prob, axis=1) / self.totalprob[:, None]


class InterpolateEfficiencyTable:
    """Order probabilities interpolated in (wavelength, blaze angle)
    (missions/mitsnl/catgrating.py:63-144): one RectBivariateSpline of degree
    ``k`` per order on a regular grid.

    ``tab`` is table-like: first column wavelength (nm), second blaze angle
    (deg), rows flattened wavelength-major as tablerows_to_2d reads them
    (utils.py:59-100), then one column per order named by the order number.
    ``from_grid`` builds the same from arrays.
    """

    def __init__(self, tab, k=1):
        from scipy.interpolate import RectBivariateSpline
        names = list(tab.colnames)
        x = np.asarray(tab[names[0]], dtype=float)
        y = np.asarray(tab[names[1]], dtype=float)
        n_x, n_y = len(set(x)), len(set(y))
        if len(x) != n_x * n_y:
            raise ValueError('Data is not on regular grid.')
        wave = x[::n_y]
        theta = y[:n_y] * (math.pi / 180.)
        self.orders = np.array([int(n) for n in names[2:]])
        self.interpolators = [
            RectBivariateSpline(wave, theta, np.asarray(tab[nm], dtype=float).reshape(n_x, n_y),
                                kx=k, ky=k) for nm in names[2:]]

    @classmethod
    def from_grid(cls, wave_nm, blaze_deg, probs, orders, k=1):
        """probs: (n_orders, n_wave, n_blaze)."""
        ww, bb = np.meshgrid(np.asarray(wave_nm, float), np.asarray(blaze_deg, float),
                             indexing='ij')
        tab = {'wave': ww.ravel(), 'blaze': bb.ravel()}
        for i, o in enumerate(orders):
            tab[str(int(o))] = np.asarray(probs[i], dtype=float).ravel()

        class _Tab(dict):
            colnames = property(lambda self: list(self.keys()))
        return cls(_Tab(tab), k=k)


class SimulationSequenceElement:
    id_col = None
    output_columns = []

    def __init__(self, **kwargs):
        self.id_num = kwargs.pop('id_num', -9)
        if 'id_col' in kwargs:
            self.id_col = kwargs.pop('id_col')
        self.name = kwargs.pop('name', self.__class__.__name__)
        if kwargs:
            raise ValueError('Initialization arguments {0} not understood'.format(
                ', '.join(kwargs.keys())))

    def __call__(self, photons):
        from .gpu import GpuSequence
        return GpuSequence(elements=[self])(photons)


class OpticalElement(SimulationSequenceElement):
    default_geometry = FinitePlane

    def __init__(self, **kwargs):
        geometry = kwargs.pop('geometry', self.default_geometry)
        if isinstance(geometry, Geometry):
            self.geometry = geometry
        else:
            self.geometry = geometry(kwargs)
        super().__init__(**kwargs)
        if not hasattr(self, 'loc_coos_name'):
            self.loc_coos_name = self.geometry.loc_coos_name

    @property
    def pos4d(self):
        return self.geometry.pos4d


class FlatOpticalElement(OpticalElement):
    pass


class PerfectLens(FlatOpticalElement):
    loc_coos_name = ['mirror_x', 'mirror_y']

    def __init__(self, **kwargs):
        self.focallength = kwargs.pop('focallength')
        self.d_center_optax = kwargs.pop('d_center_optical_axis', 0)
        self.reflectivity_interpolator = kwargs.pop('reflectivity_interpolator', None)
        super().__init__(**kwargs)


class RadialMirrorScatter(FlatOpticalElement):
    inplanescattercol = 'inplanescatter'
    perpplanescattercol = 'perpplanescatter'

    def __init__(self, **kwargs):
        self.inplanescatter = _to_rad(kwargs.pop('inplanescatter'))
        self.perpplanescatter = _to_rad(kwargs.pop('perpplanescatter', 0.))
        super().__init__(**kwargs)


class FlatDetector(FlatOpticalElement):
    loc_coos_name = ['det_x', 'det_y']
    detpix_name = ['detpix_x', 'detpix_y']

    def __init__(self, pixsize=1, ignore_pixel_warning=False, **kwargs):
        self.pixsize = pixsize
        super().__init__(**kwargs)
        zoom = decompose44(self.pos4d)[2]
        self.npix = [0, 0]
        self.centerpix = [0, 0]
        for i in (0, 1):
            z = zoom[i + 1]
            self.npix[i] = int(np.round(2. * z / self.pixsize))
            if (np.abs(2. * z / self.pixsize - self.npix[i]) > 1e-2) and not ignore_pixel_warning:
                warnings.warn('Detector size is not an integer multiple of pixel size in '
                              'direction {0}. It will be rounded.'.format('xy'[i]),
                              SimulationSetupWarning)
            self.centerpix[i] = (self.npix[i] - 1) / 2


class CircularDetector(OpticalElement):
    loc_coos_name = ['det_phi', 'det_y']
    detpix_name = ['detpix_x', 'detpix_y']
    centerpix = [0, 0]
    default_geometry = Cylinder

    def __init__(self, pixsize=1, **kwargs):
        self.pixsize = pixsize
        super().__init__(**kwargs)


class FlatGrating(FlatOpticalElement):
    loc_coos_name = ['grat_y', 'grat_z']
    order_name = 'order'
    blaze_name = 'blaze'
    order_sign_kind = 'flat'   # sign = -1 (grating.py:145-172)

    def __init__(self, **kwargs):
        self.order_selector = kwargs.pop('order_selector')
        self.transmission = kwargs.pop('transmission', True)
        if 'd' not in kwargs:
            raise ValueError('Input parameter "d" (Grating constant) is required.')
        self._d = kwargs.pop('d')
        groove_angle = kwargs.pop('groove_angle', 0.)
        super().__init__(**kwargs)
        self.geometry._geometry['groove_angle'] = groove_angle


class CATGrating(FlatGrating):
    order_sign_kind = 'cat'    # sign = sign(p . d), 0 -> +1 (grating.py:291-301)


class NonParallelCATGrating(CATGrating):
    """CAT grating whose bar walls tilt linearly across the facet: blaze +=
    blaze_center + local y * d_blaze_mm (missions/mitsnl/catgrating.py:305-333)."""

    def __init__(self, **kwargs):
        self.d_blaze_mm = kwargs.pop('d_blaze_mm', 0)
        self.blaze_center = kwargs.pop('blaze_center', 0)
        super().__init__(**kwargs)


class QualityFactor(FlatOpticalElement):
    """probability *= exp(-(2 pi sigma / d)^2) ** (order^2) (catgrating.py:147-162);
    ``qualityfactor`` = {'d': ..., 'sigma': ...} in one length unit."""

    def __init__(self, qualityfactor=None, **kwargs):
        q = qualityfactor or {'d': 200., 'sigma': 1.75}
        self.factor = np.exp(- (2 * np.pi * q['sigma'] / q['d']) ** 2)
        super().__init__(**kwargs)


class L1(CATGrating):
    """L1 support of a CAT grating (catgrating.py:171-207): a CAT grating of
    period l1_dims['period'] (mm); a fraction 1 - openfraction of the photons
    hits the support bars instead, keeps its direction, gets order 0 and the
    transmission ``transmission`` = (energy keV, fraction) interpolated
    linearly (scipy interp1d, as the reference builds from its Si table)."""
    blaze_name = 'blaze_L1'
    order_name = 'order_L1'

    def __init__(self, l1_dims=None, transmission=None, **kwargs):
        from scipy.interpolate import interp1d
        dims = l1_dims or {'bardepth': 0.004, 'period': 0.005, 'barwidth': 0.0009}
        if not dims['barwidth'] < dims['period']:
            raise ValueError('Period of grating must be larger than bar width.')
        if transmission is None:
            raise ValueError('L1 needs the support transmission table (energy keV, fraction)')
        self.openfraction = 1 - dims['barwidth'] / dims['period']
        self.transfunc = interp1d(np.asarray(transmission[0], dtype=float),
                                  np.asarray(transmission[1], dtype=float))
        kwargs['d'] = dims['period']
        super().__init__(**kwargs)


class L2Abs(FlatOpticalElement):
    """L2 absorption and shadowing (catgrating.py:210-245): probability *=
    (inner/period)^2 - bardepth inner sin(angle) / (period^2 / 2 sqrt 3)."""

    def __init__(self, l2_dims=None, **kwargs):
        dims = l2_dims or {'bardepth': 0.5, 'period': 0.9622504, 'barwidth': 0.0962250}
        if not dims['barwidth'] < dims['period']:
            raise ValueError('Period of grating must be larger than bar width.')
        self.bardepth = dims['bardepth']
        self.period = dims['period']
        self.barwidth = dims['barwidth']
        super().__init__(**kwargs)
        self.innerfree = self.period - self.barwidth


class L2Diffraction(FlatOpticalElement):
    """Gaussian scatter by the L2 hexagons (catgrating.py:248-268): sigma =
    1.22 * 0.4 * arcsin(lambda / inner), a random direction around the ray
    (RandomGaussianScatter, optics/scatter.py:80-150)."""
    scattername = 'L2Diffraction'

    def __init__(self, l2_dims=None, **kwargs):
        dims = l2_dims or {'bardepth': 0.5, 'period': 0.9622504, 'barwidth': 0.0962250}
        self.innerfree = dims['period'] - dims['barwidth']
        super().__init__(**kwargs)


class FlatStack(FlatOpticalElement):
    """Several layers acting at one flat element (optics/base.py:218-281):
    ``elements`` classes, ``keywords`` their keyword dicts; every layer gets
    the stack's pose."""

    def __init__(self, **kwargs):
        elements = kwargs.pop('elements')
        keywords = kwargs.pop('keywords')
        super().__init__(**kwargs)
        self.elements = [elem(pos4d=self.pos4d, **k) for elem, k in zip(elements, keywords)]


# L1 diffraction orders of the 2018 Arcus gratings (catgrating.py:44-48)
L1_ORDER_SELECTOR = OrderSelector(
    np.array([-4, -3, -2, -1, 0, 1, 2, 3, 4]),
    p=np.array([0.006, 0.0135, 0.022, 0.028, 0.861, 0.028, 0.022, 0.0135, 0.006]))


class CATL1L2Stack(FlatStack):
    """CAT facet with its L1 and L2 supports (catgrating.py:336-377): layers
    NonParallelCATGrating, QualityFactor, L1 (grooves at pi/2 + groove_angle),
    L2Abs, L2Diffraction.  ``l1_transmission`` = (energy keV, fraction)."""

    def __init__(self, l1_dims=None, l2_dims=None, l1_order_selector=None, qualityfactor=None,
                 l1_transmission=None, **kwargs):
        if l1_order_selector is None:
            l1_order_selector = L1_ORDER_SELECTOR
        groove_angle = kwargs.pop('groove_angle', 0.)
        kwargs['elements'] = [NonParallelCATGrating, QualityFactor, L1, L2Abs, L2Diffraction]
        kwargs['keywords'] = [{'order_selector': kwargs.pop('order_selector'),
                               'd': kwargs.pop('d', 0.0002), 'groove_angle': groove_angle},
                              {'qualityfactor': qualityfactor},
                              {'l1_dims': l1_dims, 'order_selector': l1_order_selector,
                               'groove_angle': np.pi / 2. + groove_angle,
                               'transmission': l1_transmission},
                              {'l2_dims': l2_dims},
                              {'l2_dims': l2_dims}]
        super().__init__(**kwargs)


class BaseContainer(SimulationSequenceElement):
    elements = []

    def __init__(self, **kwargs):
        self.preprocess_steps = kwargs.pop('preprocess_steps', [])
        self.postprocess_steps = kwargs.pop('postprocess_steps', [])
        for elem in self.elements + self.preprocess_steps + self.postprocess_steps:
            if not callable(elem):
                from .simulator import SimulationSetupError
                raise SimulationSetupError('{0} is not callable.'.format(str(elem)))
        super().__init__(**kwargs)


__all__ = ['GeometryError', 'FinitePlane', 'Cylinder', 'OrderSelector', 'EfficiencyFile',
           'PerfectLens', 'RadialMirrorScatter', 'FlatDetector', 'CircularDetector',
           'FlatGrating', 'CATGrating', 'NonParallelCATGrating', 'QualityFactor', 'L1', 'L2Abs',
           'L2Diffraction', 'FlatStack', 'CATL1L2Stack', 'InterpolateEfficiencyTable']


def catsupportbars(photons):
    """Metal support of the CAT facets (missions/mitsnl/catgrating.py:314-324):
    photons that passed no facet (``facet`` < 0) are absorbed; without a
    ``facet`` column every photon is.  On the GPU it is a chain stage; this
    host function acts on a photon table directly."""
    if 'facet' in photons.colnames:
        prob = photons['probability']
        prob[np.asarray(photons['facet']) < 0] = 0.
    else:
        photons['probability'][...] = 0.
    return photons
