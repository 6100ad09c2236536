"""Lower a MARXS element tree to the GPU chain description (host, numpy).

Works on this package's element classes and on genuine MARXS objects
alike: elements are recognised by class name (anywhere in the MRO) and
read through the attributes MARXS itself uses (``geometry.pos4d``,
``order_selector``, ``_d``, ``focallength`` ...).  Frame vectors are derived
from ``pos4d`` with the same numpy expressions as Geometry.__getitem__
(marxs/math/geometry.py:108-160) so the kernels see identical inputs.

Unsupported elements raise ``NotImplementedError``: there is no CPU path.
"""
import math
import operator
from dataclasses import dataclass, field
from typing import Any, List, Optional

import numpy as np

from . import _abi


def classnames(obj):
    return {c.__name__ for c in type(obj).__mro__}


def _vec(pos4d, key):
    if key == 'center':
        return pos4d[:, 3]
    val = pos4d[:, {'x': 0, 'y': 1, 'z': 2}[key[-1]]]
    if key[:2] == 'e_':
        return val / np.linalg.norm(val)
    return val


def plane_frame(pos4d):
    """c, e_x, e_y, e_z, |v_y|, |v_z| as used by FinitePlane.intersect."""
    pos4d = np.asarray(pos4d, dtype=float)
    f = np.empty(14)
    f[0:3] = _vec(pos4d, 'center')[:3]
    f[3:6] = _vec(pos4d, 'e_x')[:3]
    f[6:9] = _vec(pos4d, 'e_y')[:3]
    f[9:12] = _vec(pos4d, 'e_z')[:3]
    f[12] = np.linalg.norm(_vec(pos4d, 'v_y'))
    f[13] = np.linalg.norm(_vec(pos4d, 'v_z'))
    return f


def _zoom(pos4d):
    c0, c1, c2 = np.array(pos4d[:3, :3]).T
    sx = np.sqrt(np.sum(c0 * c0))
    c0 = c0 / sx
    c1 = c1 - np.dot(c0, c1) * c0
    sy = np.sqrt(np.sum(c1 * c1))
    c1 = c1 / sy
    c2 = c2 - (np.dot(c0, c2) * c0 + np.dot(c1, c2) * c1)
    sz = np.sqrt(np.sum(c2 * c2))
    if np.linalg.det(np.array([c0, c1, c2 / sz]).T) < 0:
        sx = -sx
    return np.array([sx, sy, sz])


def cylinder_block(geometry):
    """pos4d rows, inverse rows, zoom_z, R, reduced phi borders (32 doubles)."""
    pos4d = np.asarray(geometry.pos4d, dtype=float)
    inv = np.linalg.inv(pos4d)
    z = _zoom(pos4d)
    twopi = 2 * np.pi
    lim = geometry.coos_limits[0]
    b = np.zeros(32)
    b[0:12] = pos4d[:3, :].ravel()
    b[12:24] = inv[:3, :].ravel()
    b[24] = z[2]
    b[25] = z[0]
    b[26] = (twopi + (lim[0] % twopi)) % twopi
    b[27] = (twopi + (lim[1] % twopi)) % twopi
    return b


@dataclass
class SelectorSpec:
    energy: np.ndarray
    cdf: np.ndarray           # (rows, orders)
    total: np.ndarray
    orders: np.ndarray        # int32
    by_energy: bool
    kind: int = 0             # _abi.SEL_CDF / SEL_SPLINE
    spline: Optional[tuple] = None   # SEL_SPLINE: (tx, ty, c[n_orders, ...])


def spline1_arrays(ip, what):
    """(tx, ty, coefficients) of a degree-1 scipy RectBivariateSpline."""
    if not (hasattr(ip, 'get_knots') and tuple(getattr(ip, 'degrees', ())) == (1, 1)):
        raise NotImplementedError('%s: only degree-1 RectBivariateSpline (kx = ky = 1) is '
                                  'supported on the GPU' % what)
    tx, ty = ip.get_knots()
    tx, ty = np.asarray(tx, dtype=float), np.asarray(ty, dtype=float)
    # the kernels index the interval below a knot and its coefficients:
    # at least two grid points (four knots) per axis, knots non-decreasing
    if len(tx) < 4 or len(ty) < 4 or np.any(np.diff(tx) < 0) or np.any(np.diff(ty) < 0):
        raise NotImplementedError('%s: a degree-1 spline needs at least two grid points per '
                                  'axis and sorted knots' % what)
    c = np.asarray(ip.get_coeffs(), dtype=float)
    if c.size != (len(tx) - 2) * (len(ty) - 2):
        raise NotImplementedError('%s: unexpected spline coefficient layout' % what)
    return tx, ty, c


def lens_spline(lens):
    """Reflectivity spline of a PerfectLens, or None for the default
    (probability unchanged, optics/mirror.py:45-48)."""
    interp = getattr(lens, 'reflectivity_interpolator', None)
    if interp is None:
        return None
    if getattr(interp, '__name__', '') == '<lambda>' and \
            'marxs' in getattr(interp, '__module__', ''):
        return None
    tx, ty, c = spline1_arrays(interp, 'PerfectLens reflectivity_interpolator')
    return tx, ty, c[None, :]


def lower_selector(sel):
    """Tables of an order selector, computed with the reference's numpy ops;
    checked so the kernels never index an empty table."""
    spec = _lower_selector(sel)
    n_rows, n_orders = spec.cdf.shape
    if n_rows < 1 or n_orders < 1 or len(spec.orders) != n_orders or len(spec.total) != n_rows:
        raise ValueError('order selector %s: needs at least one order and one row, and '
                         'matching table shapes' % type(sel).__name__)
    if spec.by_energy and len(spec.energy) != n_rows:
        raise ValueError('order selector %s: %d energies for %d table rows'
                         % (type(sel).__name__, len(spec.energy), n_rows))
    return spec


def _lower_selector(sel):
    names = classnames(sel)
    if hasattr(sel, 'interpolators') and hasattr(sel, 'orders'):
        # InterpolateEfficiencyTable (missions/mitsnl/catgrating.py:63-144)
        tx = ty = None
        cs = []
        for ip in sel.interpolators:
            kx, ky, c = spline1_arrays(ip, 'InterpolateEfficiencyTable')
            if tx is None:
                tx, ty = kx, ky
            elif not (np.array_equal(tx, kx) and np.array_equal(ty, ky)):
                raise NotImplementedError('InterpolateEfficiencyTable: orders on different grids')
            cs.append(c)
        n = len(cs)
        return SelectorSpec(energy=np.zeros(1), cdf=np.zeros((1, n)), total=np.zeros(1),
                            orders=np.asarray(sel.orders).astype(np.int32), by_energy=False,
                            kind=_abi.SEL_SPLINE, spline=(tx, ty, np.stack(cs)))
    if 'EfficiencyFile' in names:
        return SelectorSpec(energy=np.asarray(sel.energy, dtype=float),
                            cdf=np.ascontiguousarray(sel.cumprob, dtype=float),
                            total=np.asarray(sel.totalprob, dtype=float),
                            orders=np.asarray(sel.orders).astype(np.int32), by_energy=True)
    if 'OrderSelector' in names:
        if len(sel.p) == 0 or len(sel.orderlist) != len(sel.p):
            raise ValueError('OrderSelector: needs at least one order, one probability each')
        p_sum = sel.p.sum()
        p = sel.p / p_sum
        cdf = p.cumsum()
        cdf /= cdf[-1]
        return SelectorSpec(energy=np.zeros(1), cdf=cdf[None, :].copy(),
                            total=np.array([p_sum], dtype=float),
                            orders=np.asarray(sel.orderlist).astype(np.int32), by_energy=False)
    raise NotImplementedError('order selector %s is not supported on the GPU' % type(sel).__name__)


@dataclass
class StageSpec:
    kind: int
    element: Any
    frame: np.ndarray = field(default_factory=lambda: np.zeros(14))
    cyl: np.ndarray = field(default_factory=lambda: np.zeros(32))
    p: np.ndarray = field(default_factory=lambda: np.zeros(8))
    id_num: int = -9
    out_names: List[Optional[str]] = field(default_factory=lambda: [None] * 4)
    id_col: Optional[str] = None
    new_col_order: List[str] = field(default_factory=list)
    draw_names: List[str] = field(default_factory=list)
    facets: Optional[np.ndarray] = None
    selectors: List[SelectorSpec] = field(default_factory=list)
    grid: Optional[dict] = None
    spline: Optional[tuple] = None   # LENS reflectivity (tx, ty, c[1, ...])
    stack: Optional[dict] = None     # GRATINGS of CATL1L2Stack facets: layer constants
    reads: Optional[str] = None      # SUPPORT: the id column it reads
    facet_cyl: Optional[np.ndarray] = None   # GRATINGS on Cylinder surfaces: (F, 34)
    host_eval: Optional[dict] = None # GRATINGS: facets with callable d / blaze modifier


def _interp_table(x, y):
    """(x, y) of an np.interp table: at least one point, x increasing."""
    x, y = np.asarray(x, dtype=float), np.asarray(y, dtype=float)
    if x.ndim != 1 or len(x) < 1 or x.shape != y.shape or np.any(np.diff(x) < 0):
        raise ValueError('interpolation table: needs at least one point, matching x and y, '
                         'and increasing x')
    return x, y


def _loc_names(elem):
    names = getattr(elem, 'loc_coos_name', None)
    return [None, None] if names is None else list(names)


def _norms(v):
    """Euclidean norms of the rows of v (F, 4)."""
    return np.sqrt(np.einsum('ij,ij->i', v, v))


def default_blaze_modifier(g):
    """True when ``g.blaze_angle_modifier`` is FlatGrating's own (zero,
    optics/grating.py:222-231): the class that defines it, found along the
    MRO, is FlatGrating, and the instance does not override it."""
    if 'blaze_angle_modifier' in getattr(g, '__dict__', {}):
        return False
    for klass in type(g).__mro__:
        if 'blaze_angle_modifier' in vars(klass):
            return klass.__name__ == 'FlatGrating'
    return True


def _plane_frames(elems, out):
    """Frames of flat elements into a facet table (vectorised over the
    elements): centre, unit e_x/e_y/e_z and half sizes as
    Geometry.__getitem__ derives them (math/geometry.py:108-160), and the id
    numbers.  Returns the homogeneous e_y, e_z (F, 4)."""
    P = np.stack([np.asarray(g.geometry.pos4d, dtype=float) for g in elems])   # (F, 4, 4)
    vx, vy, vz = P[:, :, 0], P[:, :, 1], P[:, :, 2]
    nx, ny, nz = _norms(vx), _norms(vy), _norms(vz)
    ex4, ey4, ez4 = vx / nx[:, None], vy / ny[:, None], vz / nz[:, None]
    out['c'] = P[:, :3, 3]
    out['ex'] = ex4[:, :3]
    out['ey'] = ey4[:, :3]
    out['ez'] = ez4[:, :3]
    out['hy'] = ny
    out['hz'] = nz
    out['id_num'] = [int(g.id_num) for g in elems]
    return ey4, ez4


def host_evaluated(gratings):
    """The facets whose grating constant or blaze modifier depends on the
    position on the facet through a Python callable: FlatGrating.d with a
    callable _d (optics/grating.py:209-220, e.g. the chirped facets of
    design/bendgratings.py:180-192) and an overridden blaze_angle_modifier
    (grating.py:222-231).  Returns ({facet index: grating} for d, the same
    for the blaze modifier)."""
    d = {i: g for i, g in enumerate(gratings) if callable(g._d)}
    blaze = {i: g for i, g in enumerate(gratings)
             if not default_blaze_modifier(g) and not hasattr(g, 'd_blaze_mm')}
    return d, blaze


def cylinder_facets(gratings, facets):
    """Gratings on Cylinder surfaces (the bent facets of
    design/bendgratings.py:24-60): per facet the cylinder block of
    Cylinder.intersect (math/geometry.py:470-564) and sin, cos of the
    negative groove angle; the facet table's frame is replaced by each
    patch's tangent plane at the middle of its phi range, half sizes the
    arc half length plus the sag and the z half length, so the candidate
    grid bounds the curved patch (the kernel intersects the cylinder)."""
    out = np.zeros((len(gratings), _abi.FACET_CYL))
    for i, g in enumerate(gratings):
        geo = g.geometry
        blk = cylinder_block(geo)
        out[i, :32] = blk
        groove = float(geo._geometry.get('groove_angle', 0.))
        out[i, 32] = math.sin(-groove)
        out[i, 33] = math.cos(-groove)
        pos4d = np.asarray(geo.pos4d, dtype=float)
        R, zz = blk[25], blk[24]
        e1 = pos4d[:3, 0] / np.linalg.norm(pos4d[:3, 0])
        e2 = pos4d[:3, 1] / np.linalg.norm(pos4d[:3, 1])
        lim = np.asarray(geo.coos_limits[0], dtype=float)
        half = 0.5 * float(lim[1] - lim[0])
        if not (0 < half < np.pi / 2):
            raise NotImplementedError('cylindrical gratings spanning more than 180 degrees')
        pm = 0.5 * float(lim[0] + lim[1])
        radial = np.cos(pm) * e1 + np.sin(pm) * e2
        facets['c'][i] = pos4d[:3, 3] + R * radial
        facets['ex'][i] = radial
        facets['ey'][i] = -np.sin(pm) * e1 + np.cos(pm) * e2
        facets['hy'][i] = R * half + R * (1 - np.cos(half))
        facets['hz'][i] = zz
    return out


def _grating_facets(gratings, selectors, sel_index):
    """Facet table of a list of gratings (vectorised over the facets): the
    frame of Geometry.__getitem__ (math/geometry.py:108-160) and the groove
    frame of FlatGrating.e_groove_coos (optics/grating.py:186-207)."""
    n = len(gratings)
    out = np.zeros(n, dtype=_abi.FACET_DTYPE)
    ey4, ez4 = _plane_frames(gratings, out)
    # FlatGrating.e_groove_coos on the flat bases (e_y, e_z, e_x): math.sin /
    # math.cos of each distinct groove angle, as the reference evaluates them
    groove = np.array([float(g.geometry._geometry.get('groove_angle', 0.)) for g in gratings])
    sn = np.empty(n)
    cs = np.empty(n)
    for gv in np.unique(groove):
        k = groove == gv
        sn[k] = math.sin(-gv)
        cs[k] = math.cos(-gv)
    e_groove = sn[:, None] * ey4 + cs[:, None] * ez4
    e_perp = cs[:, None] * ey4 - sn[:, None] * ez4
    out['l'] = e_groove[:, :3]
    out['dneg'] = (-e_perp)[:, :3]
    # a callable grating constant is evaluated per photon (host_evaluated)
    out['dgrat'] = [float('nan') if callable(g._d) else float(g._d) for g in gratings]
    sel = np.empty(n, dtype=np.int32)
    for i, g in enumerate(gratings):
        key = id(g.order_selector)
        if key not in sel_index:
            sel_index[key] = len(selectors)
            selectors.append(lower_selector(g.order_selector))
        sel[i] = sel_index[key]
    out['selector'] = sel
    out['cat'] = [1 if 'CATGrating' in classnames(g) else 0 for g in gratings]
    out['transmission'] = [1 if g.transmission else 0 for g in gratings]
    return out


def grid_params(facets, slope_max=0.1, margin=0.05, cells_per_facet=24.0, max_cells=1 << 20):
    """Mean plane, depth model, extents and cell size of the candidate grid
    for a facet table.

    The host computes each facet's grown footprint the same way the device
    builder does; the extents cover all of them (with a 1 mm pad) and the
    capacity bounds the total number of (cell, facet) entries.  Cells are
    1/cells_per_facet of a facet edge (24 measured fastest on the CAT array
    with the depth model, ~1 % ahead of 16 and 32; 2 gives ~3.6 candidates
    per cell on a tiled array), coarsened if the grid would exceed
    ``max_cells``.
    """
    g = _grid_params(facets, slope_max, margin, cells_per_facet)
    while g['nu'] * g['nv'] > max_cells and cells_per_facet > 1.0:
        cells_per_facet = max(1.0, cells_per_facet * 0.9 * (max_cells / (g['nu'] * g['nv'])) ** 0.5)
        g = _grid_params(facets, slope_max, margin, cells_per_facet)
    return g


def depth_model(c, o, n, a, b):
    """Least-squares quadric D(u, v) = d0 + d1 u + d2 v + d3 u^2 + d4 u v +
    d5 v^2 of the facet centres' depth (c - o).n over the grid plane (zero
    for fewer than six facets)."""
    rel = np.asarray(c, dtype=float) - o
    u, v, h = rel @ a, rel @ b, rel @ n
    if len(u) < 6:
        return np.zeros(6)
    A = np.stack([np.ones_like(u), u, v, u * u, u * v, v * v], axis=1)
    coef, *_ = np.linalg.lstsq(A, h, rcond=None)
    return coef


def depth_at(d, u, v):
    """The depth model D(u, v)."""
    return d[0] + u * (d[1] + d[3] * u + d[4] * v) + v * (d[2] + d[5] * v)


def depth_lipschitz(d, umin, umax, vmin, vmax):
    """max |dD/du| + |dD/dv| over a box (both partials are linear in (u, v),
    so the maximum sits at a corner)."""
    best = 0.0
    for u in (umin, umax):
        for v in (vmin, vmax):
            best = max(best, abs(d[1] + 2 * d[3] * u + d[4] * v) + abs(d[2] + d[4] * u + 2 * d[5] * v))
    return best


def facet_depth_deviation(facets, o, n, a, b, d):
    """Per facet max over its rectangle of |depth - D(u, v)|: a quadratic in
    the rectangle's coordinates (s, t) in [-1, 1]^2, whose largest magnitude
    is at a corner, at an edge's stationary point or at the interior one
    (the builder on the device evaluates the same candidates)."""
    c, ey, ez = facets['c'], facets['ey'], facets['ez']
    hy, hz = facets['hy'][:, None], facets['hz'][:, None]

    def q(s, t):
        p = c + (s * hy) * ey + (t * hz) * ez - o
        return p @ n - depth_at(d, p @ a, p @ b)
    q0 = q(0., 0.)
    qp0, qm0, q0p, q0m = q(1., 0.), q(-1., 0.), q(0., 1.), q(0., -1.)
    qs, qt = (qp0 - qm0) / 2, (q0p - q0m) / 2
    qss, qtt = (qp0 + qm0) / 2 - q0, (q0p + q0m) / 2 - q0
    qst = (q(1., 1.) - q(1., -1.) - q(-1., 1.) + q(-1., -1.)) / 4

    def Q(s, t):
        return q0 + qs * s + qt * t + qss * s * s + qst * s * t + qtt * t * t
    best = np.zeros(len(c))
    for s_ in (-1., 1.):
        for t_ in (-1., 1.):
            best = np.maximum(best, np.abs(Q(s_, t_)))
    with np.errstate(divide='ignore', invalid='ignore'):
        for e in (-1., 1.):
            ts = -(qt + e * qst) / (2 * qtt)            # edges s = e
            ok = np.isfinite(ts) & (np.abs(ts) < 1)
            best = np.where(ok, np.maximum(best, np.abs(Q(e, np.where(ok, ts, 0.)))), best)
            ss = -(qs + e * qst) / (2 * qss)            # edges t = e
            ok = np.isfinite(ss) & (np.abs(ss) < 1)
            best = np.where(ok, np.maximum(best, np.abs(Q(np.where(ok, ss, 0.), e))), best)
        det = 4 * qss * qtt - qst * qst
        si = (-2 * qtt * qs + qst * qt) / det
        ti = (-2 * qss * qt + qst * qs) / det
        ok = np.isfinite(si) & np.isfinite(ti) & (np.abs(si) < 1) & (np.abs(ti) < 1)
        best = np.where(ok, np.maximum(best, np.abs(Q(np.where(ok, si, 0.), np.where(ok, ti, 0.)))),
                        best)
    return best


def _grid_params(facets, slope_max, margin, cells_per_facet):
    F = len(facets)
    c = facets['c']
    nrm = facets['ex'].mean(axis=0)
    nrm /= np.linalg.norm(nrm)
    ay = facets['ey'].mean(axis=0)
    a = ay - np.dot(ay, nrm) * nrm
    a /= np.linalg.norm(a)
    b = np.cross(nrm, a)
    o = c.mean(axis=0)
    size = 2 * max(facets['hy'].max(), facets['hz'].max())
    cell = size / cells_per_facet
    corners = []
    for sy in (-1, 1):
        for sz in (-1, 1):
            corners.append(c + (sy * facets['hy'])[:, None] * facets['ey'] +
                           (sz * facets['hz'])[:, None] * facets['ez'])
    corners = np.stack(corners, axis=1) - o           # (F, 4, 3)
    u = corners @ a
    v = corners @ b
    dep = np.abs(corners @ nrm).max(axis=1)
    # depth model of the facet surface: a ray is looked up where it meets
    # the model, so a facet's footprint grows by its deviation from the
    # model plus the model's change over the ray's drift, not by its depth
    d = depth_model(c, o, nrm, a, b)
    # L over the facets' area plus the rays' drift and 50 mm for facets that
    # move after the fit (tolerancing rebuilds the grid on the device)
    pad = slope_max * dep.max() + 50.0
    lip = depth_lipschitz(d, u.min() - pad, u.max() + pad, v.min() - pad, v.max() + pad)
    dev = facet_depth_deviation(facets, o, nrm, a, b, d)
    grow_model = slope_max * (dev + lip * slope_max * dep) + margin
    grow_plane = dep * slope_max + margin
    if not np.max(grow_model) < np.max(grow_plane):
        d, lip = np.zeros(6), 0.0                     # the model does not pay: the plane
    grow = slope_max * (facet_depth_deviation(facets, o, nrm, a, b, d) + lip * slope_max * dep) + margin
    umin, umax = u.min(axis=1) - grow, u.max(axis=1) + grow
    vmin, vmax = v.min(axis=1) - grow, v.max(axis=1) + grow
    u0 = umin.min() - 1.0
    v0 = vmin.min() - 1.0
    nu = int(np.floor((umax.max() + 1.0 - u0) / cell)) + 1
    nv = int(np.floor((vmax.max() + 1.0 - v0) / cell)) + 1
    # host estimate of the entries, with one spare row/column per facet
    iu0 = np.floor((umin - 1e-6 - u0) / cell)
    iu1 = np.floor((umax + 1e-6 - u0) / cell)
    iv0 = np.floor((vmin - 1e-6 - v0) / cell)
    iv1 = np.floor((vmax + 1e-6 - v0) / cell)
    capacity = int(np.sum((iu1 - iu0 + 2) * (iv1 - iv0 + 2))) + 16
    return dict(o=o, n=nrm, a=a, b=b, u0=u0, v0=v0, cell=cell, nu=nu, nv=nv,
                slope_max=slope_max, margin=margin, capacity=capacity, n_facets=F,
                depth=np.asarray(d, dtype=float), depth_lip=float(lip))


# element attributes the lowering reads, so a change makes a chain lower
# again (the geometry's pos4d is watched separately)
WATCHED_ATTRS = ('order_selector', 'focallength', 'inplanescatter', 'perpplanescatter',
                 'pixsize', 'centerpix', '_d', 'd_center_optax', 'transmission', 'id_num',
                 'id_col', 'reflectivity_interpolator', 'order_name', 'blaze_name',
                 'detpix_name', 'inplanescattercol', 'perpplanescattercol', 'scattername',
                 'blaze_center', 'd_blaze_mm', 'factor', 'openfraction', 'bardepth', 'period',
                 'innerfree')


def _same(a, b):
    if a is b:
        return True
    if isinstance(a, np.ndarray) or isinstance(b, np.ndarray):
        return (isinstance(a, np.ndarray) and isinstance(b, np.ndarray) and a.shape == b.shape
                and bool(np.array_equal(a, b)))
    try:
        return bool(a == b)
    except Exception:
        return False


def _snapshot(v):
    return np.array(v, copy=True) if isinstance(v, np.ndarray) else v


def _inner_arrays(obj, depth=2):
    """The ndarrays an object holds (in its ``__dict__``, in lists and tuples
    there, and in the objects it holds, ``depth`` levels down): the tables of
    an order selector or an interpolator (a scipy spline keeps its knots and
    coefficients in ``tck``)."""
    out, seen = [], set()

    def visit(o, d):
        if id(o) in seen:
            return
        seen.add(id(o))
        if isinstance(o, np.ndarray):
            out.append(o)
        elif isinstance(o, (list, tuple)):
            for x in o:
                visit(x, d)
        elif d > 0 and isinstance(getattr(o, '__dict__', None), dict):
            for v in vars(o).values():
                visit(v, d - 1)
    visit(obj, depth)
    return out


class ChangeWatch:
    """What a lowered chain was built from, for a cheap check on every call.

    MARXS users move elements by assigning or editing ``geometry.pos4d`` in
    place (design/tolerancing.py:133) and swap order selectors on facets
    (analysis/gratings.py:117-124), so every call must notice such changes.
    The element tree is walked once; a call then compares the containers'
    element lists and the geometry objects by identity, all pos4d matrices
    (assigned or edited in place) as one stacked array, and the watched
    attributes by identity (by value where the identity changed, and always
    for array values).  Objects held in watched attributes (order selectors,
    interpolators) are also compared by the values of the tables they hold,
    so a selector's probability table edited in place is noticed too.
    """

    def __init__(self, elements):
        self.top = tuple(elements)
        containers, holders, geoms = [], [], []
        objs = {name: [] for name in WATCHED_ATTRS}

        def walk(e):
            g = getattr(e, 'geometry', None)
            if g is not None and hasattr(g, 'pos4d'):
                holders.append(e)
                geoms.append(g)
            for name in WATCHED_ATTRS:
                if hasattr(e, name):
                    objs[name].append(e)
            sub = getattr(e, 'elements', None)
            if sub:
                containers.append((e, tuple(sub)))
                for x in sub:
                    walk(x)
        for e in elements:
            walk(e)
        self.containers = containers
        self.holders = holders
        self.geoms = geoms
        self.geom_ids = [id(g) for g in geoms]
        self.pos = self._stack(list(map(_POS4D, geoms)))
        self.attrs = []
        for name, ol in objs.items():
            if not ol:
                continue
            vals = list(map(operator.attrgetter(name), ol))
            arrays = [k for k, v in enumerate(vals) if isinstance(v, np.ndarray)]
            self.attrs.append((operator.attrgetter(name), ol, [id(v) for v in vals],
                               [_snapshot(v) for v in vals], arrays))
        # tables inside the distinct objects held by watched attributes
        held = {}
        for _, ol, _, snaps, _ in self.attrs:
            for v in snaps:
                if not isinstance(v, (np.ndarray, str, bytes, int, float, bool, type(None))) and \
                        isinstance(getattr(v, '__dict__', None), dict):
                    held[id(v)] = v
        self.held = [(o, [np.array(a, copy=True) for a in _inner_arrays(o)])
                     for o in held.values()]

    @staticmethod
    def _stack(mats):
        if not mats:
            return np.zeros((0, 4, 4))
        try:
            return np.array(mats, dtype=float)
        except ValueError:
            return np.array([np.asarray(m, dtype=float) for m in mats])

    def changed(self, elements):
        """True when ``elements`` no longer match what was watched."""
        if tuple(elements) != self.top:
            return True
        for c, snap in self.containers:
            if tuple(getattr(c, 'elements', ()) or ()) != snap:
                return True
        if list(map(id, map(_GEOMETRY, self.holders))) != self.geom_ids:
            return True
        stacked = self._stack(list(map(_POS4D, self.geoms)))
        if stacked.shape != self.pos.shape or not np.array_equal(stacked, self.pos):
            return True
        for get, ol, ids, snaps, arrays in self.attrs:
            vals = list(map(get, ol))
            if list(map(id, vals)) != ids:
                for v, i0, s0 in zip(vals, ids, snaps):
                    if id(v) != i0 and not _same(v, s0):
                        return True
            for k in arrays:
                if not _same(vals[k], snaps[k]):
                    return True
        for o, tables in self.held:
            now = _inner_arrays(o)
            if len(now) != len(tables) or not all(map(_same, now, tables)):
                return True
        return False


_POS4D = operator.attrgetter('pos4d')
_GEOMETRY = operator.attrgetter('geometry')


def lower_elements(elements):
    """Flatten a chain into StageSpecs (depth-first through containers)."""
    stages = []
    for e in elements:
        stages.extend(_lower_one(e))
    if len(stages) > _abi.MAX_STAGES:
        raise NotImplementedError('chains of more than %d stages' % _abi.MAX_STAGES)
    return stages


def _grating_stage(owner, gratings, id_col):
    first = gratings[0]
    for g in gratings:
        if not ({'FlatGrating', 'CATGrating'} & classnames(g)):
            raise NotImplementedError('a Parallel mixing %s with gratings' % type(g).__name__)
    selectors, sel_index = [], {}
    facets = _grating_facets(gratings, selectors, sel_index)
    loc = _loc_names(first)
    order_name = getattr(first, 'order_name', 'order')
    blaze_name = getattr(first, 'blaze_name', 'blaze')
    st = StageSpec(kind=_abi.STAGE_GRATINGS, element=owner,
                   out_names=[loc[0], loc[1], order_name, blaze_name], id_col=id_col,
                   draw_names=['order_u'], facets=facets, selectors=selectors)
    st.new_col_order = [order_name, blaze_name] + ([id_col] if id_col else []) + \
        [n for n in loc if n is not None]
    if len(gratings) > 1:
        st.grid = grid_params(facets)
    on_cyl = ['Cylinder' in classnames(g.geometry) for g in gratings]
    if any(on_cyl):
        if not all(on_cyl):
            raise NotImplementedError('a Parallel mixing flat and cylindrical gratings')
        st.facet_cyl = cylinder_facets(gratings, facets)
        if st.grid is not None:
            st.grid = grid_params(facets)
    hd, hb = host_evaluated(gratings)
    if hd or hb:
        # the callables take the photons' local coordinates, which the stage
        # writes to its loc columns; facets are told apart by id number
        if loc[0] is None or loc[1] is None:
            raise NotImplementedError('a position-dependent grating needs its local '
                                      'coordinate columns (loc_coos_name)')
        if len(gratings) > 1 and (id_col is None or
                                  len(set(facets['id_num'].tolist())) != len(gratings)):
            raise NotImplementedError('position-dependent facets need an id column with a '
                                      'distinct id number per facet')
        st.host_eval = {'d': hd, 'blaze': hb}
    return st


def _detector_array_stage(owner, dets, id_col):
    """Stage for a Parallel of FlatDetectors, a CCD array
    (simulator/tests/test_parallel.py:11-23; the cameras of
    missions/arcus/arcus.py:342-360): the element table of the grating stages
    with each element's pixel size and centre pixel (FlatDetector,
    optics/detector.py:18-75) in place of the groove constants."""
    first = dets[0]
    loc = _loc_names(first)
    dp = list(getattr(first, 'detpix_name', ['detpix_x', 'detpix_y']))
    for d in dets:
        if 'FlatDetector' not in classnames(d):
            raise NotImplementedError('a Parallel mixing %s with FlatDetectors' % type(d).__name__)
        if _loc_names(d) != loc or list(getattr(d, 'detpix_name', dp)) != dp:
            raise NotImplementedError('a Parallel of FlatDetectors with different column names')
    facets = np.zeros(len(dets), dtype=_abi.FACET_DTYPE)
    _plane_frames(dets, facets)
    facets['dgrat'] = [float(d.pixsize) for d in dets]
    facets['l'][:, 0] = [float(d.centerpix[0]) for d in dets]
    facets['l'][:, 1] = [float(d.centerpix[1]) for d in dets]
    facets['selector'] = -1
    st = StageSpec(kind=_abi.STAGE_DETARRAY, element=owner,
                   out_names=[loc[0], loc[1], dp[0], dp[1]], id_col=id_col, facets=facets)
    st.new_col_order = dp + ([id_col] if id_col else []) + [n for n in loc if n is not None]
    if len(dets) > 1:
        st.grid = grid_params(facets)
    return st


def _is_detector(e):
    return 'FlatDetector' in classnames(e)


_STACK_LAYERS = ('CATGrating', 'QualityFactor', 'L1', 'L2Abs', 'L2Diffraction')


def _is_cat_stack(e):
    layers = getattr(e, 'elements', None)
    return ('FlatStack' in classnames(e) and layers is not None and len(layers) == 5 and
            all(name in classnames(layer) for name, layer in zip(_STACK_LAYERS, layers)))


def _value(q):
    return float(np.asarray(q, dtype=float))


def _cat_stack_stage(owner, stacks, id_col):
    """Facet-array stage for a Parallel of CATL1L2Stack facets
    (missions/mitsnl/catgrating.py:336-377)."""
    membranes = [st.elements[0] for st in stacks]
    st = _grating_stage(owner, membranes, id_col)
    if st.facet_cyl is not None or st.host_eval:
        raise NotImplementedError('CATL1L2Stack facets on Cylinder surfaces or with '
                                  'position-dependent membranes')
    st.facets['id_num'] = [int(x.id_num) for x in stacks]
    l1s = [x.elements[2] for x in stacks]
    # one L1 order table for all facets (their selectors must agree)
    spec0 = lower_selector(l1s[0].order_selector)
    for x in l1s[1:]:
        if x.order_selector is not l1s[0].order_selector:
            sp = lower_selector(x.order_selector)
            if not (np.array_equal(sp.cdf, spec0.cdf) and np.array_equal(sp.total, spec0.total)
                    and np.array_equal(sp.orders, spec0.orders)):
                raise NotImplementedError('CATL1L2Stack facets with different L1 order selectors')
    st.selectors.append(spec0)
    l1tab = _grating_facets(l1s, st.selectors,
                            {id(x.order_selector): len(st.selectors) - 1 for x in l1s})
    m0, qf, l1, l2abs, l2diff = stacks[0].elements

    def shared(get, what):
        v0 = get(stacks[0])
        for x in stacks[1:]:
            if not np.array_equal(np.asarray(get(x), dtype=float), np.asarray(v0, dtype=float)):
                raise NotImplementedError('CATL1L2Stack facets with different %s' % what)
        return v0
    shared(lambda x: [_value(getattr(x.elements[0], 'blaze_center', 0.)),
                      _value(getattr(x.elements[0], 'd_blaze_mm', 0.))], 'blaze modifiers')
    shared(lambda x: _value(x.elements[1].factor), 'quality factors')
    shared(lambda x: [_value(x.elements[2].openfraction), _value(x.elements[2]._d)], 'L1 support')
    shared(lambda x: np.r_[np.asarray(x.elements[2].transfunc.x, dtype=float),
                           np.asarray(x.elements[2].transfunc.y, dtype=float)], 'L1 transmission')
    shared(lambda x: [_value(x.elements[3].bardepth), _value(x.elements[3].period),
                      _value(x.elements[3].innerfree), _value(x.elements[4].innerfree)], 'L2 support')
    if len(set(l1tab['selector'])) != 1 or not np.all(l1tab['cat'] == 1) or \
            not np.all(l1tab['transmission'] == 1):
        raise NotImplementedError('CATL1L2Stack: L1 layers must share one order selector')
    inner, period = _value(l2abs.innerfree), _value(l2abs.period)
    st.stack = dict(
        blaze_center=_value(getattr(m0, 'blaze_center', 0.)),
        d_blaze_mm=_value(getattr(m0, 'd_blaze_mm', 0.)),
        qf=_value(qf.factor), l1_open=_value(l1.openfraction), l1_d=float(l1tab['dgrat'][0]),
        l1_vec=np.ascontiguousarray(np.concatenate([l1tab['l'], l1tab['dneg']], axis=1)),
        l1_selector=int(l1tab['selector'][0]),
        l1_trans_e=_interp_table(l1.transfunc.x, l1.transfunc.y)[0],
        l1_trans_t=_interp_table(l1.transfunc.x, l1.transfunc.y)[1],
        l2_open=(inner / period) ** 2, l2_shadow=_value(l2abs.bardepth) * inner,
        l2_total=period ** 2 / 2 * np.sqrt(3), l2_inner=_value(l2diff.innerfree))
    loc_stack = _loc_names(stacks[0])
    loc = _loc_names(m0)
    st.out_names = [loc[0], loc[1], getattr(m0, 'order_name', 'order'),
                    getattr(m0, 'blaze_name', 'blaze'), loc_stack[0], loc_stack[1],
                    getattr(l1, 'order_name', 'order_L1'), getattr(l1, 'blaze_name', 'blaze_L1'),
                    getattr(l2diff, 'scattername', 'L2Diffraction')]
    st.new_col_order = [c for c in ([id_col] + loc_stack + st.out_names[2:4] + loc +
                                    st.out_names[6:9]) if c is not None]
    st.draw_names = ['order_u', 'l1_order_u', 'l1_support_u', 'l2_normal', 'l2_phi_u']
    return st


def is_support_bars(e):
    """catsupportbars (missions/mitsnl/catgrating.py:314-324), the reference's
    function or this package's."""
    return callable(e) and getattr(e, '__name__', None) == 'catsupportbars' and \
        not hasattr(e, 'geometry')


def _lower_one(e):
    if is_support_bars(e):
        return [StageSpec(kind=_abi.STAGE_SUPPORT, element=e, reads='facet')]
    names = classnames(e)
    if 'Parallel' in names:
        id_col = None
        if e.elements:
            id_col = getattr(e.elements[0], 'id_col', None)
        if not e.elements:
            return []
        if all(_is_cat_stack(x) for x in e.elements):
            return [_cat_stack_stage(e, list(e.elements), id_col)]
        if _is_detector(e.elements[0]):
            return [_detector_array_stage(e, list(e.elements), id_col)]
        return [_grating_stage(e, list(e.elements), id_col)]
    if 'FlatGrating' in names:
        return [_grating_stage(e, [e], getattr(e, 'id_col', None))]
    if hasattr(e, 'elements') and ({'Sequence', 'BaseContainer'} & names):
        out = []
        for sub in e.elements:
            out.extend(_lower_one(sub))
        return out
    if 'PerfectLens' in names:
        loc = _loc_names(e)
        st = StageSpec(kind=_abi.STAGE_LENS, element=e, frame=plane_frame(e.geometry.pos4d),
                       out_names=[loc[0], loc[1], None, None], spline=lens_spline(e))
        st.p[0] = float(e.focallength)
        st.p[1] = float(getattr(e, 'd_center_optax', 0.))
        st.new_col_order = [n for n in loc if n is not None]
        return [_with_id(st, e)]
    if 'RadialMirrorScatter' in names:
        loc = _loc_names(e)
        ic = getattr(e, 'inplanescattercol', 'inplanescatter')
        pc = getattr(e, 'perpplanescattercol', 'perpplanescatter')
        st = StageSpec(kind=_abi.STAGE_SCATTER, element=e, frame=plane_frame(e.geometry.pos4d),
                       out_names=[loc[0], loc[1], ic, pc],
                       draw_names=['inplanescatter', 'perpplanescatter'])
        st.p[0] = float(e.inplanescatter)
        st.p[1] = float(e.perpplanescatter)
        st.new_col_order = [ic, pc] + [n for n in loc if n is not None]
        return [_with_id(st, e)]
    if 'FlatDetector' in names:
        loc = _loc_names(e)
        dp = list(getattr(e, 'detpix_name', ['detpix_x', 'detpix_y']))
        st = StageSpec(kind=_abi.STAGE_FLATDET, element=e, frame=plane_frame(e.geometry.pos4d),
                       out_names=[loc[0], loc[1], dp[0], dp[1]])
        st.p[0] = float(e.pixsize)
        st.p[1] = float(e.centerpix[0])
        st.p[2] = float(e.centerpix[1])
        st.new_col_order = dp + [n for n in loc if n is not None]
        return [_with_id(st, e)]
    if 'CircularDetector' in names:
        loc = _loc_names(e)
        dp = list(getattr(e, 'detpix_name', ['detpix_x', 'detpix_y']))
        st = StageSpec(kind=_abi.STAGE_CYLDET, element=e, cyl=cylinder_block(e.geometry),
                       out_names=[loc[0], loc[1], dp[0], dp[1]])
        st.p[0] = float(e.pixsize)
        st.p[1] = float(e.centerpix[0])
        st.p[2] = float(e.centerpix[1])
        st.new_col_order = dp + [n for n in loc if n is not None]
        return [_with_id(st, e)]
    raise NotImplementedError('element %s is not supported by the GPU backend' % type(e).__name__)


def _with_id(st, e):
    idc = getattr(e, 'id_col', None)
    if idc is not None:
        st.id_col = idc
        st.id_num = int(getattr(e, 'id_num', -9))
        # the id column is created right after the element's output columns
        n_extra = {_abi.STAGE_LENS: 0, _abi.STAGE_SCATTER: 2}.get(st.kind, 2)
        st.new_col_order.insert(n_extra, idc)
    return st


def fingerprint(stages):
    """Hash of everything lowered; a change triggers a re-upload."""
    import hashlib
    h = hashlib.sha1()
    for st in stages:
        h.update(np.asarray([st.kind, st.id_num], dtype=np.int64).tobytes())
        h.update(st.frame.tobytes())
        h.update(st.cyl.tobytes())
        h.update(st.p.tobytes())
        h.update(repr((st.out_names, st.id_col)).encode())
        if st.facets is not None:
            h.update(st.facets.tobytes())
        for sp in [st.spline] + [s.spline for s in st.selectors]:
            if sp is not None:
                for a in sp:
                    h.update(np.ascontiguousarray(a).tobytes())
        for s in st.selectors:
            for a in (s.energy, s.cdf, s.total, s.orders):
                h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


# ---------------------------------------------------------------------------
# FP32-local constant blocks
# ---------------------------------------------------------------------------
def split_ff(x):
    """float64 -> (hi, lo) float32 pair with hi + lo ~ x to ~2^-48."""
    x = np.asarray(x, dtype=np.float64)
    hi = x.astype(np.float32)
    lo = (x - hi.astype(np.float64)).astype(np.float32)
    return hi, lo


def split_ff_array(x):
    """float64 array -> float32 array of (hi, lo) pairs, shape (n, 2)."""
    hi, lo = split_ff(np.ravel(x))
    return np.ascontiguousarray(np.stack([hi, lo], axis=1))


def u53_threshold(x):
    """floor(x * 2^53), at least -1: for a 53-bit draw U (u = U * 2^-53),
    u > x exactly when U > this value."""
    v = math.floor(float(x) * 2.0 ** 53) if math.isfinite(float(x)) else (
        2 ** 62 if float(x) > 0 else -1)
    return int(min(max(v, -1), 2 ** 62))


def selector_rows32(sel):
    """FP32-local row lookup of a sorted energy-row selector: the midpoints
    of adjacent rows (float64) and the float32 guess constants E_0 and
    (n - 1) / (E_last - E_0); None when the selector has no such rows."""
    e = np.asarray(sel.energy, dtype=np.float64)
    if not (sel.by_energy and selector_sorted(sel) and len(e) >= 2):
        return None
    mid = np.ascontiguousarray(0.5 * (e[:-1] + e[1:]))
    return mid, float(np.float32(e[0])), float(np.float32((len(e) - 1) / (e[-1] - e[0])))


def flat32_block(st):
    b = _abi.MgpuFlat32()
    hi, lo = split_ff(st.frame[0:3])
    b.c_hi[:] = [float(v) for v in hi]
    b.c_lo[:] = [float(v) for v in lo]
    b.ex[:] = [float(v) for v in np.float32(st.frame[3:6])]
    b.ey[:] = [float(v) for v in np.float32(st.frame[6:9])]
    b.ez[:] = [float(v) for v in np.float32(st.frame[9:12])]
    b.hy = float(np.float32(st.frame[12]))
    b.hz = float(np.float32(st.frame[13]))
    p = [float(v) for v in st.p[:6]]
    if st.kind == _abi.STAGE_FLATDET:
        p[3] = 1.0 / st.p[0]
    b.p[:] = p
    return bytes(b)


def facets32_table(facets, detectors=False):
    """FP32-local element records of a facet table: the centre as
    float-float, frame, half sizes; for gratings the groove vectors and
    energy2wave / d as float-float, for detectors (``detectors``) in l the
    inverse pixel size and the centre pixel."""
    out = np.zeros(len(facets), dtype=_abi.FACET32_DTYPE)
    hi, lo = split_ff(facets['c'])
    out['c_hi'], out['c_lo'] = hi, lo
    for k in ('ex', 'ey', 'ez'):
        out[k] = facets[k].astype(np.float32)
    out['hy'] = facets['hy'].astype(np.float32)
    out['hz'] = facets['hz'].astype(np.float32)
    out['id_num'] = facets['id_num']
    out['selector'] = facets['selector']
    if detectors:
        out['l'][:, 0] = 1.0 / facets['dgrat']
        out['l'][:, 1:3] = facets['l'][:, 0:2]
        return out
    for k in ('l', 'dneg'):
        out[k] = facets[k].astype(np.float32)
    wd = 1.2398419292004202e-06 / facets['dgrat']
    out['wd_hi'], out['wd_lo'] = split_ff(wd)
    out['flags'] = facets['cat'] | (facets['transmission'] << 1)
    return out


def grid32_block(g):
    b = _abi.MgpuGrid32()
    hi, lo = split_ff(g['o'])
    b.o_hi[:] = [float(v) for v in hi]
    b.o_lo[:] = [float(v) for v in lo]
    for key in ('n', 'a', 'b'):
        getattr(b, key)[:] = [float(v) for v in np.float32(g[key])]
    # the float32 lookup grows every footprint by 0.05 mm on the host side
    b.u0 = float(g['u0'])
    b.v0 = float(g['v0'])
    b.inv_cell = float(1.0 / g['cell'])
    b.slope_max = float(g['slope_max'])
    b.nu, b.nv = g['nu'], g['nv']
    b.depth[:] = [float(v) for v in np.float32(g['depth'])]
    return bytes(b)


PHI_TABLE_STEP = 1024


def cyl32_block(st):
    """Cylinder constants and the table of reference points k/1024 rad:
    per k the global point P_k = c + R u_k (float-float), the radial u_k and
    the tangent t_k, as three float4 (P_k hi, u.x), (P_k lo, u.y), (t_k, u.z)."""
    from .geomath import decompose44
    e = st.element
    pos4d = np.asarray(e.geometry.pos4d, dtype=float)
    T, R, Z, S = decompose44(pos4d)
    if not np.isclose(Z[0], Z[1], rtol=1e-12, atol=0) or not np.allclose(S, 0, atol=1e-12):
        raise NotImplementedError('fp32local supports circular, unsheared cylinders only')
    b = _abi.MgpuCyl32()
    hi, lo = split_ff(T)
    b.c_hi[:] = [float(v) for v in hi]
    b.c_lo[:] = [float(v) for v in lo]
    for name, vec in (('e1', R[:, 0]), ('e2', R[:, 1]), ('a', R[:, 2])):
        getattr(b, name)[:] = [float(v) for v in np.float32(vec)]
    b.R = float(np.float32(Z[0]))
    b.Rz = float(Z[2])
    b1, b2 = float(st.cyl[26]), float(st.cyl[27])
    b.w1[:] = [float(np.float32(np.cos(b1))), float(np.float32(np.sin(b1)))]
    b.w2[:] = [float(np.float32(np.cos(b2))), float(np.float32(np.sin(b2)))]
    arc = (b2 - b1) if b1 < b2 else (2 * np.pi - b1 + b2)
    b.arc = 2 if b1 == b2 else (0 if arc <= np.pi else 1)
    ph, pl = split_ff(Z[0] / st.p[0])
    b.rpix_hi, b.rpix_lo = float(ph), float(pl)
    b.inv_pix = float(1.0 / st.p[0])
    b.cp0 = float(st.p[1])
    b.cp1 = float(st.p[2])
    kmax = int(np.ceil((np.pi + 0.01) * PHI_TABLE_STEP))
    k = np.arange(-kmax, kmax + 1)
    ang = k / PHI_TABLE_STEP
    u = np.cos(ang)[:, None] * R[:, 0] + np.sin(ang)[:, None] * R[:, 1]
    tg = -np.sin(ang)[:, None] * R[:, 0] + np.cos(ang)[:, None] * R[:, 1]
    P = T + Z[0] * u
    phi_, plo = split_ff(P)
    table = np.empty((len(k), 12), dtype=np.float32)
    table[:, 0:3], table[:, 3] = phi_, u[:, 0]
    table[:, 4:7], table[:, 7] = plo, u[:, 1]
    table[:, 8:11], table[:, 11] = tg, u[:, 2]
    b.k0 = int(k[0])
    b.nk = int(len(k))
    return bytes(b), table


def selector_thresholds(sel):
    """ceil(cdf * 2^53) per entry: for u = U * 2^-53, cdf > u  <=>  U < threshold."""
    scaled = np.ascontiguousarray(sel.cdf, dtype=np.float64) * 2.0 ** 53   # exact
    return np.ceil(scaled).astype(np.uint64)


def selector_guide(sel):
    """Guide table for the order search of a sorted selector: per row, 64
    entries, entry b = first order index k with U < threshold[k] for the draw
    U = b * 2^47 (uint8); None when the rows are not sorted or too long."""
    if not selector_sorted(sel) or sel.cdf.shape[1] > 255:
        return None
    th = selector_thresholds(sel).reshape(sel.cdf.shape)
    starts = np.arange(64, dtype=np.uint64) << np.uint64(47)
    guide = np.empty((th.shape[0], 64), dtype=np.uint8)
    for r in range(th.shape[0]):
        # number of thresholds <= U = first index with U < threshold
        guide[r] = np.searchsorted(th[r], starts, side='right')
    return guide


def selector_sorted(sel):
    """Energy rows strictly increasing and every cumulative row
    non-decreasing: the FP32-local kernel may then binary-search both."""
    e = np.asarray(sel.energy, dtype=np.float64)
    cdf = np.asarray(sel.cdf, dtype=np.float64)
    return bool(sel.by_energy and len(e) > 0 and np.all(e > 0) and np.all(np.diff(e) > 0) and
                np.all(np.diff(cdf, axis=1) >= 0))