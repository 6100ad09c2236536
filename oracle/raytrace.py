"""CPU oracle for the MARXS photon-raytrace hot path (float64 numpy).

TEST INFRASTRUCTURE ONLY.  This module restates the reference algorithm so
that tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` can check and time the GPU backend against it.  The product
path never imports it.

Each function follows the reference function named in its docstring
(paths relative to the MARXS source tree).  Randomness is not drawn here:
every stochastic step reads per-photon pre-drawn values, so that the same
draws can be fed to the GPU kernels.  ``draws`` maps an element object to a
dict of per-photon arrays (length N, indexed by photon row):

* RadialMirrorScatter: ``'inplanescatter'``, ``'perpplanescatter'`` (angles, rad)
* a grating (or a Parallel of gratings): ``'order_u'`` (uniform in [0, 1))

Parity of this oracle with the reference itself is pinned by golden vectors
recorded from the reference (``tests/golden/``).
"""
import math

import numpy as np

ENERGY2WAVE = 1.2398419292004202e-06   # keV -> mm, marxs/__init__.py:14


def _classnames(obj):
    return {c.__name__ for c in type(obj).__mro__}


# --------------------------------------------------------------------------
# math helpers: marxs/math/utils.py
# --------------------------------------------------------------------------
def norm_vector(vec):
    """marxs/math/utils.py:150-164"""
    length2 = np.sum(vec * vec, axis=-1)
    return vec / np.sqrt(length2)[:, None]


def e2h(e, w):
    """marxs/math/utils.py:10-34"""
    shape = list(e.shape)
    shape[-1] += 1
    h = np.empty(shape)
    h[..., :3] = e
    h[..., 3] = w
    return h


def h2e(h):
    """marxs/math/utils.py:37-64"""
    if np.all(h[..., 3] == 0) or np.allclose(h[..., 3], 1):
        return h[..., :3]
    elif np.all(h[..., 3] != 0):
        return h[..., :3] / h[..., 3][..., None]
    raise ValueError('mixed homogeneous points and directions')


def _npmod(a, b):
    """numpy floor-modulo for floats."""
    return np.mod(a, b)


def angle_between(angle, border1, border2):
    """marxs/math/utils.py:180-215"""
    twopi = 2 * np.pi
    b1 = (twopi + (border1 % twopi)) % twopi
    b2 = (twopi + (border2 % twopi)) % twopi
    ang = (twopi + _npmod(angle, twopi)) % twopi
    if b1 < b2:
        return (b1 <= ang) & (ang <= b2)
    return (b1 <= ang) | (ang <= b2)


def axangle2mat(axes, angles):
    """Vectorised Rodrigues matrices, marxs/math/rotations.py:50-87"""
    axes = axes / np.linalg.norm(axes, axis=1)[:, None]
    c = np.cos(angles)
    s = np.sin(angles)
    C = 1 - c
    x = axes[:, 0]
    y = axes[:, 1]
    z = axes[:, 2]
    xs = x * s
    ys = y * s
    zs = z * s
    xC = x * C
    yC = y * C
    zC = z * C
    xyC = x * yC
    yzC = y * zC
    zxC = z * xC
    return np.array([[x * xC + c, xyC - zs, zxC + ys],
                     [xyC + zs, y * yC + c, yzC - xs],
                     [zxC - ys, yzC + xs, z * zC + c]]).swapaxes(0, 2).swapaxes(1, 2)


# --------------------------------------------------------------------------
# polarization: marxs/math/polarization.py
# --------------------------------------------------------------------------
def paralleltransport_matrix(dir1, dir2):
    """marxs/math/polarization.py:90-149 (jones = identity, replace_nans=True)"""
    dir1 = norm_vector(dir1)
    dir2 = norm_vector(dir2)
    pmat = np.zeros((dir1.shape[0], 3, 3))
    s = np.cross(dir1, dir2)
    s_norm = np.linalg.norm(s, axis=1)
    ind = np.isclose(s_norm, 0)
    if (~ind).sum() > 0:
        s = s[~ind, :] / s_norm[~ind][:, None]
        p_in = np.cross(dir1[~ind, :], s)
        p_out = np.cross(dir2[~ind, :], s)
        Oininv = np.array([s, p_in, dir1[~ind, :]]).swapaxes(1, 0)
        Oout = np.array([s, p_out, dir2[~ind, :]]).swapaxes(1, 2).T
        temp = np.einsum('...ij,kjl->kil', np.eye(3), Oininv)
        pmat[~ind, :, :] = np.einsum('ijk,ikl->ijl', Oout, temp)
    pmat[ind, :, :] = np.eye(3)[None, :, :]
    return pmat


def parallel_transport(dir_old, dir_new, pol_old):
    """marxs/math/polarization.py:151-170"""
    pmat = paralleltransport_matrix(dir_old[:, :3], dir_new[:, :3])
    out = np.einsum('ijk,ik->ij', pmat, pol_old[:, :3])
    return e2h(out, 0)


# --------------------------------------------------------------------------
# geometry: marxs/math/geometry.py
# --------------------------------------------------------------------------
def _geom_vec(pos4d, key):
    """Geometry.__getitem__, marxs/math/geometry.py:108-160"""
    if key == 'center':
        return pos4d[:, 3]
    col = {'x': 0, 'y': 1, 'z': 2}[key[-1]]
    val = pos4d[:, col]
    if key[:2] == 'e_':
        return val / np.linalg.norm(val)
    return val


def finite_plane_intersect(pos4d, dir, pos):
    """FinitePlane.intersect, marxs/math/geometry.py:211-261"""
    center = _geom_vec(pos4d, 'center')
    e_x = _geom_vec(pos4d, 'e_x')
    k_nominator = np.dot(center - pos, e_x)
    k_denom = np.dot(dir, e_x)
    is_parallel = k_denom == 0
    with np.errstate(divide='ignore', invalid='ignore'):
        k = k_nominator / k_denom
        forward = k >= 0
        interpos = pos + k[:, None] * dir
    vec_center_inter = interpos - center
    interpos_local = np.vstack([np.dot(vec_center_inter, _geom_vec(pos4d, 'e_y')),
                                np.dot(vec_center_inter, _geom_vec(pos4d, 'e_z'))]).T
    with np.errstate(invalid='ignore'):
        intersect = (~is_parallel & forward &
                     (np.abs(interpos_local[:, 0]) <= np.linalg.norm(_geom_vec(pos4d, 'v_y'))) &
                     (np.abs(interpos_local[:, 1]) <= np.linalg.norm(_geom_vec(pos4d, 'v_z'))))
    for i in [interpos, interpos_local]:
        i[~intersect, :3] = np.nan
    return intersect, interpos, interpos_local


def _decompose_zoom(pos4d):
    """Zoom vector of an affine pose (Gram-Schmidt on the columns), as the
    reference obtains it through ``decompose44`` (geometry.py:447, 556;
    detector.py:61)."""
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


def cylinder_intersect(pos4d, phi_lim, dir, pos):
    """Cylinder.intersect, marxs/math/geometry.py:470-564"""
    if not np.all(dir[:, 3] == 0):
        raise ValueError('First input must be direction vectors.')
    invpos4d = np.linalg.inv(pos4d)
    dir = np.dot(invpos4d, dir.T).T
    pos = np.dot(invpos4d, pos.T).T
    xyz = h2e(pos)
    dir_e = h2e(dir)
    xy = xyz[:, :2]
    r = dir[:, :2]
    c = np.sum(xy ** 2, axis=1) - 1.
    b = 2 * np.sum(xy * r, axis=1)
    a = np.sum(r ** 2, axis=1)
    underroot = b ** 2 - 4 * a * c
    with np.errstate(invalid='ignore'):
        intersect = (underroot >= 0)
    i = intersect
    interpos_local = np.ones((pos.shape[0], 2))
    interpos_local[:] = np.nan
    interpos = np.ones_like(pos)
    interpos[:] = np.nan
    if intersect.sum() > 0:
        i_ind = intersect.nonzero()[0]
        denom = 2 * a[i]
        with np.errstate(divide='ignore', invalid='ignore'):
            a1 = (- b[i] + np.sqrt(underroot[i])) / denom
            a2 = (- b[i] - np.sqrt(underroot[i])) / denom
        xy_1 = xy[i, :] + a1[:, np.newaxis] * r[i, :]
        phi_1 = np.arctan2(xy_1[:, 1], xy_1[:, 0])
        xy_2 = xy[i, :] + a2[:, np.newaxis] * r[i, :]
        phi_2 = np.arctan2(xy_2[:, 1], xy_2[:, 0])
        z_1 = xyz[i, 2] + a1 * dir[i, 2]
        z_2 = xyz[i, 2] + a2 * dir[i, 2]
        with np.errstate(invalid='ignore'):
            hit_1 = ((a1 >= 0) & (np.abs(z_1) <= 1.) &
                     angle_between(phi_1, phi_lim[0], phi_lim[1]))
            hit_2 = ((a2 >= 0) & (np.abs(z_2) <= 1.) &
                     angle_between(phi_2, phi_lim[0], phi_lim[1]))
            hit_1[hit_2 & (a2 < a1)] = False
            hit_2[hit_1 & (a2 >= a1)] = False
        intersect[i_ind] = hit_1 | hit_2
        interpos_local[i_ind[hit_1], 0] = phi_1[hit_1]
        interpos_local[i_ind[hit_1], 1] = z_1[hit_1]
        interpos_local[i_ind[hit_2], 0] = phi_2[hit_2]
        interpos_local[i_ind[hit_2], 1] = z_2[hit_2]
        interpos[i_ind[hit_1], :] = e2h(xyz[i_ind, :] + a1[:, None] * dir_e[i_ind, :], 1)[hit_1, :]
        interpos[i_ind[hit_2], :] = e2h(xyz[i_ind, :] + a2[:, None] * dir_e[i_ind, :], 1)[hit_2, :]
        zoom = _decompose_zoom(pos4d)
        interpos_local[:, 1] = interpos_local[:, 1] * zoom[2]
        interpos = np.dot(pos4d, interpos.T).T
    return intersect, interpos, interpos_local


# --------------------------------------------------------------------------
# order selection: marxs/optics/grating.py
# --------------------------------------------------------------------------
HC_KEV_NM = 1.2398419843320026   # h c in keV nm (CODATA 2018, as astropy's spectral())


def bisp_k1(tx, ty, c, x, y):
    """scipy RectBivariateSpline(kx=1, ky=1).ev(x, y): FITPACK fpbisp for
    degree 1 (arguments clamped to [t[1], t[n-2]]; interval l = last knot
    <= arg, at most n-3; de Boor weights f = 1/(t[l+1]-t[l]),
    h0 = f (t[l+1]-arg), h1 = f (arg-t[l]); value = sum over the 2x2
    coefficients of (c * hx) * hy in x-major order)."""
    x = np.asarray(x, dtype=float)
    y = np.asarray(y, dtype=float)
    tx, ty, c = np.asarray(tx), np.asarray(ty), np.asarray(c)

    def weights(t, a):
        n = len(t)
        arg = np.minimum(np.maximum(a, t[1]), t[n - 2])
        l = np.minimum(1 + np.searchsorted(t[2:n - 1], arg, side='right'), n - 3)
        f = 1.0 / (t[l + 1] - t[l])
        return l, f * (t[l + 1] - arg), f * (arg - t[l])

    lx, hx0, hx1 = weights(tx, x)
    ly, hy0, hy1 = weights(ty, y)
    nky1 = len(ty) - 2
    base = (lx - 1) * nky1 + (ly - 1)
    sp = np.zeros(len(x))
    for dx, hx in ((0, hx0), (1, hx1)):
        for dy, hy in ((0, hy0), (1, hy1)):
            sp = sp + c[base + dx * nky1 + dy] * hx * hy
    return sp


def order_select(selector, energy, u, blaze=None):
    """OrderSelector (grating.py:51-57) / EfficiencyFile (grating.py:88-96) /
    InterpolateEfficiencyTable (missions/mitsnl/catgrating.py:101-144).

    ``u`` holds one uniform per photon.  OrderSelector draws through
    ``np.random.choice(p=...)``, i.e. ``searchsorted(cdf/cdf[-1], u, 'right')``;
    EfficiencyFile takes the nearest energy row and the first order whose
    cumulative probability exceeds ``u``; InterpolateEfficiencyTable
    evaluates one spline per order at (wavelength in nm, blaze angle), sums
    them (row by row), normalises the running sum and takes
    ``argmax(cumprob > u)`` -- order index 0 when no entry exceeds ``u``.
    """
    names = _classnames(selector)
    if hasattr(selector, 'interpolators'):
        wave = HC_KEV_NM / np.asarray(energy, dtype=float)
        interpprobs = np.empty((len(selector.orders), len(energy)))
        for i, ip in enumerate(selector.interpolators):
            interpprobs[i, :] = ip.ev(wave, blaze)
        totalprob = np.sum(interpprobs, axis=0)
        cumprob = np.cumsum(interpprobs, axis=0) / totalprob
        ind = np.argmax(cumprob > u, axis=0)
        return np.asarray(selector.orders)[ind], totalprob
    if 'EfficiencyFile' in names:
        ind = np.array([np.argmin(np.abs(selector.energy - e)) for e in energy], dtype=int)
        orderind = np.empty(len(energy), dtype=int)
        for j in range(len(energy)):
            orderind[j] = np.min(np.nonzero(selector.cumprob[ind[j]] > u[j]))
        return selector.orders[orderind], selector.totalprob[ind]
    if 'OrderSelector' in names:
        p_sum = selector.p.sum()
        p = selector.p / p_sum
        cdf = p.cumsum()
        cdf /= cdf[-1]
        idx = cdf.searchsorted(u, side='right')
        return np.asarray(selector.orderlist)[idx], p_sum * np.ones_like(energy)
    raise NotImplementedError('order selector %r' % type(selector))


def _grating_params(g):
    ga = g.geometry._geometry.get('groove_angle', 0.)
    return ga


def e_groove_coos(pos4d, groove):
    """FlatGrating.e_groove_coos, grating.py:186-207 with the flat bases
    of FinitePlane.get_local_euklid_bases (geometry.py:263-281)."""
    ex = _geom_vec(pos4d, 'e_y')
    ey = _geom_vec(pos4d, 'e_z')
    en = _geom_vec(pos4d, 'e_x')
    e_groove = math.sin(-groove) * ex + math.cos(-groove) * ey
    e_perp_groove = math.cos(-groove) * ex - math.sin(-groove) * ey
    return e_groove, e_perp_groove, en


def _custom_blaze_modifier(g):
    """blaze_angle_modifier overridden on the instance or by a subclass of
    FlatGrating (whose own returns zeros, grating.py:222-231)."""
    if 'blaze_angle_modifier' in vars(g):
        return True
    for klass in type(g).__mro__:
        if 'blaze_angle_modifier' in vars(klass):
            return klass.__name__ != 'FlatGrating'
    return False


def cylinder_groove_coos(geometry, groove, intercoos):
    """FlatGrating.e_groove_coos (grating.py:186-207) on a Cylinder surface:
    the local bases of Cylinder.get_local_euklid_bases
    (math/geometry.py:602-626) at each photon's angle phi."""
    phi = intercoos[:, 0]
    zeros = np.zeros_like(phi)
    e_phi = np.array([-np.sin(phi), np.cos(phi), zeros, zeros]).T
    e_z = np.tile(_geom_vec(geometry.pos4d, 'e_z'), (intercoos.shape[0], 1))
    e_n = np.array([np.cos(phi), np.sin(phi), zeros, zeros]).T
    e_phi = norm_vector(np.einsum('...ij,...j', geometry.pos4d, e_phi))
    e_n = norm_vector(np.einsum('...ij,...j', geometry.pos4d, e_n))
    e_groove = math.sin(-groove) * e_phi + math.cos(-groove) * e_z
    e_perp_groove = math.cos(-groove) * e_phi - math.sin(-groove) * e_z
    return e_groove, e_perp_groove, e_n


def flat_grating_process(g, photons, intersect, intercoos, u):
    """FlatGrating.diffract_photons + specific_process_photons, grating.py:233-277"""
    n_hit = intersect.sum()
    p = norm_vector(photons['dir'][intersect])
    if 'Cylinder' in _classnames(g.geometry):
        l, d, n = cylinder_groove_coos(g.geometry, _grating_params(g), intercoos[intersect])
    else:
        l1, d1, n1 = e_groove_coos(g.geometry.pos4d, _grating_params(g))
        l = np.tile(l1, (n_hit, 1))
        d = np.tile(d1, (n_hit, 1))
        n = np.tile(n1, (n_hit, 1))
    d = - d
    wave = ENERGY2WAVE / photons['energy'][intersect]
    p_perp_to_grooves = norm_vector(p - np.einsum('ij,ij->i', p, l)[:, None] * l)
    blazeangle = np.arccos(np.clip(np.abs(np.einsum('ij,ij->i', p_perp_to_grooves, n)), 0, 1))
    if hasattr(g, 'd_blaze_mm'):
        # NonParallelCATGrating.blaze_angle_modifier, missions/mitsnl/catgrating.py:324-333
        blazeangle += g.blaze_center + intercoos[intersect, 0] * g.d_blaze_mm
    elif _custom_blaze_modifier(g):
        # an overridden blaze_angle_modifier, called as grating.py:255 does
        blazeangle += g.blaze_angle_modifier(intercoos[intersect, :])
    else:
        blazeangle += np.zeros(n_hit)
    m, prob = order_select(g.order_selector, photons['energy'][intersect], u[intersect],
                           blazeangle)
    if 'CATGrating' in _classnames(g):
        dotproduct = np.einsum('ij,ij->i', p, d)
        sign = np.sign(dotproduct)
        sign[sign == 0] = 1
    else:
        sign = -1
    dval = g._d if not callable(g._d) else g._d(intercoos[intersect, :])
    p_d = np.einsum('ij,ij->i', p, d) + sign * m * wave / dval
    p_l = np.einsum('ij,ij->i', p, l)
    with np.errstate(invalid='ignore'):
        p_n = np.sqrt(1. - p_d ** 2 - p_l ** 2)
    direction = np.sign(np.einsum('ij,ij->i', p, n), dtype=float)
    if not g.transmission:
        direction *= -1
    newdir = p_d[:, None] * d + p_l[:, None] * l + (direction * p_n)[:, None] * n
    pol = parallel_transport(photons['dir'][intersect, :], newdir,
                             photons['polarization'][intersect, :])
    return {'dir': newdir, 'probability': prob, 'polarization': pol,
            g.order_name: m, g.blaze_name: blazeangle}


def perfect_lens_process(lens, photons, intersect, interpos):
    """PerfectLens.specific_process_photons, marxs/optics/mirror.py:53-82"""
    pos4d = lens.geometry.pos4d
    p_opt_axis = _geom_vec(pos4d, 'center') - lens.d_center_optax * _geom_vec(pos4d, 'e_z')
    focuspoints = h2e(p_opt_axis) + lens.focallength * norm_vector(h2e(photons['dir'][intersect]))
    newdir = norm_vector(e2h(focuspoints - h2e(interpos[intersect]), 0))
    pol = parallel_transport(photons['dir'][intersect, :], newdir,
                             photons['polarization'][intersect, :])
    interp = getattr(lens, 'reflectivity_interpolator', None)
    if interp is None:
        prob = np.ones(intersect.sum())
    else:
        angle = np.arccos(np.abs(np.einsum('ij,ij->i', h2e(newdir),
                                           norm_vector(h2e(photons['dir'][intersect])))))
        prob = interp(photons['energy'][intersect], angle / 4, grid=False) ** 2
    return {'dir': newdir, 'polarization': pol, 'probability': prob}


def radial_mirror_scatter_process(rms, photons, intersect, inplane_draw, perp_draw):
    """RadialMirrorScatter.specific_process_photons, marxs/optics/scatter.py:49-77

    The drawn angles replace ``np.random.normal(0, sigma, n)``."""
    n = intersect.sum()
    center = rms.geometry.pos4d[:-1, -1]
    radial = h2e(photons['pos'][intersect]) - center
    perpplane = np.cross(h2e(photons['dir'][intersect]), radial)
    if rms.inplanescatter != 0:
        inplaneangle = inplane_draw[intersect]
        rot = axangle2mat(perpplane, inplaneangle)
        outdir = e2h(np.einsum('...ij,...i->...j', rot, h2e(photons['dir'][intersect])), 0)
    else:
        inplaneangle = np.zeros(n)
        outdir = photons['dir'][intersect]
    if rms.perpplanescatter != 0:
        perpangle = perp_draw[intersect]
        rot = axangle2mat(radial, perpangle)
        outdir = e2h(np.einsum('...ij,...i->...j', rot, h2e(outdir)), 0)
    else:
        perpangle = np.zeros_like(inplaneangle)
    pol = parallel_transport(photons['dir'][intersect, :], outdir,
                             photons['polarization'][intersect, :])
    return {'dir': outdir, 'polarization': pol,
            rms.inplanescattercol: inplaneangle, rms.perpplanescattercol: perpangle}


def flat_detector_process(det, intersect, intercoos):
    """FlatDetector.specific_process_photons, marxs/optics/detector.py:72-75"""
    detx = intercoos[intersect, 0] / det.pixsize + det.centerpix[0]
    dety = intercoos[intersect, 1] / det.pixsize + det.centerpix[1]
    return {det.detpix_name[0]: detx, det.detpix_name[1]: dety}


def circular_detector_process(det, intersect, intercoos):
    """CircularDetector.specific_process_photons, marxs/optics/detector.py:115-118"""
    R = _decompose_zoom(det.geometry.pos4d)[0]
    detx = intercoos[intersect, 0] * R / det.pixsize + det.centerpix[0]
    dety = intercoos[intersect, 1] / det.pixsize + det.centerpix[1]
    return {det.detpix_name[0]: detx, det.detpix_name[1]: dety}


# --------------------------------------------------------------------------
# element protocol: marxs/optics/base.py, marxs/base/base.py
# --------------------------------------------------------------------------
def add_output_cols(elem, photons, colnames):
    """SimulationSequenceElement.add_output_cols, marxs/base/base.py:249-286"""
    n = len(photons['energy'])
    for c in list(getattr(elem, 'output_columns', [])) + list(colnames):
        if c is not None and c not in photons:
            photons[c] = np.full(n, np.nan)
    idc = getattr(elem, 'id_col', None)
    if idc is not None and idc not in photons:
        photons[idc] = np.full(n, -1, dtype=int)


def assign_col_value(photons, col, index, value):
    """_assign_col_value, marxs/optics/base.py:12-51"""
    if col == 'probability':
        if np.any(value < 0) or np.any(value > 1):
            raise ValueError('Found probability outside of the 0..1 arange.')
        photons[col][index] *= value
    elif col is None:
        pass
    else:
        photons[col][index] = value


def process_photons(elem, photons, intersect, interpos, intercoos, outcols):
    """OpticalElement.process_photons, marxs/optics/base.py:149-211"""
    add_output_cols(elem, photons, list(outcols.keys()))
    for col in outcols:
        assign_col_value(photons, col, intersect, np.asarray(outcols[col]))
    if elem.loc_coos_name is not None:
        add_output_cols(elem, photons, list(elem.loc_coos_name))
        photons[elem.loc_coos_name[0]][intersect] = intercoos[intersect, 0]
        photons[elem.loc_coos_name[1]][intersect] = intercoos[intersect, 1]
    if getattr(elem, 'id_col', None) is not None:
        photons[elem.id_col][intersect] = elem.id_num
    photons['pos'][intersect] = interpos[intersect]
    return photons


def gaussian_scatter_process(elem, photons, intersect, normals, phi_u):
    """RandomGaussianScatter.specific_process_photons (optics/scatter.py:109-150)
    with L2Diffraction.scatter (missions/mitsnl/catgrating.py:263-268):
    sigma = 1.22 * 0.4 * arcsin(lambda / inner), angle = N(0, 1) * sigma about
    dir x guess, then a uniform turn about the direction."""
    pdir = norm_vector(h2e(photons['dir'][intersect]))
    guessvec = np.zeros_like(pdir)
    ind = np.abs(pdir[:, 0]) < 0.99999
    guessvec[ind, 0] = 1
    guessvec[~ind, 1] = 1
    perpvec = np.cross(pdir, guessvec)
    wave = (HC_KEV_NM / (photons['energy'][intersect] * 1.0)) * (1e-6 / 1.0)   # keV -> mm
    sigma = 1.22 * 0.4 * np.arcsin(wave / elem.innerfree)
    angle = normals[intersect] * sigma
    rot = axangle2mat(perpvec, angle)
    outdir = np.einsum('...ij,...i->...j', rot, pdir)
    angle2 = phi_u[intersect] * 2 * np.pi
    rot = axangle2mat(pdir, angle2)
    outdir = e2h(np.einsum('...ij,...i->...j', rot, outdir), 0)
    pol = parallel_transport(photons['dir'][intersect, :], outdir,
                             photons['polarization'][intersect, :])
    return {'dir': outdir, 'polarization': pol, elem.scattername: angle}


def cat_stack_process(stack, photons, intersect, interpos, intercoos, d):
    """FlatStack.process_photons (optics/base.py:264-281) of a CATL1L2Stack
    (missions/mitsnl/catgrating.py:336-377): the stack's own id and local
    columns, then each layer at the same intersection."""
    process_photons(stack, photons, intersect, interpos, intercoos, {})
    grat, qf, l1, l2abs, l2diff = stack.elements
    # membrane (NonParallelCATGrating)
    out = flat_grating_process(grat, photons, intersect, intercoos, d['order_u'])
    process_photons(grat, photons, intersect, interpos, intercoos, out)
    # QualityFactor, catgrating.py:160-161
    process_photons(qf, photons, intersect, interpos, intercoos,
                    {'probability': qf.factor ** (photons['order'][intersect] ** 2)})
    # L1, catgrating.py:196-207: a CAT grating, or the support bars
    out = flat_grating_process(l1, photons, intersect, intercoos, d['l1_order_u'])
    sup = d['l1_support_u'][intersect] > l1.openfraction
    ind = intersect.nonzero()[0][sup]
    out['dir'][sup] = photons['dir'][ind, :]
    out['polarization'][sup] = photons['polarization'][ind, :]
    out[l1.order_name][sup] = 0
    out['probability'][sup] = l1.transfunc(photons['energy'][ind])
    process_photons(l1, photons, intersect, interpos, intercoos, out)
    # L2Abs, catgrating.py:231-245 (en = e_x of the flat element)
    p3 = norm_vector(photons['dir'][intersect])
    en = np.tile(_geom_vec(l2abs.geometry.pos4d, 'e_x'), (len(p3), 1))
    angle = np.arccos(np.abs(np.einsum('ij,ij->i', p3, en)))
    openfraction = (l2abs.innerfree / l2abs.period) ** 2
    shadowarea = (l2abs.bardepth * l2abs.innerfree * np.sin(angle))
    totalarea = l2abs.period ** 2 / 2 * np.sqrt(3)
    process_photons(l2abs, photons, intersect, interpos, intercoos,
                    {'probability': openfraction - shadowarea / totalarea})
    # L2Diffraction
    out = gaussian_scatter_process(l2diff, photons, intersect, d['l2_normal'], d['l2_phi_u'])
    process_photons(l2diff, photons, intersect, interpos, intercoos, out)
    return photons


def run_element(elem, photons, draws, stats):
    """One leaf element: OpticalElement.__call__ (optics/base.py:144-147)."""
    names = _classnames(elem)
    if 'CircularDetector' in names or 'Cylinder' in _classnames(elem.geometry):
        # any element on a Cylinder surface (detectors, bent gratings)
        intersect, interpos, intercoos = cylinder_intersect(
            elem.geometry.pos4d, elem.geometry.coos_limits[0], photons['dir'], photons['pos'])
    else:
        intersect, interpos, intercoos = finite_plane_intersect(
            elem.geometry.pos4d, photons['dir'], photons['pos'])
    if intersect.sum() == 0:
        return photons, intersect
    d = draws.get(elem, {})
    if 'CATL1L2Stack' in names:
        cat_stack_process(elem, photons, intersect, interpos, intercoos, d)
        return photons, intersect
    if 'FlatGrating' in names:
        u = d['order_u']
        outcols = flat_grating_process(elem, photons, intersect, intercoos, u)
    elif 'PerfectLens' in names:
        outcols = perfect_lens_process(elem, photons, intersect, interpos)
    elif 'RadialMirrorScatter' in names:
        outcols = radial_mirror_scatter_process(elem, photons, intersect,
                                                d.get('inplanescatter'), d.get('perpplanescatter'))
    elif 'FlatDetector' in names:
        outcols = flat_detector_process(elem, intersect, intercoos)
    elif 'CircularDetector' in names:
        outcols = circular_detector_process(elem, intersect, intercoos)
    else:
        raise NotImplementedError('oracle does not implement %s' % type(elem).__name__)
    process_photons(elem, photons, intersect, interpos, intercoos, outcols)
    return photons, intersect


def run_parallel(par, photons, draws, stats, mode='sequential'):
    """Parallel.__call__ = BaseContainer.__call__ (simulator.py:42-49).

    ``mode='sequential'`` is the reference semantics (each facet in order,
    later facets see rays already changed by earlier ones).  Per-photon
    draws of the container (``draws[par]``) are shared by all its facets.
    ``stats['multi_hit']`` counts photons processed by more than one facet.
    """
    d = draws.get(par, {})
    nhit = np.zeros(len(photons['energy']), dtype=int)
    for elem in par.elements:
        sub = dict(draws)
        if d:
            sub[elem] = d
        photons, inter = run_element(elem, photons, sub, stats)
        nhit += inter
    stats.setdefault('multi_hit', 0)
    stats['multi_hit'] += int((nhit > 1).sum())
    stats.setdefault('multi_hit_mask', np.zeros(len(nhit), dtype=bool))
    stats['multi_hit_mask'] |= nhit > 1
    return photons


def run_sequence(elements, photons, draws=None, stats=None):
    """Run an element chain on a dict-of-arrays photon list (copied).

    Containers (objects with ``elements``) recurse; a ``Parallel`` uses the
    sequential reference semantics.  Returns ``(photons, stats)``.
    """
    draws = {} if draws is None else draws
    stats = {} if stats is None else stats
    photons = {k: np.array(v, copy=True) for k, v in photons.items()}
    for elem in elements:
        photons = _run_any(elem, photons, draws, stats)
    return photons, stats


def support_bars(photons):
    """catsupportbars, missions/mitsnl/catgrating.py:314-324: probability 0
    where facet < 0, or everywhere without a facet column."""
    if 'facet' in photons:
        photons['probability'][np.asarray(photons['facet']) < 0] = 0.
    else:
        photons['probability'][...] = 0.
    return photons


def _run_any(elem, photons, draws, stats):
    if callable(elem) and getattr(elem, '__name__', None) == 'catsupportbars' and \
            not hasattr(elem, 'geometry'):
        return support_bars(photons)
    names = _classnames(elem)
    if 'Parallel' in names:
        return run_parallel(elem, photons, draws, stats)
    if hasattr(elem, 'elements') and ('Sequence' in names or 'BaseContainer' in names):
        for e in elem.elements:
            photons = _run_any(e, photons, draws, stats)
        return photons
    photons, _ = run_element(elem, photons, draws, stats)
    return photons
