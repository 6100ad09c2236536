"""Host-side FP64 frame math: homogeneous coordinates and 4x4 pose algebra.

These run once per geometry version (set-up), never per photon.  They
restate the helpers the MARXS element constructors and ``Parallel`` use:

* ``e2h`` / ``h2e`` / ``norm_vector``       -- marxs/math/utils.py:10-64, 150-164
* ``translation2aff`` / ``zoom2aff`` / ``mat2aff`` -- marxs/math/utils.py:89-148
* ``compose`` / ``decompose44``           -- affine A = T R Z S (transforms3d
  convention used at marxs/base/base.py:317 and simulator.py:413-418)
* ``axangle2mat`` / ``euler2mat``         -- rotations used by element poses
  (marxs/math/rotations.py:50-87, design/uncertainties.py:36-38)
* ``parse_position_keywords``             -- marxs/base/base.py:292-336
* ``ex2vec_fix``                          -- marxs/math/rotations.py:9-47
"""
import numpy as np


def e2h(e, w):
    if not ((w == 0) or (w == 1)):
        raise ValueError('w must be 0 or 1.')
    e = np.asarray(e, dtype=float)
    shape = list(e.shape)
    shape[-1] += 1
    h = np.empty(shape)
    h[..., :3] = e
    h[..., 3] = w
    return h


def h2e(h):
    h = np.asarray(h, dtype=float)
    if np.all(h[..., 3] == 0) or np.allclose(h[..., 3], 1):
        return h[..., :3]
    if np.all(h[..., 3] != 0):
        return h[..., :3] / h[..., 3][..., None]
    raise ValueError('Input array must be either all Euclidean points or all points at infinity.')


def norm_vector(vec):
    vec = np.asarray(vec, dtype=float)
    return vec / np.sqrt(np.sum(vec * vec, axis=-1))[..., None]


def translation2aff(vec):
    if len(vec) != 3:
        raise ValueError('3d translation vector expected.')
    m = np.eye(4)
    m[:3, 3] = vec
    return m


def zoom2aff(zoom):
    z = np.eye(4)
    if np.isscalar(zoom):
        z[:3, :3] = zoom * z[:3, :3]
    elif len(zoom) == 3:
        z[:3, :3] = np.diag(zoom)
    else:
        raise ValueError('Zoom must be either scalar or 3 element vector.')
    return z


def mat2aff(mat):
    m = np.eye(4)
    m[:3, :3] = mat
    return m


def compose(T, R, Z, S=None):
    """Affine 4x4 from translation, rotation, zoom (and optional shears)."""
    T = np.asarray(T, dtype=float)
    R = np.asarray(R, dtype=float)
    Z = np.asarray(Z, dtype=float)
    A = np.eye(4)
    Smat = np.eye(3)
    if S is not None:
        Smat[np.triu_indices(3, 1)] = S
    A[:3, :3] = R @ (np.diag(Z) @ Smat)
    A[:3, 3] = T
    return A


def decompose44(A44):
    """Split an affine into (T, R, Z, S) by Gram-Schmidt on the columns."""
    A44 = np.asarray(A44, dtype=float)
    T = A44[:3, 3].copy()
    c0, c1, c2 = np.array(A44[:3, :3]).T
    sx = np.sqrt(np.sum(c0 * c0))
    c0 = c0 / sx
    sx_sxy = np.dot(c0, c1)
    c1 = c1 - sx_sxy * c0
    sy = np.sqrt(np.sum(c1 * c1))
    c1 = c1 / sy
    sx_sxz = np.dot(c0, c2)
    sy_syz = np.dot(c1, c2)
    c2 = c2 - (sx_sxz * c0 + sy_syz * c1)
    sz = np.sqrt(np.sum(c2 * c2))
    c2 = c2 / sz
    R = np.array([c0, c1, c2]).T
    if np.linalg.det(R) < 0:
        sx = -sx
        R[:, 0] *= -1
    return T, R, np.array([sx, sy, sz]), np.array([sx_sxy / sx, sx_sxz / sx, sy_syz / sy])


def axangle2mat(axis, angle, is_normalized=False):
    """Rodrigues rotation matrix for one axis and angle."""
    x, y, z = np.asarray(axis, dtype=float)[:3]
    if not is_normalized:
        n = np.sqrt(x * x + y * y + z * z)
        x, y, z = x / n, y / n, z / n
    c, s = np.cos(angle), np.sin(angle)
    C = 1 - c
    return np.array([[x * x * C + c, x * y * C - z * s, x * z * C + y * s],
                     [y * x * C + z * s, y * y * C + c, y * z * C - x * s],
                     [z * x * C - y * s, z * y * C + x * s, z * z * C + c]])


def _rot(axis, a):
    c, s = np.cos(a), np.sin(a)
    if axis == 'x':
        return np.array([[1., 0, 0], [0, c, -s], [0, s, c]])
    if axis == 'y':
        return np.array([[c, 0, s], [0, 1., 0], [-s, 0, c]])
    return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1.]])


def euler2mat(ai, aj, ak, axes='sxyz'):
    """Euler sequence; 's' = static frame (R3 R2 R1), 'r' = rotating (R1 R2 R3)."""
    r1, r2, r3 = _rot(axes[1], ai), _rot(axes[2], aj), _rot(axes[3], ak)
    return r3 @ r2 @ r1 if axes[0] == 's' else r1 @ r2 @ r3


def parse_position_keywords(kwargs):
    """pos4d from ``pos4d`` or ``position``/``orientation``/``zoom`` (pops keys)."""
    pos4d = kwargs.pop('pos4d', None)
    if pos4d is None:
        position = kwargs.pop('position', np.zeros(3))
        orientation = kwargs.pop('orientation', np.eye(3))
        zoom = kwargs.pop('zoom', 1.)
        if np.isscalar(zoom):
            zoom = np.ones(3) * zoom
        if not len(zoom) == 3:
            raise ValueError('zoom must have three elements for x,y,z or be a scalar (global zoom).')
        if np.any(np.array(zoom) <= 0):
            raise ValueError('All values in zoom must be positive-definite to keep pos4d matrix valid.')
        pos4d = compose(position, orientation, zoom)
    else:
        if ('position' in kwargs) or ('orientation' in kwargs) or ('zoom' in kwargs):
            raise ValueError('If pos4d is specificed, the following keywords cannot be given at '
                             'the same time: position, orientation, zoom.')
    pos4d = np.array(pos4d, dtype=float)
    if np.linalg.det(pos4d) == 0:
        raise ValueError('pos4d matrix is invalid (determinant is 0).')
    return pos4d


def ex2vec_fix(e1, efix):
    """Rotation taking x to ``e1`` with the new y coplanar with ``efix``."""
    e1 = np.asarray(e1, dtype=float)
    e1 = e1 / np.linalg.norm(e1)
    efix = np.asarray(efix, dtype=float)
    efix = efix / np.linalg.norm(efix)
    if np.allclose(e1, efix) or np.allclose(e1, -efix):
        raise ValueError('Input vectors are parallel - Rotation matrix is ambiguous.')
    rot = np.empty((3, 3))
    rot[:, 0] = e1
    v = efix - np.dot(efix, e1) * e1
    rot[:, 1] = v / np.linalg.norm(v)
    rot[:, 2] = np.cross(rot[:, 0], rot[:, 1])
    return rot


def anglediff(phi):
    d = phi[1] - phi[0]
    if (d < 0.) or (d > (2. * np.pi)):
        d = d % (2. * np.pi)
    return d


def polarization_vectors(dir_array, angles):
    """Polarization unit vectors from angles (marxs/math/polarization.py:12-63)."""
    dir_array = np.asarray(dir_array, dtype=float)
    angles = np.asarray(angles, dtype=float)
    n = len(angles)
    polarization = np.zeros((n, 4))
    x = np.array([1., 0., 0.])
    y = np.array([0., 1., 0.])
    r = dir_array.copy()[:, 0:3]
    r /= np.linalg.norm(r, axis=1)[:, np.newaxis]
    conv_x = np.isclose(r[:, 0], 0.) & np.isclose(r[:, 2], 0.)
    v_1 = ~conv_x[:, None] * (y - r * np.dot(r, y)[:, None])
    v_1 += conv_x[:, None] * (x - r * np.dot(r, x)[:, None])
    v_1 /= np.linalg.norm(v_1, axis=1)[:, None]
    v_2 = np.cross(r, v_1)
    polarization[:, 0:3] = v_1 * np.cos(angles)[:, None] + v_2 * np.sin(angles)[:, None]
    return polarization
