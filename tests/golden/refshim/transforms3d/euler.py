"""Euler angle sequences as products of elementary rotations.

``axes`` is a 4-letter code: 's' (static frame) or 'r' (rotating frame)
followed by the three axis letters in the order the angles are applied.
A static sequence ``sXYZ`` applies ai about X first, then aj about Y, then
ak about Z, all about the fixed frame: R = R_Z(ak) R_Y(aj) R_X(ai).
A rotating sequence ``rXYZ`` is R = R_X(ai) R_Y(aj) R_Z(ak).
"""
import numpy as np


def _elementary(axis, angle):
    c, s = np.cos(angle), np.sin(angle)
    if axis == 'x':
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]], dtype=float)
    if axis == 'y':
        return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]], dtype=float)
    if axis == 'z':
        return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]], dtype=float)
    raise ValueError(axis)


def euler2mat(ai, aj, ak, axes='sxyz'):
    frame, a1, a2, a3 = axes[0], axes[1], axes[2], axes[3]
    r1 = _elementary(a1, ai)
    r2 = _elementary(a2, aj)
    r3 = _elementary(a3, ak)
    if frame == 's':
        return r3 @ r2 @ r1
    if frame == 'r':
        return r1 @ r2 @ r3
    raise ValueError(axes)
