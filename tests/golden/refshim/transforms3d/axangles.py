"""Rotation about an axis (Rodrigues' formula)."""
import numpy as np


def axangle2mat(axis, angle, is_normalized=False):
    x, y, z = np.asarray(axis, dtype=float)
    if not is_normalized:
        n = np.sqrt(x * x + y * y + z * z)
        x, y, z = x / n, y / n, z / n
    c = np.cos(angle)
    s = np.sin(angle)
    C = 1 - c
    return np.array([
        [x * x * C + c, x * y * C - z * s, x * z * C + y * s],
        [y * x * C + z * s, y * y * C + c, y * z * C - x * s],
        [z * x * C - y * s, z * y * C + x * s, z * z * C + c]])


def axangle2aff(axis, angle, point=None):
    M = np.eye(4)
    R = axangle2mat(axis, angle)
    M[:3, :3] = R
    if point is not None:
        point = np.asarray(point[:3], dtype=float)
        M[:3, 3] = point - np.dot(R, point)
    return M
