"""Affine compose / decompose written from the definition A = T * R * Z * S.

``Z`` is the diagonal zoom, ``S`` the upper-triangular shear with unit
diagonal (three shear factors ``sxy, sxz, syz`` for 3-D).  Decomposition is a
Gram-Schmidt orthogonalisation of the columns of the upper-left block.
"""
import numpy as np


def _shear_matrix(S, n):
    Smat = np.eye(n)
    if S is not None:
        Smat[np.triu_indices(n, 1)] = S
    return Smat


def compose(T, R, Z, S=None):
    T = np.asarray(T, dtype=float)
    R = np.asarray(R, dtype=float)
    Z = np.asarray(Z, dtype=float)
    n = len(T)
    if R.shape != (n, n):
        raise ValueError('Expecting shape (%d, %d) for rotations' % (n, n))
    A = np.eye(n + 1)
    ZS = np.dot(np.diag(Z), _shear_matrix(S, n))
    A[:n, :n] = np.dot(R, ZS)
    A[:n, n] = T[:]
    return A


def decompose44(A44):
    A44 = np.asarray(A44, dtype=float)
    T = A44[:-1, -1]
    RZS = A44[:-1, :-1]
    M0, M1, M2 = np.array(RZS).T
    sx = np.sqrt(np.sum(M0 * M0))
    M0 = M0 / sx
    sx_sxy = np.dot(M0, M1)
    M1 = M1 - sx_sxy * M0
    sy = np.sqrt(np.sum(M1 * M1))
    M1 = M1 / sy
    sxy = sx_sxy / sx
    sx_sxz = np.dot(M0, M2)
    sy_syz = np.dot(M1, M2)
    M2 = M2 - (sx_sxz * M0 + sy_syz * M1)
    sz = np.sqrt(np.sum(M2 * M2))
    M2 = M2 / sz
    sxz = sx_sxz / sx
    syz = sy_syz / sy
    R = np.array([M0, M1, M2]).T
    if np.linalg.det(R) < 0:
        sx *= -1
        R[:, 0] *= -1
    return T, R, np.array([sx, sy, sz]), np.array([sxy, sxz, syz])


def decompose(A):
    return decompose44(A)
