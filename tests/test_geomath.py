"""Pose and frame helpers restated from the mathematics (no GPU): affine
composition and its Gram-Schmidt decomposition, the static-frame Euler
convention the uncertainties use (design/uncertainties.py:36-38), Rodrigues
rotations, MARXS's position keywords (base/base.py:292-336) and the
polarization basis (math/polarization.py:12-63)."""
import numpy as np
import pytest

from marxs_gb300 import geomath as G


def _random_rotation(rng):
    q, r = np.linalg.qr(rng.normal(size=(3, 3)))
    q = q @ np.diag(np.sign(np.diag(r)))
    if np.linalg.det(q) < 0:
        q[:, 0] *= -1
    return q


def test_compose_decompose_round_trip():
    rng = np.random.default_rng(1)
    for _ in range(20):
        T, R, Z = rng.normal(size=3) * 100, _random_rotation(rng), rng.uniform(0.1, 30, 3)
        A = G.compose(T, R, Z)
        T2, R2, Z2, S2 = G.decompose44(A)
        np.testing.assert_allclose(T2, T, atol=1e-12)
        np.testing.assert_allclose(R2, R, atol=1e-12)
        np.testing.assert_allclose(Z2, Z, rtol=1e-12)
        np.testing.assert_allclose(S2, 0, atol=1e-12)


def test_compose_with_shear_is_recovered():
    rng = np.random.default_rng(2)
    S = np.array([0.1, -0.2, 0.3])
    A = G.compose([1, 2, 3], _random_rotation(rng), [2, 3, 4], S)
    T, R, Z, S2 = G.decompose44(A)
    np.testing.assert_allclose(S2, S, atol=1e-12)
    np.testing.assert_allclose(G.compose(T, R, Z, S2), A, atol=1e-12)


@pytest.mark.parametrize('k, axis', [(0, [1, 0, 0]), (1, [0, 1, 0]), (2, [0, 0, 1])])
def test_single_euler_angles_are_rotations_about_the_fixed_axes(k, axis):
    a = [0.0, 0.0, 0.0]
    a[k] = 0.3
    np.testing.assert_allclose(G.euler2mat(*a, axes='sxyz'), G.axangle2mat(axis, 0.3), atol=1e-15)


def test_static_xyz_order():
    """'sxyz': rotate about x, then the fixed y, then the fixed z."""
    ai, aj, ak = 0.1, -0.2, 0.35
    M = G.euler2mat(ai, aj, ak, 'sxyz')
    want = G.axangle2mat([0, 0, 1], ak) @ G.axangle2mat([0, 1, 0], aj) @ \
        G.axangle2mat([1, 0, 0], ai)
    np.testing.assert_allclose(M, want, atol=1e-15)
    np.testing.assert_allclose(M @ M.T, np.eye(3), atol=1e-15)


def test_axangle_is_rodrigues():
    rng = np.random.default_rng(3)
    for _ in range(10):
        k = rng.normal(size=3)
        th = rng.uniform(-np.pi, np.pi)
        v = rng.normal(size=3)
        ku = k / np.linalg.norm(k)
        want = v * np.cos(th) + np.cross(ku, v) * np.sin(th) + ku * np.dot(ku, v) * (1 - np.cos(th))
        np.testing.assert_allclose(G.axangle2mat(k, th) @ v, want, atol=1e-13)
        np.testing.assert_allclose(G.axangle2mat(ku, th, is_normalized=True) @ v, want,
                                   atol=1e-13)


def test_position_keywords():
    R = G.axangle2mat([0, 0, 1], 0.5)
    pos4d = G.parse_position_keywords({'position': [1, 2, 3], 'orientation': R, 'zoom': [2, 3, 4]})
    np.testing.assert_allclose(pos4d[:3, 3], [1, 2, 3])
    np.testing.assert_allclose(pos4d[:3, :3], R @ np.diag([2, 3, 4]))
    np.testing.assert_allclose(G.parse_position_keywords({'zoom': 5})[:3, :3], 5 * np.eye(3))
    np.testing.assert_array_equal(G.parse_position_keywords({'pos4d': pos4d}), pos4d)
    with pytest.raises(ValueError):
        G.parse_position_keywords({'pos4d': pos4d, 'zoom': 2})
    with pytest.raises(ValueError):
        G.parse_position_keywords({'zoom': [1, -1, 1]})
    with pytest.raises(ValueError):
        G.parse_position_keywords({'zoom': [1, 1]})
    with pytest.raises(ValueError):
        G.parse_position_keywords({'pos4d': np.zeros((4, 4))})


def test_homogeneous_round_trip():
    rng = np.random.default_rng(5)
    e = rng.normal(size=(10, 3))
    h = G.e2h(e, 1)
    assert h.shape == (10, 4) and np.all(h[:, 3] == 1)
    np.testing.assert_allclose(G.h2e(h), e)


def test_polarization_vectors_are_unit_and_transverse():
    rng = np.random.default_rng(7)
    d = np.concatenate([rng.normal(size=(200, 3)), [[0, 1, 0], [0, -3, 0]]])
    d4 = np.concatenate([d, np.zeros((len(d), 1))], axis=1)
    ang = rng.uniform(0, np.pi, len(d))
    p = G.polarization_vectors(d4, ang)
    assert np.all(p[:, 3] == 0)
    np.testing.assert_allclose(np.linalg.norm(p[:, :3], axis=1), 1, atol=1e-14)
    du = d / np.linalg.norm(d, axis=1)[:, None]
    np.testing.assert_allclose(np.einsum('ij,ij->i', p[:, :3], du), 0, atol=1e-14)
    # the angle is measured from the projection of +y (of +x for rays along y)
    p0 = G.polarization_vectors(np.array([[1., 0, 0, 0]]), np.array([0.0]))
    np.testing.assert_allclose(p0[0, :3], [0, 1, 0], atol=1e-15)
    p1 = G.polarization_vectors(np.array([[0., 1, 0, 0]]), np.array([0.0]))
    np.testing.assert_allclose(p1[0, :3], [1, 0, 0], atol=1e-15)


def test_anglediff_wraps_into_one_turn():
    assert G.anglediff([0.0, 1.0]) == pytest.approx(1.0)
    assert G.anglediff([1.0, 0.5]) == pytest.approx(2 * np.pi - 0.5)
    assert 0 <= G.anglediff([-10.0, 10.0]) <= 2 * np.pi
