"""CPU restatement of photon generation for a point source seen through a
CircleAperture (test infrastructure: only tests and the measurement harness
use it).

Each function follows the reference step it names and takes its uniforms as
arrays, so that fed the uniforms the reference drew it reproduces the
reference's columns:
* RandomArbitraryPdf.__call__, marxs/math/random.py:79-95
* unpolarized angles, marxs/source/basesources.py:203-204
* polarization_vectors, marxs/math/polarization.py:12-63
* CircleAperture.generate_local_xy, marxs/optics/aperture.py:138-146, and
  FlatAperture.specific_process_photons, aperture.py:67-77
"""
import numpy as np


def arbitrary_pdf_sample(x, bin_width, cdf, sortindex, u_choice, u_bin, randomize_in_bin=True):
    """RandomArbitraryPdf.__call__: choice = uniform(0, cdf[-1]) = cdf[-1] u,
    index = searchsorted(cdf, choice), mapped through the sort index, then
    x[index - 1] + width[index] * rand (or x[index])."""
    choice = 0.0 + (cdf[-1] - 0.0) * np.asarray(u_choice)
    index = np.searchsorted(cdf, choice)
    if sortindex is not None:
        index = sortindex[index]
    if randomize_in_bin:
        return x[index - 1] + bin_width[index] * np.asarray(u_bin)
    return x[index]


def unpolarized_angles(u):
    """np.random.uniform(0, 2 pi, n)."""
    return 0 + (2 * np.pi - 0) * np.asarray(u)


def polarization_basis(direction):
    """(v_1, v_2) of polarization_vectors for one direction of travel."""
    r = np.asarray(direction, dtype=float)[:3].copy()
    r /= np.linalg.norm(r)
    x = np.array([1., 0., 0.])
    y = np.array([0., 1., 0.])
    if np.isclose(r[0], 0.) and np.isclose(r[2], 0.):
        v1 = x - r * np.dot(r, x)
    else:
        v1 = y - r * np.dot(r, y)
    v1 = v1 / np.linalg.norm(v1)
    return v1, np.cross(r, v1)


def circle_aperture_xy(phi_lim, r_inner_norm, u_phi, u_r):
    """generate_local_xy: phi = uniform(phi0, phi1), r = sqrt(uniform(ri^2, 1))."""
    phi = phi_lim[0] + (phi_lim[1] - phi_lim[0]) * np.asarray(u_phi)
    lo = r_inner_norm ** 2
    r = np.sqrt(lo + (1. - lo) * np.asarray(u_r))
    return r * np.cos(phi), r * np.sin(phi)


def generate(center, v_y, v_z, e_x, phi_lim, r_inner_norm, direction, energy, pol_angle, draws):
    """Photon columns (pos, dir, energy, polarization, probability) as (N,4)
    homogeneous arrays.  ``energy``: a keV value or (x, bin_width, cdf,
    sortindex, randomize_in_bin); ``pol_angle`` None for unpolarized;
    ``draws``: (5, N) uniforms (energy choice, in-bin, angle, phi, r)."""
    draws = np.asarray(draws, dtype=float)
    n = draws.shape[1]
    if np.isscalar(energy):
        en = np.full(n, float(energy))
    else:
        en = arbitrary_pdf_sample(*energy[:4], draws[0], draws[1], randomize_in_bin=energy[4])
    ang = unpolarized_angles(draws[2]) if pol_angle is None else np.full(n, float(pol_angle))
    d4 = np.tile(np.r_[np.asarray(direction, dtype=float)[:3], 0.], (n, 1))
    v1, v2 = polarization_basis(direction)
    pol = np.zeros((n, 4))
    pol[:, 0:3] = v1 * np.cos(ang)[:, None] + v2 * np.sin(ang)[:, None]
    x, y = circle_aperture_xy(phi_lim, r_inner_norm, draws[3], draws[4])
    c4 = np.r_[np.asarray(center, dtype=float)[:3], 1.]
    vy4 = np.r_[np.asarray(v_y, dtype=float)[:3], 0.]
    vz4 = np.r_[np.asarray(v_z, dtype=float)[:3], 0.]
    pos = c4 + x.reshape((-1, 1)) * vy4 + y.reshape((-1, 1)) * vz4
    ex4 = np.r_[np.asarray(e_x, dtype=float)[:3], 0.]
    prob = np.clip(np.dot(d4, -ex4), 0, 1)
    return {'pos': pos, 'dir': d4, 'energy': en, 'polarization': pol, 'probability': prob}
